// ORACLE (test infrastructure): a C-ABI wrapper of our own around the
// reference's CPU KD-tree (createKDTree, src/kdtree.hpp:494-534, and
// KDTreeKNNSearch, src/kdtree.cpp:164-194), compiled with the reference's
// unmodified src/kdtree.cpp (included below) by `make -C oracle ref`.  It plays
// the part of the reference's pybind class KDTreeCPU{1,2,3}D[F] (and of the
// classes its README's recipe adds for more dimensions)
// (src/interface.cpp:13-95): build on the host, expose the layout getters,
// query with raw pointers.  Used by tests/golden/make_golden.py to produce
// fixtures and, where it was built, as the timed CPU baseline.
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>

// The reference's src/kdtree.cpp, unmodified, compiled in this translation
// unit: its KD-tree search and PartitionInfo are templates defined there, and
// seeing the definitions lets this wrapper instantiate them for 4-8 dimensions
// too (the reference's README recipe for more dimensions is to add such
// instantiations).
#include "kdtree.cpp"

namespace {

thread_local std::string g_err;

struct RefTree {
    int dims;
    int dtype;  // 0 = float, 1 = double
    void* info; // PartitionInfo<T, dims>*
};

template <typename T, dim_t D>
void* build(const T* pts, int32_t n, int levels) {
    return new PartitionInfo<T, D>(createKDTree<T, D>(pts, n, levels));
}

template <typename T, dim_t D>
void layout(void* p, T* structured, int32_t* perm, T* medians, uint8_t* axes, int32_t* leaf_off,
            int32_t* leaf_cnt) {
    auto* info = static_cast<PartitionInfo<T, D>*>(p);
    std::memcpy(structured, info->structured_points, sizeof(T) * D * (size_t)info->nr_points);
    std::memcpy(perm, info->shuffled_inds, sizeof(int32_t) * (size_t)info->nr_points);
    for (int i = 0; i < info->nr_partitions; ++i) {
        medians[i] = info->partitions[i].median;
        axes[i] = info->partitions[i].axis_split;
    }
    for (int i = 0; i < info->nr_leaves; ++i) {
        leaf_off[i] = info->leaves[i].offset;
        leaf_cnt[i] = info->leaves[i].nr_points;
    }
}

template <typename T, dim_t D>
void query(void* p, const T* q, int32_t nq, int k, T* dists, int32_t* idx) {
    auto* info = static_cast<PartitionInfo<T, D>*>(p);
    KDTreeKNNSearch<T, T, D>(*info, nq, reinterpret_cast<const std::array<T, D>*>(q), dists, idx, k);
}

template <typename T, dim_t D>
void destroy(void* p) {
    delete static_cast<PartitionInfo<T, D>*>(p);
}

// Dimensions 1-3 are the reference's own instantiations (src/interface.cpp:128-141);
// 4-8 follow its README recipe for more dimensions (more template instantiations).
#define TK_DISPATCH_T(tree_dims, TT, CALL)                                         \
    do {                                                                           \
        using T = TT;                                                              \
        switch (tree_dims) {                                                       \
            case 1: { constexpr dim_t D = 1; CALL; break; }                        \
            case 2: { constexpr dim_t D = 2; CALL; break; }                        \
            case 3: { constexpr dim_t D = 3; CALL; break; }                        \
            case 4: { constexpr dim_t D = 4; CALL; break; }                        \
            case 5: { constexpr dim_t D = 5; CALL; break; }                        \
            case 6: { constexpr dim_t D = 6; CALL; break; }                        \
            case 7: { constexpr dim_t D = 7; CALL; break; }                        \
            default: { constexpr dim_t D = 8; CALL; break; }                       \
        }                                                                          \
    } while (0)
#define TK_DISPATCH(tree_dims, tree_dtype, CALL)                                   \
    do {                                                                           \
        if ((tree_dtype) == 0) TK_DISPATCH_T(tree_dims, float, CALL);              \
        else TK_DISPATCH_T(tree_dims, double, CALL);                               \
    } while (0)

}  // namespace

extern "C" {

const char* ref_last_error(void) { return g_err.c_str(); }

void* ref_tree_create(const void* pts, int32_t n, int dims, int dtype, int levels) {
    if (dims < 1 || dims > 8 || (dtype != 0 && dtype != 1)) {
        g_err = "unsupported dims/dtype";
        return nullptr;
    }
    try {
        RefTree* t = new RefTree{dims, dtype, nullptr};
        TK_DISPATCH(dims, dtype, t->info = (build<T, D>(static_cast<const T*>(pts), n, levels)));
        return t;
    } catch (const std::exception& e) {
        g_err = e.what();
        return nullptr;
    }
}

int ref_tree_layout(void* h, void* structured, int32_t* perm, void* medians, uint8_t* axes,
                    int32_t* leaf_off, int32_t* leaf_cnt) {
    RefTree* t = static_cast<RefTree*>(h);
    TK_DISPATCH(t->dims, t->dtype,
                (layout<T, D>(t->info, static_cast<T*>(structured), perm, static_cast<T*>(medians),
                              axes, leaf_off, leaf_cnt)));
    return 0;
}

int ref_tree_query(void* h, const void* q, int32_t nq, int k, void* dists, int32_t* idx) {
    RefTree* t = static_cast<RefTree*>(h);
    TK_DISPATCH(t->dims, t->dtype,
                (query<T, D>(t->info, static_cast<const T*>(q), nq, k, static_cast<T*>(dists), idx)));
    return 0;
}

void ref_tree_destroy(void* h) {
    RefTree* t = static_cast<RefTree*>(h);
    if (!t) return;
    TK_DISPATCH(t->dims, t->dtype, (destroy<T, D>(t->info)));
    delete t;
}

}  // extern "C"
