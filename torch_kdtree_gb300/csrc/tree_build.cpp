// Host KD-tree construction in the reference's layout.
//
// Semantics of createKDTree / createPartitionRecursive / compMedian
// (src/kdtree.hpp:392-534):
//   * node at depth t splits on axis t % dims;
//   * the node's points, ordered along that axis, go first floor(n/2) to the
//     left child and the rest to the right child;
//   * split value = middle element (odd n) or 0.5 * (a + b) of the two middle
//     elements (even n), a + b rounded in T, the product taken in double;
//   * heap numbering 2i+1 / 2i+2; leaves numbered left to right, stored
//     contiguously; inside a leaf the points are ordered along the leaf
//     parent's axis;
//   * a split node that receives no point is an error.
// The reference sorts the whole range at every level (O(N log^2 N)); here
// upper levels use a linear-time selection and only leaf parents sort, which
// yields the same layout for tie-free coordinates.  Ties on a coordinate are
// ordered by original index (the reference's std::sort leaves them in an
// unspecified order).  Subtrees are built in parallel threads.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <limits>
#include <thread>

#include "tk_internal.h"

namespace tk {
namespace {

// NC coordinates per record: 3 for clouds of up to 3 dimensions, 8 above.
template <typename T, int NC>
struct Rec {
    T c[NC];
    int32_t orig;
};

template <typename T, int NC>
struct Builder {
    using R = Rec<T, NC>;
    int dims;
    int levels;
    int32_t nparts;
    R* recs;
    T* medians;
    int32_t* leaf_off;
    std::atomic<bool> failed{false};  // set by any worker that meets an empty split node

    static bool less(const R& a, const R& b, int ax) {
        if (a.c[ax] < b.c[ax]) return true;
        if (b.c[ax] < a.c[ax]) return false;
        return a.orig < b.orig;
    }

    // compMedian (src/kdtree.hpp:392-401) on the values at ranks h-1 and h.
    static T median_of(T lower_mid, T upper_mid, int32_t n) {
        if (n % 2 == 1) return upper_mid;
        const T s = lower_mid + upper_mid;  // rounded in T
        return static_cast<T>(0.5 * static_cast<double>(s));
    }

    void node(int32_t lo, int32_t n, int32_t id, int depth, int spawn_depth) {
        if (n == 0) {
            failed.store(true);
            return;
        }
        const int ax = depth % dims;
        R* r = recs + lo;
        const int32_t h = n / 2;
        auto cmp = [ax](const R& a, const R& b) { return less(a, b, ax); };
        if (depth == levels - 1) {
            std::sort(r, r + n, cmp);
            medians[id] = median_of(h > 0 ? r[h - 1].c[ax] : r[h].c[ax], r[h].c[ax], n);
            const int32_t leaf = 2 * id + 1 - nparts;
            leaf_off[leaf] = lo;
            leaf_off[leaf + 1] = lo + h;
            return;
        }
        std::nth_element(r, r + h, r + n, cmp);
        T lower_mid = r[h].c[ax];
        if (h > 0) lower_mid = std::max_element(r, r + h, cmp)->c[ax];
        medians[id] = median_of(lower_mid, r[h].c[ax], n);
        if (depth < spawn_depth && n > 65536) {
            std::thread left([=] { node(lo, h, 2 * id + 1, depth + 1, spawn_depth); });
            node(lo + h, n - h, 2 * id + 2, depth + 1, spawn_depth);
            left.join();
        } else {
            node(lo, h, 2 * id + 1, depth + 1, spawn_depth);
            node(lo + h, n - h, 2 * id + 2, depth + 1, spawn_depth);
        }
    }
};

// Tight bounding box of every node's points: leaves from their points,
// inner nodes from their children; heap order over all 2^(L+1) - 1 nodes,
// box_stride() coordinates per node (unused ones 0; empty nodes +inf / -inf).
template <typename T>
void compute_boxes(HostTree<T>& out) {
    const int bs = out.box_stride();
    const int64_t nleaves = int64_t(1) << out.levels;
    const int64_t nnodes = 2 * nleaves - 1;
    const T inf = std::numeric_limits<T>::infinity();
    out.box_lo.assign(static_cast<size_t>(nnodes) * bs, inf);
    out.box_hi.assign(static_cast<size_t>(nnodes) * bs, -inf);
    for (int64_t l = 0; l < nleaves; ++l) {
        const int64_t node = nleaves - 1 + l;
        T* lo = &out.box_lo[node * bs];
        T* hi = &out.box_hi[node * bs];
        for (int32_t i = out.leaf_off[l]; i < out.leaf_off[l + 1]; ++i)
            for (int c = 0; c < out.dims; ++c) {
                const T v = out.structured[size_t(i) * out.dims + c];
                lo[c] = std::min(lo[c], v);
                hi[c] = std::max(hi[c], v);
            }
        if (out.leaf_off[l + 1] > out.leaf_off[l])
            for (int c = out.dims; c < bs; ++c) lo[c] = hi[c] = T(0);  // unused coordinates are 0
    }
    for (int64_t node = nleaves - 2; node >= 0; --node)
        for (int c = 0; c < bs; ++c) {
            out.box_lo[node * bs + c] = std::min(out.box_lo[(2 * node + 1) * bs + c], out.box_lo[(2 * node + 2) * bs + c]);
            out.box_hi[node * bs + c] = std::max(out.box_hi[(2 * node + 1) * bs + c], out.box_hi[(2 * node + 2) * bs + c]);
        }
}

template <typename T, int NC>
bool run_builder(const T* pts, int64_t n, int dims, int levels, int n_threads, HostTree<T>& out) {
    const int32_t nparts = int32_t((1u << levels) - 1u);
    std::vector<Rec<T, NC>> recs(static_cast<size_t>(n));
    for (int64_t i = 0; i < n; ++i) {
        for (int c = 0; c < NC; ++c) recs[i].c[c] = c < dims ? pts[i * dims + c] : T(0);
        recs[i].orig = int32_t(i);
    }
    if (n_threads <= 0) n_threads = int(std::max(1u, std::thread::hardware_concurrency()));
    int spawn_depth = 0;
    while ((1 << spawn_depth) < n_threads && spawn_depth < 8) ++spawn_depth;
    Builder<T, NC> b;
    b.dims = dims;
    b.levels = levels;
    b.nparts = nparts;
    b.recs = recs.data();
    b.medians = out.medians.data();
    b.leaf_off = out.leaf_off.data();
    b.node(0, int32_t(n), 0, 0, spawn_depth);
    if (b.failed.load()) return false;
    out.structured.resize(static_cast<size_t>(n) * dims);
    out.perm.resize(static_cast<size_t>(n));
    for (int64_t i = 0; i < n; ++i) {
        for (int c = 0; c < dims; ++c) out.structured[i * dims + c] = recs[i].c[c];
        out.perm[i] = recs[i].orig;
    }
    return true;
}

}  // namespace

template <typename T>
int build_host_tree(const T* pts, int64_t n, int dims, int levels, int n_threads, HostTree<T>& out) {
    if (pts == nullptr) return fail(TK_EINVAL, "points pointer is null");
    if (dims < 1 || dims > kMaxDims)
        return fail(TK_EINVAL, "KD-tree supports dims 1 to " + std::to_string(kMaxDims) + " (got " +
                                   std::to_string(dims) + ")");
    if (n < 1) return fail(TK_EINVAL, "the reference point cloud is empty");
    if (n >= (int64_t(1) << 31)) return fail(TK_EINVAL, "only 32 bit signed indexing implemented (n < 2^31)");
    if (levels < 1 || levels > kMaxLevels)
        return fail(TK_EINVAL, "levels must be in [1, " + std::to_string(kMaxLevels) + "]");
    for (int64_t i = 0; i < n * dims; ++i)
        if (std::isnan(pts[i])) return fail(TK_EINVAL, "reference points contain NaN");

    const int32_t nparts = int32_t((1u << levels) - 1u);
    out.n = n;
    out.dims = dims;
    out.levels = levels;
    out.medians.assign(static_cast<size_t>(nparts), T(0));
    out.leaf_off.assign(static_cast<size_t>(nparts) + 2, 0);
    const bool ok = dims <= 3 ? run_builder<T, 3>(pts, n, dims, levels, n_threads, out)
                              : run_builder<T, 8>(pts, n, dims, levels, n_threads, out);
    if (!ok)
        return fail(TK_EINVAL,
                    "Ran out of points while building KD-Tree. Either you required too many levels, "
                    "or you used a lot of coplanar points");
    out.leaf_off.resize(static_cast<size_t>(nparts) + 2);
    out.leaf_off[nparts + 1] = int32_t(n);  // 2^L leaves -> 2^L + 1 offsets
    compute_boxes(out);
    return TK_OK;
}

template <typename T>
int tree_from_layout(const T* structured, const int32_t* perm, const T* medians, const int32_t* leaf_off, int64_t n,
                     int dims, int levels, HostTree<T>& out) {
    if (!structured || !perm || !medians || !leaf_off) return fail(TK_EINVAL, "layout pointer is null");
    if (dims < 1 || dims > kMaxDims)
        return fail(TK_EINVAL, "KD-tree supports dims 1 to " + std::to_string(kMaxDims) + " (got " +
                                   std::to_string(dims) + ")");
    if (n < 1) return fail(TK_EINVAL, "the reference point cloud is empty");
    if (n >= (int64_t(1) << 31)) return fail(TK_EINVAL, "only 32 bit signed indexing implemented (n < 2^31)");
    if (levels < 1 || levels > kMaxLevels)
        return fail(TK_EINVAL, "levels must be in [1, " + std::to_string(kMaxLevels) + "]");
    const int64_t nleaves = int64_t(1) << levels;
    const int64_t nparts = nleaves - 1;
    // leaf offsets: from 0 to n, non-decreasing
    if (leaf_off[0] != 0 || leaf_off[nleaves] != n) return fail(TK_EINVAL, "leaf offsets must run from 0 to n");
    for (int64_t l = 0; l < nleaves; ++l)
        if (leaf_off[l + 1] < leaf_off[l]) return fail(TK_EINVAL, "leaf offsets must be non-decreasing");
    // perm: a permutation of 0..n-1
    std::vector<unsigned char> seen(static_cast<size_t>(n), 0);
    for (int64_t i = 0; i < n; ++i) {
        const int32_t p = perm[i];
        if (p < 0 || p >= n || seen[size_t(p)]) return fail(TK_EINVAL, "perm is not a permutation of 0..n-1");
        seen[size_t(p)] = 1;
    }
    for (int64_t i = 0; i < n * dims; ++i)
        if (std::isnan(structured[i])) return fail(TK_EINVAL, "reference points contain NaN");
    for (int64_t i = 0; i < nparts; ++i)
        if (std::isnan(medians[i])) return fail(TK_EINVAL, "split values contain NaN");
    out.n = n;
    out.dims = dims;
    out.levels = levels;
    out.structured.assign(structured, structured + n * dims);
    out.perm.assign(perm, perm + n);
    out.medians.assign(medians, medians + nparts);
    out.leaf_off.assign(leaf_off, leaf_off + nleaves + 1);
    compute_boxes(out);
    // Every split must separate its children along its axis (left <= split <=
    // right, the property the search's plane bounds rely on); otherwise the
    // answers would silently stop being exact.
    for (int64_t node = 0; node < nparts; ++node) {
        const int depth = 63 - __builtin_clzll(uint64_t(node + 1));
        const int ax = depth % dims;
        const T m = out.medians[size_t(node)];
        const int bs = out.box_stride();
        const T left_hi = out.box_hi[size_t(2 * node + 1) * bs + ax];
        const T right_lo = out.box_lo[size_t(2 * node + 2) * bs + ax];
        if (left_hi > m || right_lo < m)
            return fail(TK_EINVAL, "layout is inconsistent: points on the wrong side of split " + std::to_string(node));
    }
    return TK_OK;
}

template int tree_from_layout<float>(const float*, const int32_t*, const float*, const int32_t*, int64_t, int, int,
                                     HostTree<float>&);
template int tree_from_layout<double>(const double*, const int32_t*, const double*, const int32_t*, int64_t, int, int,
                                      HostTree<double>&);

template int build_host_tree<float>(const float*, int64_t, int, int, int, HostTree<float>&);
template int build_host_tree<double>(const double*, int64_t, int, int, int, HostTree<double>&);

}  // namespace tk
