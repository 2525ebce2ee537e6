// Exact KNN of host queries on a host-built tree ("CPU trees"): the query the
// reference binds as KDTreeCPU<dims>[F].query (src/interface.cpp:60-86 ->
// KDTreeKNNSearch, src/kdtree.cpp:164-194), under this engine's contract:
//  * squared distances with the reference's arithmetic: d_c = q_c - p_c and
//    ((0 + d0^2) + d1^2) + ... in T, every operation rounded on its own
//    (this file is compiled without floating-point contraction);
//  * original point indices, and among equal distances the lower index --
//    the same answer, bit for bit, as the GPU query of the same tree.
// The search is depth first from the root: a node is entered only if the
// bound of its bounding box (per axis the gap from the query to the box,
// squared and summed like a distance, so by monotonicity of rounding never
// above the distance of a point inside) does not exceed the current k-th
// distance; children are taken near side first (the reference's rule,
// src/kdtree.cpp:30).  Boxes that only tie the k-th distance are still
// entered, so the result equals an exhaustive search ordered by
// (distance, original index).  Queries are searched in tree-cell order by
// host threads pulling chunks of that order.
#include <algorithm>
#include <atomic>
#include <cstdint>
#include <limits>
#include <thread>
#include <vector>

#include "tk_internal.h"

namespace tk {
namespace {

template <typename T>
inline bool key_less(T da, uint32_t ia, T db, uint32_t ib) {
    return da < db || (da == db && ia < ib);  // false whenever da is NaN
}

template <typename T, int D>
struct CpuSearch {
    const HostTree<T>& h;
    int k;
    std::vector<T> ld;         // the k best distances, ascending
    std::vector<uint32_t> li;  // their original indices
    std::vector<int> stack;
    static constexpr int kChunk = 64;
    T dist[kChunk];

    CpuSearch(const HostTree<T>& tree, int kk) : h(tree), k(kk), ld(kk), li(kk) {
        stack.reserve(2 * kMaxLevels + 2);
    }

    T box_bound(int node, const T* q) const {
        const int S = h.box_stride();
        const T* lo = h.box_lo.data() + size_t(node) * S;
        const T* hi = h.box_hi.data() + size_t(node) * S;
        T b = T(0);
        for (int c = 0; c < D; ++c) {
            const T g = q[c] < lo[c] ? T(q[c] - lo[c]) : (q[c] > hi[c] ? T(q[c] - hi[c]) : T(0));
            const T e = T(g * g);
            b = c == 0 ? e : T(b + e);
        }
        return b;
    }

    void offer(T d, uint32_t i) {
        if (!key_less(d, i, ld[k - 1], li[k - 1])) return;
        int p = k - 1;
        while (p > 0 && key_less(d, i, ld[p - 1], li[p - 1])) {
            ld[p] = ld[p - 1];
            li[p] = li[p - 1];
            --p;
        }
        ld[p] = d;
        li[p] = i;
    }

    void run(const T* q, T* out_d, int32_t* out_i) {
        std::fill(ld.begin(), ld.end(), std::numeric_limits<T>::infinity());
        std::fill(li.begin(), li.end(), 0xFFFFFFFFu);
        bool nan_q = false;
        for (int c = 0; c < D; ++c) nan_q |= q[c] != q[c];
        if (!nan_q) {  // a query with a NaN coordinate has only NaN distances: nothing enters its list
            const int L = h.levels;
            const int first_leaf = (1 << L) - 1;
            stack.clear();
            stack.push_back(0);
            while (!stack.empty()) {
                const int node = stack.back();
                stack.pop_back();
                if (!(box_bound(node, q) <= ld[k - 1])) continue;
                if (node >= first_leaf) {
                    const int leaf = node - first_leaf;
                    const int beg = h.leaf_off[leaf], end = h.leaf_off[leaf + 1];
                    // distances of a chunk of the leaf first (a loop without
                    // branches, which the compiler vectorises), then the offers
                    for (int j0 = beg; j0 < end; j0 += kChunk) {
                        const int m = std::min(kChunk, end - j0);
                        const T* p = h.structured.data() + size_t(j0) * D;
                        for (int j = 0; j < m; ++j) {
                            const T* pj = p + size_t(j) * D;
                            const T d0 = T(q[0] - pj[0]);
                            T acc = T(d0 * d0);
                            for (int c = 1; c < D; ++c) {
                                const T dc = T(q[c] - pj[c]);
                                acc = T(acc + T(dc * dc));
                            }
                            dist[j] = acc;
                        }
                        const T worst = ld[k - 1];
                        for (int j = 0; j < m; ++j)
                            if (dist[j] <= worst) offer(dist[j], uint32_t(h.perm[j0 + j]));
                    }
                    continue;
                }
                const int depth = 31 - __builtin_clz(unsigned(node) + 1u);
                const int ax = depth % D;
                const bool left_near = q[ax] < h.medians[node];
                stack.push_back(2 * node + (left_near ? 2 : 1));  // far child: visited after the near one
                stack.push_back(2 * node + (left_near ? 1 : 2));
            }
        }
        for (int r = 0; r < k; ++r) {
            out_d[r] = ld[r];
            out_i[r] = int32_t(li[r]);
        }
    }
};

// Cell of a query at depth B (the search's descent rule), for the order below.
template <typename T, int D>
uint32_t home_cell(const HostTree<T>& h, const T* q, int B) {
    int node = 0;
    for (int depth = 0; depth < B; ++depth) node = 2 * node + (q[depth % D] < h.medians[node] ? 1 : 2);
    return uint32_t(node - ((1 << B) - 1));
}

template <typename T, int D>
void search_all(const HostTree<T>& h, const T* q, int64_t nq, int k, T* dists, int32_t* idx, int n_threads) {
    int nt = n_threads > 0 ? n_threads : int(std::max(1u, std::thread::hardware_concurrency()));
    nt = int(std::min<int64_t>(nt, std::max<int64_t>(1, nq / 64)));
    // Queries are taken in the order of the tree cell they fall into (a
    // counting sort over the cells at depth B), so consecutive searches of a
    // thread walk nearly the same nodes and leaves while they are in cache;
    // threads pull chunks of that order from a shared counter.
    int B = 0;
    while (B < h.levels && B < 16 && (int64_t(1) << (B + 6)) <= nq) ++B;
    std::vector<int32_t> order;
    if (B > 0) {
        const size_t ncell = size_t(1) << B;
        std::vector<uint32_t> cell(static_cast<size_t>(nq));
        std::vector<int64_t> start(ncell + 1, 0);
        for (int64_t i = 0; i < nq; ++i) {
            cell[size_t(i)] = home_cell<T, D>(h, q + i * D, B);
            ++start[cell[size_t(i)] + 1];
        }
        for (size_t c = 0; c < ncell; ++c) start[c + 1] += start[c];
        order.resize(size_t(nq));
        for (int64_t i = 0; i < nq; ++i) order[size_t(start[cell[size_t(i)]]++)] = int32_t(i);
    }
    const int64_t chunk = 256;
    std::atomic<int64_t> next{0};
    auto work = [&]() {
        CpuSearch<T, D> s(h, k);
        for (;;) {
            const int64_t b = next.fetch_add(chunk);
            if (b >= nq) break;
            const int64_t e = std::min(nq, b + chunk);
            for (int64_t t = b; t < e; ++t) {
                const int64_t i = order.empty() ? t : order[size_t(t)];
                s.run(q + i * D, dists + i * k, idx + i * k);
            }
        }
    };
    if (nt <= 1) {
        work();
        return;
    }
    std::vector<std::thread> pool;
    pool.reserve(nt);
    for (int t = 0; t < nt; ++t) pool.emplace_back(work);
    for (auto& th : pool) th.join();
}

template <typename T>
int query_cpu(const HostTree<T>& h, const T* q, int64_t nq, int k, T* dists, int32_t* idx, int n_threads) {
    switch (h.dims) {
        case 1: search_all<T, 1>(h, q, nq, k, dists, idx, n_threads); break;
        case 2: search_all<T, 2>(h, q, nq, k, dists, idx, n_threads); break;
        case 3: search_all<T, 3>(h, q, nq, k, dists, idx, n_threads); break;
        case 4: search_all<T, 4>(h, q, nq, k, dists, idx, n_threads); break;
        case 5: search_all<T, 5>(h, q, nq, k, dists, idx, n_threads); break;
        case 6: search_all<T, 6>(h, q, nq, k, dists, idx, n_threads); break;
        case 7: search_all<T, 7>(h, q, nq, k, dists, idx, n_threads); break;
        case 8: search_all<T, 8>(h, q, nq, k, dists, idx, n_threads); break;
        default: return fail(TK_EUNSUPPORTED, "CPU query: dims must be 1..8");
    }
    return TK_OK;
}

}  // namespace
}  // namespace tk

extern "C" int tk_tree_query_cpu(const tk_tree* t, const void* q, int64_t nq, int k, void* dists, int32_t* idx,
                                 int n_threads) {
    using namespace tk;
    clear_error();
    if (!t) return fail(TK_EINVAL, "tree is null");
    if (!t->host_layout)
        return fail(TK_EINVAL, "tree was built on the GPU and keeps no host layout; build it on the host "
                               "(tk_tree_create) to query it on the CPU");
    if (nq < 0 || nq >= (int64_t(1) << 31)) return fail(TK_EINVAL, "number of queries must be in [0, 2^31)");
    if (k < 1) return fail(TK_EINVAL, "k must be >= 1");
    if (k > t->n) return fail(TK_EINVAL, "You requested more nearest neighbors than there are in the KD-Tree");
    if (nq == 0) return TK_OK;
    if (!q || !dists || !idx) return fail(TK_EINVAL, "null query or output pointer");
    if (t->dtype == TK_F32)
        return query_cpu<float>(t->h32, static_cast<const float*>(q), nq, k, static_cast<float*>(dists), idx,
                                n_threads);
    return query_cpu<double>(t->h64, static_cast<const double*>(q), nq, k, static_cast<double*>(dists), idx,
                             n_threads);
}
