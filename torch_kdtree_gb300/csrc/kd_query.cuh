// Exact KD-tree KNN query kernels (sm_103a).
//
// What the reference does (src/kdtree_g.cu:286-457): one query per 64-thread
// block, thread 0 alone walks the tree with 2-bit visited tags in shared
// memory, leaf distances go through a 256-entry shared buffer and every
// candidate is inserted serially with a block barrier.
//
// What this file does instead:
//  1. Calls of at least a wave of queries (SMs x 1024) first bin them by the
//     tree cell they fall into (a counting sort over the cells at depth B), so
//     neighbouring lanes follow nearly the same path through the tree and hit
//     the same leaves in L1; smaller calls keep the input order (see
//     prepare_order in tk_api.cu).
//  2. A group of G lanes (G = 1..32, "threads per query") serves one query.
//     The walk is a depth-first descent with an explicit short stack of far
//     siblings; each entry carries the per-axis squared plane distances of
//     its cell, whose rounded sum is a lower bound on every distance inside
//     (exactly safe under round-to-nearest, see sqdist), so pruning never
//     drops a neighbour and the result equals an exhaustive search ordered by
//     (distance, original index) -- independent of tree shape and launch
//     shape.
//  3. The top split levels are staged in shared memory; deeper split values
//     and the leaf buckets (16-byte point records: xyz + original index) are
//     read through the read-only path, coalesced across the G lanes.
//  4. The k best keys live in registers, distributed over the group
//     (TopK in tk_device.cuh); candidates are offered in lane order.
//  5. Warps pull work from a global counter (persistent grid sized to the
//     SM count), so no block waits for a slow neighbour.  A warp takes 32/G
//     consecutive binned queries at once and finishes them together: handing
//     a lane a new query as soon as its own ends was measured slower, as the
//     lanes of a warp then stop sharing the leaves they load.
//  6. Alternatively (k_kd_packet) the 32 queries of a warp walk the tree
//     together, one lane each, which keeps the warp converged at the price of
//     visiting the union of the lanes' leaves.
#pragma once

#include <cuda_runtime.h>

#include "tk_device.cuh"
#include "tk_internal.h"

namespace tk {

template <typename T>
struct KdArgs {
    const PointRec<T>* pts;  // [n] in leaf order
    const T* medians;        // [2^L - 1] heap order
    const int32_t* leaf_off; // [2^L + 1]
    const PointRec<T>* boxes;// [2 * (2^(L+1) - 1)] node bounding boxes (lo, hi), or null
    int levels;              // L
    int smem_levels;         // S <= L: levels staged in shared memory
    const T* q;              // [nq, D]
    int nq;
    int k;
    const int32_t* order;    // [nq] processing order (binned), or null for identity
    T* out_d;                // [nq, k]
    int32_t* out_i;          // [nq, k]
    int* work;               // global work counter, zero at launch
};

template <typename T, int D>
__device__ __forceinline__ T cell_bound(const T (&e)[D]) {
    T b = e[0];
    if (D > 1) b = add_rn(b, e[1]);
    if (D > 2) b = add_rn(b, e[2]);
    return b;
}

// Value of lane `src` of a G-lane group (every lane of the group calls it).
template <typename T, int G>
__device__ __forceinline__ T shfl_group(unsigned gmask, T v, int src) {
    return __shfl_sync(gmask, v, src, G);
}

template <typename T, int D>
__device__ __forceinline__ T pick(const T (&v)[D], int ax) {
    T r = v[0];
    if (D > 1) r = ax == 1 ? v[1] : r;
    if (D > 2) r = ax == 2 ? v[2] : r;
    return r;
}

// One tree as the search sees it.
template <typename T>
struct TreeView {
    const PointRec<T>* pts;
    const T* medians;
    const int32_t* leaf_off;
    int levels;
    int smem_levels;  // top levels whose split values are in s_med
    const T* s_med;
    const PointRec<T>* boxes;  // node bounding boxes, or null
};

// Lower bound on the computed distance from q to any point inside the
// bounding box of `node`: per axis the gap to the box, rounded and squared
// as sqdist does, summed in the same order.  By monotonicity of rounding it
// never exceeds sqdist(q, p) for a point p in the box; an empty box
// (lo = +inf, hi = -inf) gives +inf.
template <typename T, int D>
__device__ __forceinline__ T box_bound_of(const PointRec<T>& lo, const PointRec<T>& hi, const T (&q)[D]) {
    const T l[3] = {lo.x, lo.y, lo.z};
    const T h[3] = {hi.x, hi.y, hi.z};
    T e[D];
#pragma unroll
    for (int c = 0; c < D; ++c) {
        const T g = q[c] < l[c] ? sub_rn(q[c], l[c]) : (q[c] > h[c] ? sub_rn(q[c], h[c]) : T(0));
        e[c] = mul_rn(g, g);
    }
    T b = e[0];
    if (D > 1) b = add_rn(b, e[1]);
    if (D > 2) b = add_rn(b, e[2]);
    return b;
}

template <typename T, int D>
__device__ __forceinline__ T box_bound(const PointRec<T>* boxes, int node, const T (&q)[D]) {
    return box_bound_of<T, D>(load_rec(boxes + 2 * node), load_rec(boxes + 2 * node + 1), q);
}

// Sort R keys ascending in registers (bitonic network, R a power of two).
template <typename T, int R>
__device__ __forceinline__ void bitonic_sort(Key<T> (&v)[R]) {
#pragma unroll
    for (int size = 2; size <= R; size <<= 1) {
#pragma unroll
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
#pragma unroll
            for (int i = 0; i < R; ++i) {
                const int j = i ^ stride;
                if (j > i) {
                    const bool up = (i & size) == 0;
                    const bool sw = up ? v[j].lt(v[i]) : v[i].lt(v[j]);
                    const Key<T> a = v[i], b = v[j];
                    v[i] = sw ? b : a;
                    v[j] = sw ? a : b;
                }
            }
        }
    }
}

// Exhaustive-equivalent KNN for one query, served by a group of G lanes;
// writes k results to out_d[0..k) / out_i[0..k).
//
// Depth-first search without a stack in memory.  The path from the root to
// the current leaf is the leaf's heap index, so a far sibling still to visit
// needs one bit: bit t of `pending` says "the sibling of the path node at
// depth t + 1 may hold a neighbour".  After a leaf the deepest pending bit is
// taken first (the same order a stack would give); the sibling's id follows
// from the leaf id by shifts.  A pending sibling is checked against the
// current k-th distance twice, cheapest first -- groups of 8 or more lanes
// by the bound of its cell recorded when it was marked (one register per
// depth, spread over the group's lanes: depth t lives in lane t % G),
// smaller groups by its parent's split plane (top levels in shared memory)
// -- then by its bounding box, whose per-axis gaps also become the axis
// bounds its own descent starts from.  All lanes of a group hold the same
// trail: no local memory, for any group size.
template <typename T, int D, int G, int R>
__device__ __forceinline__ void kd_search(const TreeView<T>& tv, const T (&q)[D], int k, T* out_d,
                                          int32_t* out_i, unsigned gmask, int gl, int gbase) {
    TopK<T, G, R> list;
    list.init(k, gl);
    Key<T> worst = Key<T>::sentinel();
    T worst_d = worst.dist();
    const int L = tv.levels;

    // recorded cell bounds of pending siblings (groups of >= 8 lanes): depth t
    // in register t / G of lane t % G
    constexpr int NB = G >= 8 ? (kMaxLevels + G - 1) / G : 0;
    T pb[NB > 0 ? NB : 1];

    // the home leaf: the cell the query falls into (src/kdtree.cpp:30 rule);
    // a sibling on the home path is bounded by its split plane alone
    int node = 0;
    for (int depth = 0, ax = 0; depth < L; ++depth) {
        const T m = depth < tv.smem_levels ? tv.s_med[node] : __ldg(tv.medians + node);
        const T qa = pick<T, D>(q, ax);
        if constexpr (NB > 0) {
            const T diff = sub_rn(qa, m);
            if (gl == depth % G) {
#pragma unroll
                for (int j = 0; j < NB; ++j)
                    if (depth / G == j) pb[j] = mul_rn(diff, diff);
            }
        }
        node = 2 * node + (qa < m ? 1 : 2);
        ax = (ax + 1 == D) ? 0 : ax + 1;
    }
    uint32_t pending = (1u << L) - 1u;  // every far sibling on the home path (L <= 24)
    bool home = true;

    for (;;) {
        // `node` is a leaf; its box records carry its point range (one round trip for both)
        {
            const PointRec<T> lo = load_rec(tv.boxes + 2 * node);
            const PointRec<T> hi = load_rec(tv.boxes + 2 * node + 1);
            int beg = int(rec_index(lo));
            const int end = int(rec_index(hi));
            if (box_bound_of<T, D>(lo, hi, q) <= worst_d) {
                if (G == 1 && home && k == R && end - beg >= R) {
                    // fill the whole list from the home cell with one sorting
                    // network instead of R single insertions
                    Key<T> v[R];
#pragma unroll
                    for (int i = 0; i < R; ++i) {
                        const PointRec<T> p = load_rec(tv.pts + beg + i);
                        v[i] = Key<T>::make(sqdist<T, D>(q, p), rec_index(p));
                    }
                    bitonic_sort<T, R>(v);
#pragma unroll
                    for (int i = 0; i < R; ++i) list.slot[i] = v[i];
                    worst = list.worst(gmask);
                    beg += R;
                }
                if constexpr (G == 1) {
                    // two records per step: independent loads and distance chains
                    int j = beg;
                    for (; j + 1 < end; j += 2) {
                        const PointRec<T> p0 = load_rec(tv.pts + j);
                        const PointRec<T> p1 = load_rec(tv.pts + j + 1);
                        const Key<T> k0 = Key<T>::make(sqdist<T, D>(q, p0), rec_index(p0));
                        const Key<T> k1 = Key<T>::make(sqdist<T, D>(q, p1), rec_index(p1));
                        worst = offer<T, G, R>(list, k0, worst, gmask, gl, gbase);
                        worst = offer<T, G, R>(list, k1, worst, gmask, gl, gbase);
                    }
                    if (j < end) {
                        const PointRec<T> p = load_rec(tv.pts + j);
                        worst = offer<T, G, R>(list, Key<T>::make(sqdist<T, D>(q, p), rec_index(p)), worst, gmask,
                                               gl, gbase);
                    }
                } else {
                    for (int j0 = beg; j0 < end; j0 += G) {
                        const int j = j0 + gl;
                        Key<T> mine = Key<T>::sentinel();
                        if (j < end) {
                            const PointRec<T> p = load_rec(tv.pts + j);
                            mine = Key<T>::make(sqdist<T, D>(q, p), rec_index(p));
                        }
                        worst = offer<T, G, R>(list, mine, worst, gmask, gl, gbase);
                    }
                }
                worst_d = worst.dist();
            }
        }
        home = false;

        // the deepest pending far sibling that can still hold a neighbour
        // (bounds are compared as !(b <= worst) so a NaN bound prunes)
        T e[D];
        int depth = 0;
        while (pending) {
            const int t = 31 - __clz(pending);
            pending ^= 1u << t;
            const int a = ((node + 1) >> (L - 1 - t)) - 1;  // path node at depth t + 1
            const int far = ((a + 1) ^ 1) - 1;              // its sibling
            if constexpr (NB > 0) {
                T v = pb[0];
#pragma unroll
                for (int j = 1; j < NB; ++j) v = (t / G == j) ? pb[j] : v;
                if (!(shfl_group<T, G>(gmask, v, t % G) <= worst_d)) continue;
            } else {
                const int parent = (a - 1) >> 1;
                const T m = t < tv.smem_levels ? tv.s_med[parent] : __ldg(tv.medians + parent);
                const T diff = sub_rn(pick<T, D>(q, t % D), m);
                if (!(mul_rn(diff, diff) <= worst_d)) continue;
            }
            const PointRec<T> lo = load_rec(tv.boxes + 2 * far);
            const PointRec<T> hi = load_rec(tv.boxes + 2 * far + 1);
            const T l[3] = {lo.x, lo.y, lo.z};
            const T h[3] = {hi.x, hi.y, hi.z};
#pragma unroll
            for (int c = 0; c < D; ++c) {
                const T g = q[c] < l[c] ? sub_rn(q[c], l[c]) : (q[c] > h[c] ? sub_rn(q[c], h[c]) : T(0));
                e[c] = mul_rn(g, g);
            }
            if (!(cell_bound<T, D>(e) <= worst_d)) continue;
            node = far;
            depth = t + 1;
            break;
        }
        if (depth == 0) break;

        // descend to the near leaf; a far child becomes pending when the
        // bound of its cell (this cell's axis bounds, the split plane on its
        // axis) is within reach
        int ax = depth % D;
        while (depth < L) {
            const T m = depth < tv.smem_levels ? tv.s_med[node] : __ldg(tv.medians + node);
            const T qa = pick<T, D>(q, ax);
            const T diff = sub_rn(qa, m);
            const T plane = mul_rn(diff, diff);
            T fe[D];
#pragma unroll
            for (int c = 0; c < D; ++c) fe[c] = (c == ax) ? plane : e[c];
            const T fb = cell_bound<T, D>(fe);
            if (fb <= worst_d) {
                pending |= 1u << depth;
                if constexpr (NB > 0) {
                    if (gl == depth % G) {
#pragma unroll
                        for (int j = 0; j < NB; ++j)
                            if (depth / G == j) pb[j] = fb;
                    }
                }
            }
            node = 2 * node + (qa < m ? 1 : 2);  // src/kdtree.cpp:30
            ++depth;
            ax = (ax + 1 == D) ? 0 : ax + 1;
        }
    }
    list.store(k, gl, out_d, out_i, 0);
}

template <typename T, int D, int G, int R>
__device__ __forceinline__ void kd_query_one(const KdArgs<T>& a, const T* s_med, int qi, unsigned gmask, int gl,
                                             int gbase) {
    T q[D];
#pragma unroll
    for (int c = 0; c < D; ++c) q[c] = a.q[(long long)qi * D + c];
    const TreeView<T> tv{a.pts, a.medians, a.leaf_off, a.levels, a.smem_levels, s_med, a.boxes};
    kd_search<T, D, G, R>(tv, q, a.k, a.out_d + (long long)qi * a.k, a.out_i + (long long)qi * a.k, gmask, gl,
                          gbase);
}

constexpr int kKdBlock = 256;  // threads per block of the KD query kernels

// Dynamic shared memory of the KD query kernels: the top split values.
template <typename T>
inline size_t kd_smem_bytes(int smem_levels) {
    return sizeof(T) * ((size_t(1) << smem_levels) - 1);
}

template <typename T, int D, int G, int R>
__global__ void __launch_bounds__(kKdBlock) k_kd_query(const KdArgs<T> a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* s_med = reinterpret_cast<T*>(smem_raw);
    const int n_smem = (1 << a.smem_levels) - 1;
    for (int i = threadIdx.x; i < n_smem; i += blockDim.x) s_med[i] = a.medians[i];
    __syncthreads();

    const int lane = threadIdx.x & 31;
    const int gl = lane & (G - 1);
    const int gbase = lane & ~(G - 1);
    const unsigned gmask = group_mask<G>(lane);
    constexpr int kGroupsPerWarp = 32 / G;
    const int gid = lane / G;

    for (;;) {
        int base = 0;
        if (lane == 0) base = atomicAdd(a.work, kGroupsPerWarp);
        base = __shfl_sync(0xFFFFFFFFu, base, 0);
        if (base >= a.nq) break;
        const int t = base + gid;
        if (t < a.nq) {
            const int qi = a.order ? __ldg(a.order + t) : t;
            kd_query_one<T, D, G, R>(a, s_med, qi, gmask, gl, gbase);
        }
        __syncwarp();
    }
}

// ------------------------------------------------------- warp packets --
//
// Packet traversal: the 32 lanes of a warp each own one query (and their own
// register list of R <= 16 keys), but walk the tree TOGETHER, so the warp
// never diverges on the traversal itself.  Queries arrive binned by tree
// cell, so the 32 queries of a warp are neighbours and need mostly the same
// nodes.
//  1. Each lane first descends to its own home leaf (L steps for every lane,
//     no divergence) and fills its list from that leaf.
//  2. The warp then runs one depth-first walk from the root.  A node is
//     entered when its bounding box can still hold a neighbour of ANY lane
//     (per-lane box_bound <= that lane's worst, ballot); the near child is
//     the side most of the interested lanes fall on.  The stack of pending
//     nodes is warp-uniform and lives one entry per lane in a register
//     (depth-first with two pushes per internal node holds <= levels + 1
//     entries, below 32).
//  3. At a leaf every lane reads the same records (one broadcast load) and
//     offers them to its own list; a lane skips its home leaf, whose points
//     it has already offered.
// A lane examines every point the per-query search would (a node it needs is
// entered by the warp), plus others that cannot enter its list, so the
// result is again the exhaustive (distance, original index) answer.

template <typename T, int D, int R>
__device__ __forceinline__ void kd_packet_search(const TreeView<T>& tv, const T (&q)[D], bool active, int k,
                                                 T* out_d, int32_t* out_i, int lane) {
    TopK<T, 1, R> list;
    list.init(k, 0);
    Key<T> worst = Key<T>::sentinel();
    const int L = tv.levels;
    const int first_leaf = (1 << L) - 1;

    // 1. own descent and home leaf
    int node = 0, ax = 0;
    for (int depth = 0; depth < L; ++depth) {
        const T m = depth < tv.smem_levels ? tv.s_med[node] : __ldg(tv.medians + node);
        node = 2 * node + (pick<T, D>(q, ax) < m ? 1 : 2);  // src/kdtree.cpp:30
        ax = (ax + 1 == D) ? 0 : ax + 1;
    }
    const int home = node - first_leaf;
    {
        int beg = __ldg(tv.leaf_off + home);
        const int end = __ldg(tv.leaf_off + home + 1);
        if (k == R && end - beg >= R) {
            Key<T> v[R];
#pragma unroll
            for (int i = 0; i < R; ++i) {
                const PointRec<T> p = load_rec(tv.pts + beg + i);
                v[i] = Key<T>::make(sqdist<T, D>(q, p), rec_index(p));
            }
            bitonic_sort<T, R>(v);
#pragma unroll
            for (int i = 0; i < R; ++i) list.slot[i] = v[i];
            worst = list.worst(0u);
            beg += R;
        }
        for (int j = beg; j < end; ++j) {
            const PointRec<T> p = load_rec(tv.pts + j);
            worst = offer<T, 1, R>(list, Key<T>::make(sqdist<T, D>(q, p), rec_index(p)), worst, 0u, 0, 0);
        }
    }
    // A lane without a query needs nothing more, and neither does a query
    // with a NaN coordinate: all its distances are NaN, and a NaN key never
    // enters the list (it orders above the sentinel).
    bool nan_q = false;
#pragma unroll
    for (int c = 0; c < D; ++c) nan_q |= q[c] != q[c];
    T worst_d = (active && !nan_q) ? worst.dist() : T(-1);

    // 2./3. the warp's walk
    int stk = 0;  // this lane's stack slot; slot `lane` of the warp's stack
    int sp = 1;   // root on the stack
    while (sp > 0) {
        --sp;
        const int nd = __shfl_sync(0xFFFFFFFFu, stk, sp);
        const bool need = box_bound<T, D>(tv.boxes, nd, q) <= worst_d;
        const unsigned needm = __ballot_sync(0xFFFFFFFFu, need);
        if (!needm) continue;
        if (nd < first_leaf) {
            const int depth = 31 - __clz(nd + 1);
            const int nax = depth % D;
            const T m = depth < tv.smem_levels ? tv.s_med[nd] : __ldg(tv.medians + nd);
            const unsigned leftm = __ballot_sync(0xFFFFFFFFu, need && pick<T, D>(q, nax) < m);
            const bool near_left = 2 * __popc(leftm) >= __popc(needm);
            const int nearc = 2 * nd + (near_left ? 1 : 2);
            const int farc = 2 * nd + (near_left ? 2 : 1);
            if (lane == sp) stk = farc;
            if (lane == sp + 1) stk = nearc;
            sp += 2;
            continue;
        }
        const int leaf = nd - first_leaf;
        const bool take = need && leaf != home;
        if (!__any_sync(0xFFFFFFFFu, take)) continue;
        const int beg = __ldg(tv.leaf_off + leaf);
        const int end = __ldg(tv.leaf_off + leaf + 1);
        int j = beg;
        for (; j + 1 < end; j += 2) {
            const PointRec<T> p0 = load_rec(tv.pts + j);
            const PointRec<T> p1 = load_rec(tv.pts + j + 1);
            const Key<T> k0 = Key<T>::make(sqdist<T, D>(q, p0), rec_index(p0));
            const Key<T> k1 = Key<T>::make(sqdist<T, D>(q, p1), rec_index(p1));
            if (take) {
                worst = offer<T, 1, R>(list, k0, worst, 0u, 0, 0);
                worst = offer<T, 1, R>(list, k1, worst, 0u, 0, 0);
            }
        }
        if (j < end) {
            const PointRec<T> p = load_rec(tv.pts + j);
            const Key<T> k0 = Key<T>::make(sqdist<T, D>(q, p), rec_index(p));
            if (take) worst = offer<T, 1, R>(list, k0, worst, 0u, 0, 0);
        }
        if (take) worst_d = worst.dist();
    }
    if (active) list.store(k, 0, out_d, out_i, 0);
}

template <typename T, int D, int R>
__global__ void __launch_bounds__(256) k_kd_packet(const KdArgs<T> a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* s_med = reinterpret_cast<T*>(smem_raw);
    const int n_smem = (1 << a.smem_levels) - 1;
    for (int i = threadIdx.x; i < n_smem; i += blockDim.x) s_med[i] = a.medians[i];
    __syncthreads();

    const int lane = threadIdx.x & 31;
    const TreeView<T> tv{a.pts, a.medians, a.leaf_off, a.levels, a.smem_levels, s_med, a.boxes};
    for (;;) {
        int base = 0;
        if (lane == 0) base = atomicAdd(a.work, 32);
        base = __shfl_sync(0xFFFFFFFFu, base, 0);
        if (base >= a.nq) break;
        const int t = base + lane;
        const bool active = t < a.nq;
        const int qi = active ? (a.order ? __ldg(a.order + t) : t) : 0;
        T q[D];
#pragma unroll
        for (int c = 0; c < D; ++c) q[c] = active ? a.q[(long long)qi * D + c] : T(0);
        kd_packet_search<T, D, R>(tv, q, active, a.k, a.out_d + (long long)qi * a.k,
                                  a.out_i + (long long)qi * a.k, lane);
        __syncwarp();
    }
}

// ---------------------------------------------------------- query binning --

// Cell id at depth B of every query (same descent rule as the search), its
// arrival rank within the cell, and (with `boxes`) its cost class from the
// home leaf at depth L: bin_of = cell | class << 16 (B <= 16).
template <typename T, int D>
__global__ void k_bin_count(const T* __restrict__ q, int nq, const T* __restrict__ medians, int B, int L,
                            const PointRec<T>* __restrict__ boxes, int* __restrict__ counts,
                            int* __restrict__ bin_of, int* __restrict__ pos_of) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nq) return;
    T p[D];
#pragma unroll
    for (int c = 0; c < D; ++c) p[c] = q[(long long)i * D + c];
    int node = 0, ax = 0, bin = 0;
    const int stop = boxes ? L : B;
    for (int depth = 0; depth < stop; ++depth) {
        if (depth == B) bin = node - ((1 << B) - 1);
        const T m = __ldg(medians + node);
        node = 2 * node + (pick<T, D>(p, ax) < m ? 1 : 2);
        ax = (ax + 1 == D) ? 0 : ax + 1;
    }
    if (stop == B) bin = node - ((1 << B) - 1);
    uint32_t cls = 0;
    if (boxes) {
        const PointRec<T> lo = load_rec(boxes + 2 * node);
        const PointRec<T> hi = load_rec(boxes + 2 * node + 1);
        const T l[3] = {lo.x, lo.y, lo.z};
        const T h[3] = {hi.x, hi.y, hi.z};
        float far2 = 0.f;
#pragma unroll
        for (int c = 0; c < D; ++c) {
            const float f = float(fmax(fabs(p[c] - l[c]), fabs(p[c] - h[c])));
            far2 += f * f;
        }
        cls = cost_class(far2);
    }
    bin_of[i] = bin | int(cls << 16);
    pos_of[i] = atomicAdd(counts + bin, 1);
}

__global__ void k_bin_scatter(int nq, const int* bin_of, const int* pos_of, const int* offsets, int* order,
                              uint32_t* classes);

// Per-(T, D) launcher implemented in kd_query_<type>_d<D>.cu.
struct KdLaunch {
    int G, R;
    int block, grid;
    size_t smem;
};
template <typename T, int D>
int kd_query_launch(const KdArgs<T>& a, const KdLaunch& l, cudaStream_t s);
template <typename T, int D>
const void* kd_query_kernel(int G, int R);
template <typename T, int D>
int kd_packet_launch(const KdArgs<T>& a, const KdLaunch& l, cudaStream_t s);  // uses l.R only
template <typename T, int D>
const void* kd_packet_kernel(int R);
template <typename T, int D>
void bin_count_launch(const T* q, int nq, const T* medians, int B, int L, const PointRec<T>* boxes, int* counts,
                      int* bin_of, int* pos_of, cudaStream_t s);

}  // namespace tk
