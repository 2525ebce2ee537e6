// Exact KD-tree KNN query for trees of 4 to 8 dimensions (sm_103a).
//
// The reference compiles its KD-tree for dims 1-3 and tells users to add
// template instantiations for more (its README); the query is the same
// algorithm at any dimension.  Trees of up to 3 dimensions keep the 16-byte
// point records of kd_query.cuh; here, a tree of `dims` in 4..8 stores
// W = 4 (dims 4), 6 (dims 5-6) or 8 (dims 7-8) zero-padded coordinates per point, its
// original indices in a separate array, and node boxes as lo / hi rows of W.
// Padded coordinates are 0 in both the records and the (padded) query, so
// each adds (0 - 0)^2 = +0 to the distance after the real terms: the sum is
// the reference's ((0 + d0^2) + d1^2) + ... bit for bit.  The split axis
// cycles with the real `dims`.
//
// The search is kd_search's (exact per-axis plane bounds on a stack of far
// cells, node-box pruning, queries binned by cell, persistent warps), with
// one lane per query (k <= 16) or a 32-lane group per query (k <= 128).  A
// leaf point is first tested as a float against the list's worst distance;
// only candidates that pass load their original index and build the
// (distance, index) key.
#pragma once

#include <cuda_runtime.h>

#include "tk_device.cuh"
#include "tk_internal.h"

namespace tk {

template <typename T>
struct KdWideArgs {
    const T* pts;             // [n][W] coordinates in leaf order, zero padded
    const int32_t* perm;      // [n] original index of each point
    const T* medians;         // [2^L - 1] heap order
    const int32_t* leaf_off;  // [2^L + 1]
    const T* boxes;           // [2 (2^(L+1) - 1)][W]: node i's lo row at 2i, hi row at 2i+1; or null
    int levels, smem_levels, dims;
    const T* q;               // [nq, dims]
    int nq, k;
    const int32_t* order;     // [nq] processing order (binned), or null
    T* out_d;                 // [nq, k]
    int32_t* out_i;           // [nq, k]
    int* work;                // global work counter, zero at launch
};

template <typename T, int W>
struct WideEntry {
    int node;
    T e[W];  // per-axis squared distance from the query to the cell's slab
};

// v[ax] for a run-time axis without indexing a register array dynamically
template <typename T, int W>
__device__ __forceinline__ T pick_w(const T (&v)[W], int ax) {
    T r = v[0];
#pragma unroll
    for (int c = 1; c < W; ++c) r = ax == c ? v[c] : r;
    return r;
}

template <typename T, int W>
__device__ __forceinline__ T sum_w(const T (&e)[W]) {
    T b = e[0];
#pragma unroll
    for (int c = 1; c < W; ++c) b = add_rn(b, e[c]);
    return b;
}

// Rows start at multiples of 4 W bytes (f32) or 8 W bytes (f64) from a
// cudaMalloc base: 16-byte loads for W = 4 and 8, 8-byte loads for W = 6 (f32).
template <typename T, int W>
__device__ __forceinline__ void load_row(const T* row, T (&c)[W]) {
    static_assert(W % 2 == 0, "rows of an even number of coordinates");
    if constexpr (sizeof(T) == 4 && W % 4 == 0) {
#pragma unroll
        for (int i = 0; i < W / 4; ++i) {
            const float4 v = __ldg(reinterpret_cast<const float4*>(row) + i);
            c[4 * i] = v.x;
            c[4 * i + 1] = v.y;
            c[4 * i + 2] = v.z;
            c[4 * i + 3] = v.w;
        }
    } else if constexpr (sizeof(T) == 4) {
#pragma unroll
        for (int i = 0; i < W / 2; ++i) {
            const float2 v = __ldg(reinterpret_cast<const float2*>(row) + i);
            c[2 * i] = v.x;
            c[2 * i + 1] = v.y;
        }
    } else {
#pragma unroll
        for (int i = 0; i < W / 2; ++i) {
            const double2 v = __ldg(reinterpret_cast<const double2*>(row) + i);
            c[2 * i] = v.x;
            c[2 * i + 1] = v.y;
        }
    }
}

// The reference's distance arithmetic over W (zero-padded) coordinates.
template <typename T, int W>
__device__ __forceinline__ T sqdist_w(const T (&q)[W], const T (&p)[W]) {
    const T d0 = sub_rn(q[0], p[0]);
    T acc = mul_rn(d0, d0);
#pragma unroll
    for (int c = 1; c < W; ++c) {
        const T dc = sub_rn(q[c], p[c]);
        acc = add_rn(acc, mul_rn(dc, dc));
    }
    return acc;
}

// Lower bound on the computed distance to any point in node's box (as
// box_bound in kd_query.cuh, over W coordinates).
template <typename T, int W>
__device__ __forceinline__ T box_bound_w(const T* boxes, int node, const T (&q)[W]) {
    T lo[W], hi[W], e[W];
    load_row<T, W>(boxes + size_t(2 * node) * W, lo);
    load_row<T, W>(boxes + size_t(2 * node + 1) * W, hi);
#pragma unroll
    for (int c = 0; c < W; ++c) {
        const T g = q[c] < lo[c] ? sub_rn(q[c], lo[c]) : (q[c] > hi[c] ? sub_rn(q[c], hi[c]) : T(0));
        e[c] = mul_rn(g, g);
    }
    return sum_w<T, W>(e);
}

template <typename T, int W, int G, int R>
__device__ __forceinline__ void kd_search_wide(const KdWideArgs<T>& a, const T* s_med, const T (&q)[W], T* out_d,
                                               int32_t* out_i, unsigned gmask, int gl, int gbase) {
    TopK<T, G, R> list;
    list.init(a.k, gl);
    Key<T> worst = Key<T>::sentinel();
    T worst_d = worst.dist();
    // Stack of far cells.  A 32-lane group's control flow is uniform, so its
    // stack lives in the group's registers, entry j in lane j (levels <= 24 <
    // 32): a push is a register move in one lane, a pop W + 1 shuffles.  Each
    // lane holding its own copy of the 36-byte entries in local memory missed
    // L1 on 98% of the pops (1M-point 8-D tree), and this form measured 2-6%
    // faster at d = 6-8.  (For 3-D trees the private copies mostly hit L1 and
    // measured faster.)  One lane per query keeps a private local array.
    constexpr bool RS = G == 32;
    WideEntry<T, W> stk[RS ? 1 : kMaxLevels];
    int rs_node = 0;
    T rs_e[W];
    int sp = 0;
    int node = 0, depth = 0;
    T e[W];
#pragma unroll
    for (int c = 0; c < W; ++c) e[c] = T(0);
    const int L = a.levels, dims = a.dims;
    const int first_leaf = (1 << L) - 1;

    for (;;) {
        int ax = depth % dims;
        while (depth < L) {
            const T m = depth < a.smem_levels ? s_med[node] : __ldg(a.medians + node);
            const T qa = pick_w<T, W>(q, ax);
            const T diff = sub_rn(qa, m);
            const T plane = mul_rn(diff, diff);
            const bool go_left = qa < m;  // src/kdtree.cpp:30
            WideEntry<T, W> far;
            far.node = 2 * node + (go_left ? 2 : 1);
#pragma unroll
            for (int c = 0; c < W; ++c) far.e[c] = (c == ax) ? plane : e[c];
            if (sum_w<T, W>(far.e) <= worst_d) {
                if constexpr (RS) {
                    if (gl == sp) {
                        rs_node = far.node;
#pragma unroll
                        for (int c = 0; c < W; ++c) rs_e[c] = far.e[c];
                    }
                } else {
                    stk[sp] = far;
                }
                ++sp;
            }
            node = 2 * node + (go_left ? 1 : 2);
            ++depth;
            ax = (ax + 1 == dims) ? 0 : ax + 1;
        }
        if (!a.boxes || box_bound_w<T, W>(a.boxes, node, q) <= worst_d) {
            const int leaf = node - first_leaf;
            const int beg = __ldg(a.leaf_off + leaf);
            const int end = __ldg(a.leaf_off + leaf + 1);
            if constexpr (G == 1) {
                for (int j = beg; j < end; ++j) {
                    T p[W];
                    load_row<T, W>(a.pts + size_t(j) * W, p);
                    const T d = sqdist_w<T, W>(q, p);
                    if (d <= worst.dist())
                        worst = offer<T, G, R>(list, Key<T>::make(d, uint32_t(__ldg(a.perm + j))), worst, gmask,
                                               gl, gbase);
                }
            } else {
                for (int j0 = beg; j0 < end; j0 += G) {
                    const int j = j0 + gl;
                    Key<T> mine = Key<T>::sentinel();
                    if (j < end) {
                        T p[W];
                        load_row<T, W>(a.pts + size_t(j) * W, p);
                        const T d = sqdist_w<T, W>(q, p);
                        if (d <= worst.dist()) mine = Key<T>::make(d, uint32_t(__ldg(a.perm + j)));
                    }
                    worst = offer<T, G, R>(list, mine, worst, gmask, gl, gbase);
                }
            }
            worst_d = worst.dist();
        }
        bool resumed = false;
        while (sp > 0) {
            --sp;
            WideEntry<T, W> s;
            if constexpr (RS) {
                s.node = __shfl_sync(gmask, rs_node, sp);
#pragma unroll
                for (int c = 0; c < W; ++c) s.e[c] = __shfl_sync(gmask, rs_e[c], sp);
            } else {
                s = stk[sp];
            }
            if (sum_w<T, W>(s.e) <= worst_d && (!a.boxes || box_bound_w<T, W>(a.boxes, s.node, q) <= worst_d)) {
                node = s.node;
#pragma unroll
                for (int c = 0; c < W; ++c) e[c] = s.e[c];
                depth = 31 - __clz(node + 1);
                resumed = true;
                break;
            }
        }
        if (!resumed) break;
    }
    list.store(a.k, gl, out_d, out_i, 0);
}

template <typename T, int W, int G, int R>
__global__ void __launch_bounds__(256) k_kd_wide(const KdWideArgs<T> a) {
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
            T q[W];
#pragma unroll
            for (int c = 0; c < W; ++c) q[c] = c < a.dims ? a.q[(long long)qi * a.dims + c] : T(0);
            kd_search_wide<T, W, G, R>(a, s_med, q, a.out_d + (long long)qi * a.k, a.out_i + (long long)qi * a.k,
                                       gmask, gl, gbase);
        }
        __syncwarp();
    }
}

// Cell id at depth B of every query (axis cycling over the real dims), its
// arrival rank within the cell, and (with `boxes`, rows of width W) its cost
// class from the home leaf at depth L, as k_bin_count for narrow trees:
// bin_of = cell | class << 16.  Ordering the launch by class took 7-8% off
// the 4- and 8-dim searches of 262,144 queries in 1,048,576 N(0,1) points.
template <typename T>
__global__ void k_bin_count_wide(const T* __restrict__ q, int nq, int dims, const T* __restrict__ medians, int B,
                                 int L, const T* __restrict__ boxes, int W, int* __restrict__ counts,
                                 int* __restrict__ bin_of, int* __restrict__ pos_of) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nq) return;
    const T* p = q + (long long)i * dims;
    int node = 0, ax = 0, bin = 0;
    const int stop = boxes ? L : B;
    for (int depth = 0; depth < stop; ++depth) {
        if (depth == B) bin = node - ((1 << B) - 1);
        const T m = __ldg(medians + node);
        node = 2 * node + (p[ax] < m ? 1 : 2);
        ax = (ax + 1 == dims) ? 0 : ax + 1;
    }
    if (stop == B) bin = node - ((1 << B) - 1);
    uint32_t cls = 0;
    if (boxes) {
        const T* lo = boxes + size_t(2 * node) * W;
        const T* hi = lo + W;
        float far2 = 0.f;
        for (int c = 0; c < dims; ++c) {
            const T x = p[c];
            const float f = float(fmax(fabs(x - __ldg(lo + c)), fabs(x - __ldg(hi + c))));
            far2 += f * f;
        }
        cls = cost_class(far2);
    }
    bin_of[i] = bin | int(cls << 16);
    pos_of[i] = atomicAdd(counts + bin, 1);
}

// Launchers (kd_wide_f32.cu, kd_wide_f64.cu): G in {1, 32}; R in {1, 2, 4, 8,
// 16} for G = 1, {1, 2, 4} for G = 32.
template <typename T>
const void* kd_wide_kernel(int W, int G, int R);
template <typename T>
int kd_wide_launch(const KdWideArgs<T>& a, int W, int G, int R, int grid, int block, size_t smem, cudaStream_t s);
template <typename T>
void bin_count_wide_launch(const T* q, int nq, int dims, const T* medians, int B, int L, const T* boxes, int W,
                           int* counts, int* bin_of, int* pos_of, cudaStream_t s);

}  // namespace tk
