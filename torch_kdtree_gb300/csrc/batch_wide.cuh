// Batched queries over many trees of 4-8 dimensions in one persistent launch:
// the plan and launch of batch.cu with the wide trees' records and search
// (kd_wide.cuh).  Every cloud of a batch has the same dims, so one record
// width W serves the whole launch; each group looks up its query's cloud and
// runs kd_search_wide with that cloud's tree and k.
#pragma once

#include <cuda_runtime.h>

#include "kd_wide.cuh"

namespace tk {

// Cloud of query qi (a global query index): prefix[c] <= qi < prefix[c + 1].
__device__ __forceinline__ int batch_cloud_of(const long long* prefix, int n_clouds, long long qi) {
    int lo = 0, hi = n_clouds;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (prefix[mid] <= qi) lo = mid; else hi = mid;
    }
    return lo;
}

template <typename T>
struct WideCloudDesc {
    const T* pts;             // [n][W] coordinates in leaf order
    const int32_t* perm;      // [n] original indices
    const T* medians;
    const int32_t* leaf_off;
    const T* boxes;           // lo / hi rows of W per node
    long long out_off;        // element offset of the cloud's [nq_c, k_c] block in the outputs
    int levels, k;
    int bins;                 // 2^B_c cells used for binning
    int bin_base;             // first cell of this cloud in the global cell array
};

template <typename T>
struct WideBatchArgs {
    const WideCloudDesc<T>* desc;
    const long long* q_prefix;  // [n_clouds + 1]
    int n_clouds, dims;
    const T* q;                 // concatenated queries [total, dims]
    int total;
    const int32_t* order;
    T* out_d;
    int32_t* out_i;
    int* work;
};

template <typename T>
__global__ void k_batch_bin_count_wide(const WideBatchArgs<T> a, int* counts, int* bin_of, int* pos_of) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.total) return;
    const int c = batch_cloud_of(a.q_prefix, a.n_clouds, i);
    const WideCloudDesc<T> cd = a.desc[c];
    int B = 0;
    while ((1 << B) < cd.bins) ++B;
    int node = 0, ax = 0;
    for (int depth = 0; depth < B; ++depth) {
        const T m = __ldg(cd.medians + node);
        node = 2 * node + (a.q[(long long)i * a.dims + ax] < m ? 1 : 2);  // src/kdtree.cpp:30
        ax = (ax + 1 == a.dims) ? 0 : ax + 1;
    }
    const int bin = cd.bin_base + node - ((1 << B) - 1);
    bin_of[i] = bin;
    pos_of[i] = atomicAdd(counts + bin, 1);
}

template <typename T, int W, int G, int R>
__device__ __forceinline__ void batch_search_wide(const WideCloudDesc<T>& cd, int dims, const T (&q)[W],
                                                  T* out_d, int32_t* out_i, unsigned gmask, int gl, int gbase) {
    KdWideArgs<T> wa{};
    wa.pts = cd.pts;
    wa.perm = cd.perm;
    wa.medians = cd.medians;
    wa.leaf_off = cd.leaf_off;
    wa.boxes = cd.boxes;
    wa.levels = cd.levels;
    wa.smem_levels = 0;  // split values come from L1 / L2: one launch serves many trees
    wa.dims = dims;
    wa.k = cd.k;
    kd_search_wide<T, W, G, R>(wa, nullptr, q, out_d, out_i, gmask, gl, gbase);
}

// G = 1: k <= 16 (R in {1, 4, 16}); G = 32: k <= 128 (R in {1, 2, 4}).
template <typename T, int W, int G>
__device__ __forceinline__ void batch_query_wide(const WideBatchArgs<T>& a) {
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
        if (base >= a.total) break;
        const int t = base + gid;
        if (t < a.total) {
            const int qi = a.order ? __ldg(a.order + t) : t;
            const int c = batch_cloud_of(a.q_prefix, a.n_clouds, qi);
            const WideCloudDesc<T> cd = a.desc[c];
            T q[W];
#pragma unroll
            for (int j = 0; j < W; ++j) q[j] = j < a.dims ? a.q[(long long)qi * a.dims + j] : T(0);
            const long long o = cd.out_off + (qi - a.q_prefix[c]) * cd.k;
            T* od = a.out_d + o;
            int32_t* oi = a.out_i + o;
            if (G == 1) {
                if (cd.k <= 1) batch_search_wide<T, W, G, 1>(cd, a.dims, q, od, oi, gmask, gl, gbase);
                else if (cd.k <= 4) batch_search_wide<T, W, G, 4>(cd, a.dims, q, od, oi, gmask, gl, gbase);
                else batch_search_wide<T, W, G, 16>(cd, a.dims, q, od, oi, gmask, gl, gbase);
            } else {
                if (cd.k <= 32) batch_search_wide<T, W, G, 1>(cd, a.dims, q, od, oi, gmask, gl, gbase);
                else if (cd.k <= 64) batch_search_wide<T, W, G, 2>(cd, a.dims, q, od, oi, gmask, gl, gbase);
                else batch_search_wide<T, W, G, 4>(cd, a.dims, q, od, oi, gmask, gl, gbase);
            }
        }
        __syncwarp();
    }
}

// One lane per query: registers left to the compiler.
template <typename T, int W>
__global__ void __launch_bounds__(256) k_batch_query_wide1(const WideBatchArgs<T> a) {
    batch_query_wide<T, W, 1>(a);
}

// 32 lanes per query, capped at 4 blocks of 256 per SM (64 registers for
// float): left free they took 80-117 registers and ran 64 clouds of 4 / 6 / 8
// dims 14% / 7% / 32% slower.
template <typename T, int W>
__global__ void __launch_bounds__(256, 4) k_batch_query_wide32(const WideBatchArgs<T> a) {
    batch_query_wide<T, W, 32>(a);
}

// Launchers (batch_wide_f32.cu, batch_wide_f64.cu): W in {4, 6, 8}, G in {1, 32}.
template <typename T>
const void* batch_wide_kernel(int W, int G);
template <typename T>
int batch_wide_launch(const WideBatchArgs<T>& a, int W, int G, int grid, cudaStream_t s);
template <typename T>
void batch_wide_bin_launch(const WideBatchArgs<T>& a, int* counts, int* bin_of, int* pos_of, cudaStream_t s);

}  // namespace tk
