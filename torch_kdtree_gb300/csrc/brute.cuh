// Exhaustive ("brute force") exact KNN: the nn_distance op.
//
// The reference's kernel (NmDistanceKernelDynamic, src/nndistance_g.cu:74-140)
// runs as ONE block for the whole problem, hard-codes d = 3 and keeps each
// thread's top-k list in a global scratch array.  Here:
//   * a block owns a tile of queries (one query per group of G lanes) and one
//     slice of the reference cloud; the grid is queries x slices so every SM
//     is busy even for few queries;
//   * reference points stream through shared memory in tiles, zero-padded to
//     DP dimensions (padding adds exact zeros, so distances are unchanged);
//   * distances use the reference's CPU arithmetic (sqdist order, no fused
//     multiply-add), so results match the KD-tree query bit for bit;
//   * each slice keeps the k best (distance, index) keys in registers (TopK);
//     with several slices a merge kernel combines the per-slice lists;
//   * with one lane per query a candidate is first tested as a float against
//     the list's worst distance (one compare), and only the rare survivors
//     build and compare the 64-bit (distance, index) key.
#pragma once

#include <cuda_runtime.h>

#include "tk_device.cuh"
#include "tk_internal.h"

namespace tk {

template <typename T>
struct BruteArgs {
    const T* ref;   // [n, d]
    const T* q;     // [nq, d]
    int n, nq, d, k;
    int nsplit;     // reference slices (gridDim.y)
    T* out_d;       // [nq, k]   (nsplit == 1)
    int32_t* out_i; // [nq, k]
    Key<T>* part;   // [nq, nsplit, k] per-slice lists (nsplit > 1)
    // Optional gather: when qlist is set, block slots index qlist[0..*qcount)
    // and results go to rows qlist[slot]; slots past *qcount do nothing.
    const int* qlist = nullptr;
    const int* qcount = nullptr;
};

// Reference rows per shared-memory tile: 32 KiB of coordinates, 32 to 256 rows.
template <typename T, int DP>
struct BruteTile {
    static constexpr int kElems = 32768 / int(sizeof(T));
    static constexpr int kRefs = (kElems / DP) > 256 ? 256 : ((kElems / DP) < 32 ? 32 : (kElems / DP));
};

template <typename T, int DP>
__device__ __forceinline__ T sqdist_padded(const T (&q)[DP], const T* r) {
    T d0 = sub_rn(q[0], r[0]);
    T acc = mul_rn(d0, d0);
#pragma unroll
    for (int c = 1; c < DP; ++c) {
        const T dc = sub_rn(q[c], r[c]);
        acc = add_rn(acc, mul_rn(dc, dc));
    }
    return acc;
}

template <typename T, int DP, int G, int R>
__global__ void __launch_bounds__(256) k_brute(const BruteArgs<T> a) {
    constexpr int TR = BruteTile<T, DP>::kRefs;
    __shared__ __align__(16) T tile[TR * DP];
    const int lane = threadIdx.x & 31;
    const int gl = lane & (G - 1);
    const int gbase = lane & ~(G - 1);
    const unsigned gmask = group_mask<G>(lane);
    const int slot = blockIdx.x * (blockDim.x / G) + threadIdx.x / G;
    int live = a.nq;
    if (a.qlist) {
        live = *a.qcount;
        if (int(blockIdx.x * (blockDim.x / G)) >= live) return;  // whole block idle (uniform)
    }
    const bool active = slot < live;
    const int qi = active ? (a.qlist ? a.qlist[slot] : slot) : 0;

    T q[DP];
#pragma unroll
    for (int c = 0; c < DP; ++c) q[c] = (active && c < a.d) ? a.q[(long long)qi * a.d + c] : T(0);

    TopK<T, G, R> list;
    list.init(a.k, gl);
    Key<T> worst = Key<T>::sentinel();

    const long long per = ((long long)a.n + a.nsplit - 1) / a.nsplit;
    const int r0 = int(min((long long)a.n, per * blockIdx.y));
    const int r1 = int(min((long long)a.n, per * (blockIdx.y + 1)));
    for (int t0 = r0; t0 < r1; t0 += TR) {
        const int len = min(TR, r1 - t0);
        __syncthreads();
        for (int e = threadIdx.x; e < TR * DP; e += blockDim.x) {
            const int j = e / DP, c = e - j * DP;
            tile[e] = (j < len && c < a.d) ? a.ref[(long long)(t0 + j) * a.d + c] : T(0);
        }
        __syncthreads();
        if constexpr (G == 1 && DP % 4 == 0 && sizeof(T) == 4) {
            // One lane per query: every lane reads the same reference row, so
            // a 16-byte shared load broadcasts four coordinates to the warp;
            // four references per step give four independent chains.  Same
            // accumulation order as sqdist (dimension by dimension).
            constexpr int U = 4;
            static_assert(TR % U == 0, "tile rows must be a multiple of the step");
            if (active) {
                const float4* rows = reinterpret_cast<const float4*>(tile);
                for (int j0 = 0; j0 < len; j0 += U) {
                    T acc[U];
#pragma unroll
                    for (int u = 0; u < U; ++u) {
                        const float4 v = rows[(j0 + u) * (DP / 4)];
                        const T d0 = sub_rn(q[0], v.x), d1 = sub_rn(q[1], v.y);
                        const T d2 = sub_rn(q[2], v.z), d3 = sub_rn(q[3], v.w);
                        acc[u] = mul_rn(d0, d0);
                        acc[u] = add_rn(acc[u], mul_rn(d1, d1));
                        acc[u] = add_rn(acc[u], mul_rn(d2, d2));
                        acc[u] = add_rn(acc[u], mul_rn(d3, d3));
                    }
#pragma unroll
                    for (int c4 = 1; c4 < DP / 4; ++c4) {
#pragma unroll
                        for (int u = 0; u < U; ++u) {
                            const float4 v = rows[(j0 + u) * (DP / 4) + c4];
                            const T d0 = sub_rn(q[4 * c4], v.x), d1 = sub_rn(q[4 * c4 + 1], v.y);
                            const T d2 = sub_rn(q[4 * c4 + 2], v.z), d3 = sub_rn(q[4 * c4 + 3], v.w);
                            acc[u] = add_rn(acc[u], mul_rn(d0, d0));
                            acc[u] = add_rn(acc[u], mul_rn(d1, d1));
                            acc[u] = add_rn(acc[u], mul_rn(d2, d2));
                            acc[u] = add_rn(acc[u], mul_rn(d3, d3));
                        }
                    }
#pragma unroll
                    for (int u = 0; u < U; ++u) {
                        if (j0 + u < len && acc[u] <= worst.dist())
                            worst = offer<T, G, R>(list, Key<T>::make(acc[u], uint32_t(t0 + j0 + u)), worst, gmask,
                                                   gl, gbase);
                    }
                }
            }
        } else if (active) {
            // four references per lane step: four independent accumulation chains
            constexpr int U = DP <= 4 ? 1 : ((DP > 32 || R >= 16) ? 2 : 4);
            for (int j0 = 0; j0 < len; j0 += G * U) {
                T acc[U];
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const int j = min(j0 + u * G + gl, TR - 1);  // rows past len are padding zeros
                    const T* r = tile + j * DP;
                    const T d0 = sub_rn(q[0], r[0]);
                    acc[u] = mul_rn(d0, d0);
                }
#pragma unroll
                for (int c = 1; c < DP; ++c) {
#pragma unroll
                    for (int u = 0; u < U; ++u) {
                        const int j = min(j0 + u * G + gl, TR - 1);
                        const T dc = sub_rn(q[c], tile[j * DP + c]);
                        acc[u] = add_rn(acc[u], mul_rn(dc, dc));
                    }
                }
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const int j = j0 + u * G + gl;
                    if constexpr (G == 1) {
                        if (j < len && acc[u] <= worst.dist())
                            worst = offer<T, G, R>(list, Key<T>::make(acc[u], uint32_t(t0 + j)), worst, gmask, gl,
                                                   gbase);
                    } else {
                        Key<T> mine = Key<T>::sentinel();
                        if (j < len) mine = Key<T>::make(acc[u], uint32_t(t0 + j));
                        worst = offer<T, G, R>(list, mine, worst, gmask, gl, gbase);
                    }
                }
            }
        }
    }
    if (!active) return;
    if (a.nsplit == 1) {
        list.store(a.k, gl, a.out_d, a.out_i, qi);
    } else {
        Key<T>* dst = a.part + ((long long)slot * a.nsplit + blockIdx.y) * a.k;
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int s = r * G + gl;
            const int o = s - (G * R - a.k);
            if (o >= 0) dst[o] = list.slot[r];
        }
    }
}

// Combine the per-slice lists of every query (group of G lanes per query).
template <typename T, int G, int R>
__global__ void __launch_bounds__(256) k_brute_merge(const BruteArgs<T> a) {
    const int lane = threadIdx.x & 31;
    const int gl = lane & (G - 1);
    const int gbase = lane & ~(G - 1);
    const unsigned gmask = group_mask<G>(lane);
    const int slot = blockIdx.x * (blockDim.x / G) + threadIdx.x / G;
    const int live = a.qlist ? *a.qcount : a.nq;
    if (slot >= live) return;  // whole groups leave together
    const int qi = a.qlist ? a.qlist[slot] : slot;
    TopK<T, G, R> list;
    list.init(a.k, gl);
    Key<T> worst = Key<T>::sentinel();
    const Key<T>* src = a.part + (long long)slot * a.nsplit * a.k;
    const int total = a.nsplit * a.k;
    for (int e0 = 0; e0 < total; e0 += G) {
        const int e = e0 + gl;
        const Key<T> mine = e < total ? src[e] : Key<T>::sentinel();
        worst = offer<T, G, R>(list, mine, worst, gmask, gl, gbase);
    }
    list.store(a.k, gl, a.out_d, a.out_i, qi);
}

// Exact search for the queries listed on the device (qlist[0..*qcount)),
// results written to their rows of dists / idx (brute.cu).
size_t brute_fallback_workspace_bytes(int64_t n, int64_t nq, int d, int k);
int brute_fallback(const float* ref, int64_t n, const float* q, int64_t nq, int d, int k, float* dists,
                   int32_t* idx, const int* qlist, const int* qcount, void* ws, size_t ws_bytes, cudaStream_t s);

// Launch shape of an exhaustive search (brute.cu: plan_brute).
struct BrutePlan {
    int DP, G, R, nsplit, qtiles;
};

template <typename T, int DP>
int launch_dp(const BruteArgs<T>& a, const BrutePlan& p, cudaStream_t s) {
    dim3 grid(p.qtiles, p.nsplit);
    bool done = false;
#define TK_BR(g, r)                                                          \
    if (!done && p.G == g && p.R == r) {                                     \
        k_brute<T, DP, g, r><<<grid, 256, 0, s>>>(a);                        \
        if (p.nsplit > 1) k_brute_merge<T, g, r><<<p.qtiles, 256, 0, s>>>(a); \
        done = true;                                                         \
    }
    TK_BR(1, 1) TK_BR(1, 4) TK_BR(1, 16) TK_BR(2, 16) TK_BR(4, 16) TK_BR(8, 16)
    if constexpr (sizeof(T) == 4 && DP % 4 == 0 && DP <= 32) {
        TK_BR(1, 32)
    }
#undef TK_BR
    if (!done) return fail(TK_EUNSUPPORTED, "no brute-force kernel for this k");
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(TK_ECUDA, std::string("brute-force launch: ") + cudaGetErrorString(e));
    return TK_OK;
}

// float64 searches of 5 to 128 dimensions (brute_f64.cu, a unit of its own).
int launch_brute_f64_wide(const BruteArgs<double>& a, const BrutePlan& p, cudaStream_t s);

}  // namespace tk
