// Deterministic backward of the KNN squared distances.
//
// Forward: dist[i, j] = sum_c (q[i, c] - ref[m, c])^2 with m = idx[i, j].
// The reference differentiates a torch re-gather of these distances
// (torch_kdtree/nn_distance.py:111-112), whose ref gradient goes through
// index_put_ with accumulate -- float atomics, run-to-run nondeterministic.
// Here:
//   grad_q[i]   = sum_j 2 g[i, j] (q[i] - ref[idx[i, j]])       (a gather, j ascending)
//   grad_ref[m] = sum_{(i,j): idx[i,j] = m} 2 g[i, j] (ref[m] - q[i])
// grad_ref is a segmented reduction over the indices, bitwise reproducible and
// without float atomics: segments are built by counting (integer atomics,
// whose returned ranks then place each pair), so the order inside a segment
// is arbitrary, and the segment's sum is made order-independent instead.  One
// pass finds the largest exponent of its terms per coordinate, a second adds
// every term as a fixed-point integer scaled to that exponent (64-bit for
// float32 terms, 128-bit for float64), and the total is rounded once -- the
// same bits whatever the order, and closer to the exact sum than a sequential
// sum in the terms' own precision.  Coordinates go 8 per pass (registers).
// Differences are recomputed from the saved indices; nothing of size
// [Q, k, d] is stored.
#include <algorithm>
#include <string>

#include "sort.cuh"
#include "tk_internal.h"

namespace tk {
namespace {

size_t align256(size_t v) { return (v + 255) / 256 * 256; }

// D: compile-time upper bound of the runtime dimension d (d <= D).
template <typename T, int D>
__global__ void k_grad_q(const T* __restrict__ q, const T* __restrict__ ref, const int32_t* __restrict__ idx,
                         const T* __restrict__ g, int nq, int n, int k, int d, T* __restrict__ grad_q) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nq) return;
    T qi[D], acc[D];
#pragma unroll
    for (int c = 0; c < D; ++c) {
        qi[c] = c < d ? q[(long long)i * d + c] : T(0);
        acc[c] = T(0);
    }
    for (int j = 0; j < k; ++j) {
        const int m = idx[(long long)i * k + j];
        if (m < 0 || m >= n) continue;
        const T w = T(2) * g[(long long)i * k + j];
#pragma unroll
        for (int c = 0; c < D; ++c)
            if (c < d) acc[c] += w * (qi[c] - ref[(long long)m * d + c]);
    }
#pragma unroll
    for (int c = 0; c < D; ++c)
        if (c < d) grad_q[(long long)i * d + c] = acc[c];
}

// Segments by counting: counts of every key (then their
// exclusive scan, n + 1 entries: starts, and the total at n), and each pair's
// arrival rank within its key, which places it in the segment without a
// second round of atomics.
__global__ void k_count_keys(const int32_t* __restrict__ idx, long long npairs, int n, int* __restrict__ cnt,
                             int* __restrict__ rank) {
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npairs) return;
    const int m = idx[p];
    rank[p] = (m >= 0 && m < n) ? atomicAdd(cnt + m, 1) : -1;
}

// Every valid pair into its key's segment (arbitrary order within it).
__global__ void k_fill_segments(const int32_t* __restrict__ idx, long long npairs, int n,
                                const int* __restrict__ starts, const int* __restrict__ rank,
                                uint32_t* __restrict__ list) {
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npairs) return;
    const int m = idx[p];
    if (m < 0 || m >= n) return;
    list[starts[m] + rank[p]] = uint32_t(p);
}

// Exponent field of a float (0 for zeros and subnormals, 255 for inf / NaN).
__device__ __forceinline__ int exp_field(float t) { return int((__float_as_uint(t) >> 23) & 0xFFu); }

// 2^e as a double, e in [-1022, 1023].
__device__ __forceinline__ double pow2(int e) { return __longlong_as_double((long long)(1023 + e) << 52); }

// t * 2^sh rounded to the nearest integer (halves away from zero), in integer
// arithmetic: a finite float is mant * 2^(max(e, 1) - 150) with its 24-bit
// significand mant.  The caller guarantees |t * 2^sh| < 2^61.
__device__ __forceinline__ long long to_fixed(float t, int sh) {
    const uint32_t b = __float_as_uint(t);
    const int e = int((b >> 23) & 0xFFu);
    const long long mant = (long long)((b & 0x7FFFFFu) | (e ? 0x800000u : 0u));
    const int amt = (e ? e : 1) - 150 + sh;
    long long v;
    if (amt >= 0)
        v = mant << amt;
    else if (amt > -25)
        v = (mant + (1ll << (-amt - 1))) >> (-amt);
    else
        v = 0;  // below half a unit
    return (b >> 31) ? -v : v;
}

// One thread per reference point: the order-independent sum of its segment
// (see the top of this file).  A term t has |t| < 2^(E - 126) for the largest
// exponent field E of its coordinate; scaled by 2^(187 - L - E), with s <
// 2^L terms in the segment, each scaled term is below 2^(61 - L) and the sum
// below 2^61, so the int64 accumulator cannot overflow.  Each scaled term is
// rounded to an integer once (to_fixed), by a rule that does not depend on
// the order.
// This pass: coordinates c0 .. c0 + dc - 1, dc = min(D, d - c0) <= 8.
template <int D>
__global__ void k_grad_ref_fixed(const float* __restrict__ q, const float* __restrict__ ref, const float* __restrict__ g,
                                 const uint32_t* __restrict__ list, const int* __restrict__ starts, int n, int k, int d,
                                 int c0, float* __restrict__ grad_ref) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= n) return;
    const int dc = min(D, d - c0);
    q += c0;
    float rm[D];
#pragma unroll
    for (int c = 0; c < D; ++c) rm[c] = c < dc ? ref[(long long)m * d + c0 + c] : 0.f;
    const int s0 = starts[m], s1 = starts[m + 1];
    int emax[D];
#pragma unroll
    for (int c = 0; c < D; ++c) emax[c] = 0;
    bool finite = true;
    // d <= 3: the first kKeep terms stay in registers for the second pass
    constexpr int kKeep = D <= 3 ? 8 : 0;
    float keep[kKeep > 0 ? kKeep : 1][D];
#pragma unroll
    for (int u = 0; u < kKeep; ++u) {
        if (s0 + u < s1) {
            const uint32_t p = list[s0 + u];
            const long long i = (long long)(p / uint32_t(k));
            const float w = 2.f * g[p];
#pragma unroll
            for (int c = 0; c < D; ++c) {
                keep[u][c] = __fmul_rn(w, __fsub_rn(rm[c], (c < dc ? q[i * d + c] : rm[c])));
                const int e = exp_field(keep[u][c]);
                finite = finite && e != 255;
                emax[c] = max(emax[c], e);
            }
        }
    }
    for (int j = s0 + kKeep; j < s1; ++j) {
        const uint32_t p = list[j];
        const long long i = (long long)(p / uint32_t(k));
        const float w = 2.f * g[p];
#pragma unroll
        for (int c = 0; c < D; ++c) {
            const int e = exp_field(__fmul_rn(w, __fsub_rn(rm[c], (c < dc ? q[i * d + c] : rm[c]))));
            finite = finite && e != 255;
            emax[c] = max(emax[c], e);
        }
    }
    float out[D];
    if (!finite) {
        // an infinite or NaN term: the sum is +-inf or NaN in any order
#pragma unroll
        for (int c = 0; c < D; ++c) out[c] = 0.f;
        for (int j = s0; j < s1; ++j) {
            const uint32_t p = list[j];
            const long long i = (long long)(p / uint32_t(k));
            const float w = 2.f * g[p];
#pragma unroll
            for (int c = 0; c < D; ++c) out[c] += __fmul_rn(w, __fsub_rn(rm[c], (c < dc ? q[i * d + c] : rm[c])));
        }
    } else {
        const int L = 32 - __clz(s1 - s0);  // s1 - s0 < 2^L
        long long acc[D];
#pragma unroll
        for (int c = 0; c < D; ++c) acc[c] = 0;
#pragma unroll
        for (int u = 0; u < kKeep; ++u)
            if (s0 + u < s1)
#pragma unroll
                for (int c = 0; c < D; ++c) acc[c] += to_fixed(keep[u][c], 187 - L - emax[c]);
        for (int j = s0 + kKeep; j < s1; ++j) {
            const uint32_t p = list[j];
            const long long i = (long long)(p / uint32_t(k));
            const float w = 2.f * g[p];
#pragma unroll
            for (int c = 0; c < D; ++c)
                acc[c] += to_fixed(__fmul_rn(w, __fsub_rn(rm[c], (c < dc ? q[i * d + c] : rm[c]))), 187 - L - emax[c]);
        }
#pragma unroll
        for (int c = 0; c < D; ++c) out[c] = float(double(acc[c]) * pow2(emax[c] + L - 187));
    }
#pragma unroll
    for (int c = 0; c < D; ++c)
        if (c < dc) grad_ref[(long long)m * d + c0 + c] = out[c];
}


// Exponent field of a double (0 for zeros and subnormals, 2047 for inf / NaN).
__device__ __forceinline__ int exp_field64(double t) { return int((__double_as_longlong(t) >> 52) & 0x7FF); }

// t * 2^sh rounded to the nearest integer (halves away from zero), in integer
// arithmetic: a finite double is mant * 2^(max(e, 1) - 1075) with its 53-bit
// significand mant.  The caller guarantees |t * 2^sh| < 2^124.
__device__ __forceinline__ __int128 to_fixed64(double t, int sh) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(t);
    const int e = int((b >> 52) & 0x7FFu);
    const long long mant = (long long)((b & 0xFFFFFFFFFFFFFull) | (e ? (1ull << 52) : 0ull));
    const int amt = (e ? e : 1) - 1075 + sh;
    __int128 v;
    if (amt >= 0)
        v = (__int128)mant << amt;
    else if (amt > -54)
        v = (__int128)((mant + (1ll << (-amt - 1))) >> (-amt));
    else
        v = 0;  // below half a unit
    return (b >> 63) ? -v : v;
}

// The float64 form of k_grad_ref_fixed: a term t has |t| < 2^(E - 1022) for
// the largest exponent field E of its coordinate (E >= 1); scaled by
// 2^(1146 - L - E), with s < 2^L terms, each scaled term is below 2^(124 - L)
// and the sum below 2^124: a 128-bit accumulator cannot overflow, and every
// term keeps 71 - L bits below the largest term's leading bit.
template <int D>
__global__ void k_grad_ref_fixed64(const double* __restrict__ q, const double* __restrict__ ref,
                                   const double* __restrict__ g, const uint32_t* __restrict__ list,
                                   const int* __restrict__ starts, int n, int k, int d, int c0,
                                   double* __restrict__ grad_ref) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= n) return;
    const int dc = min(D, d - c0);
    q += c0;
    double rm[D];
#pragma unroll
    for (int c = 0; c < D; ++c) rm[c] = c < dc ? ref[(long long)m * d + c0 + c] : 0.0;
    const int s0 = starts[m], s1 = starts[m + 1];
    int emax[D];
#pragma unroll
    for (int c = 0; c < D; ++c) emax[c] = 1;
    bool finite = true;
    for (int j = s0; j < s1; ++j) {
        const uint32_t p = list[j];
        const long long i = (long long)(p / uint32_t(k));
        const double w = 2.0 * g[p];
#pragma unroll
        for (int c = 0; c < D; ++c) {
            const int e = exp_field64(__dmul_rn(w, __dsub_rn(rm[c], (c < dc ? q[i * d + c] : rm[c]))));
            finite = finite && e != 2047;
            emax[c] = max(emax[c], e);
        }
    }
    double out[D];
    if (!finite) {
        // an infinite or NaN term: the sum is +-inf or NaN in any order
#pragma unroll
        for (int c = 0; c < D; ++c) out[c] = 0.0;
        for (int j = s0; j < s1; ++j) {
            const uint32_t p = list[j];
            const long long i = (long long)(p / uint32_t(k));
            const double w = 2.0 * g[p];
#pragma unroll
            for (int c = 0; c < D; ++c) out[c] += __dmul_rn(w, __dsub_rn(rm[c], (c < dc ? q[i * d + c] : rm[c])));
        }
    } else {
        const int L = 32 - __clz(s1 - s0);  // s1 - s0 < 2^L
        __int128 acc[D];
#pragma unroll
        for (int c = 0; c < D; ++c) acc[c] = 0;
        for (int j = s0; j < s1; ++j) {
            const uint32_t p = list[j];
            const long long i = (long long)(p / uint32_t(k));
            const double w = 2.0 * g[p];
#pragma unroll
            for (int c = 0; c < D; ++c)
                acc[c] += to_fixed64(__dmul_rn(w, __dsub_rn(rm[c], (c < dc ? q[i * d + c] : rm[c]))),
                                     1146 - L - emax[c]);
        }
#pragma unroll
        for (int c = 0; c < D; ++c) {
            const bool neg = acc[c] < 0;
            const unsigned __int128 mag = neg ? (unsigned __int128)(-acc[c]) : (unsigned __int128)acc[c];
            const double v = ldexp(double((unsigned long long)(mag >> 64)), 64) + double((unsigned long long)mag);
            out[c] = ldexp(neg ? -v : v, emax[c] + L - 1146);
        }
    }
#pragma unroll
    for (int c = 0; c < D; ++c)
        if (c < dc) grad_ref[(long long)m * d + c0 + c] = out[c];
}

// Workspace: each pair's rank within its key, the segment list, the n + 1
// counts / segment starts and the scan's scratch.
struct BwLayout {
    size_t rank = 0, list = 0, starts = 0, scan_ws = 0, total = 0;
};

BwLayout bw_layout(int64_t nq, int k, int64_t n) {
    BwLayout w;
    const int64_t np = std::max<int64_t>(1, nq * k);
    size_t o = 0;
    w.rank = o;
    o += align256(4 * size_t(np));
    w.list = o;
    o += align256(4 * size_t(np));
    w.starts = o;
    o += align256(4 * size_t(std::max<int64_t>(n, 1) + 1));
    w.scan_ws = o;
    o += scan_workspace_bytes(std::max<int64_t>(n, 1) + 1);
    w.total = o;
    return w;
}

template <typename T, int D>
int run_backward(const T* q, const T* ref, const int32_t* idx, const T* g, int nq, int n, int k, int d, T* grad_q,
                 T* grad_ref, char* ws, cudaStream_t s) {
    const int bs = D > 32 ? 64 : 256;
    if (grad_q && nq > 0) k_grad_q<T, D><<<(nq + bs - 1) / bs, bs, 0, s>>>(q, ref, idx, g, nq, n, k, d, grad_q);
    if (grad_ref) {
        const BwLayout w = bw_layout(nq, k, n);
        const long long np = (long long)nq * k;
        int* starts = reinterpret_cast<int*>(ws + w.starts);  // n + 1
        int* rank = reinterpret_cast<int*>(ws + w.rank);      // np
        uint32_t* list = reinterpret_cast<uint32_t*>(ws + w.list);
        cudaError_t e = cudaMemsetAsync(starts, 0, sizeof(int) * (size_t(n) + 1), s);
        if (e != cudaSuccess) return fail(TK_ECUDA, std::string("memset: ") + cudaGetErrorString(e));
        if (np > 0) k_count_keys<<<unsigned((np + 255) / 256), 256, 0, s>>>(idx, np, n, starts, rank);
        e = exclusive_scan(starts, int64_t(n) + 1, ws + w.scan_ws, s);
        if (e != cudaSuccess) return fail(TK_ECUDA, std::string("backward scan: ") + cudaGetErrorString(e));
        if (np > 0) k_fill_segments<<<unsigned((np + 255) / 256), 256, 0, s>>>(idx, np, n, starts, rank, list);
        // coordinates 8 per pass (one pass up to 8 dims; D = 1..3 keep their exact width)
        constexpr int DC = D <= 3 ? D : 8;
        for (int c0 = 0; c0 < d; c0 += DC) {
            if constexpr (sizeof(T) == 4)
                k_grad_ref_fixed<DC><<<(n + 255) / 256, 256, 0, s>>>(
                    reinterpret_cast<const float*>(q), reinterpret_cast<const float*>(ref),
                    reinterpret_cast<const float*>(g), list, starts, n, k, d, c0, reinterpret_cast<float*>(grad_ref));
            else
                k_grad_ref_fixed64<DC><<<(n + 255) / 256, 256, 0, s>>>(
                    reinterpret_cast<const double*>(q), reinterpret_cast<const double*>(ref),
                    reinterpret_cast<const double*>(g), list, starts, n, k, d, c0,
                    reinterpret_cast<double*>(grad_ref));
        }
    }
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(TK_ECUDA, std::string("backward launch: ") + cudaGetErrorString(e));
    return TK_OK;
}

}  // namespace
}  // namespace tk

using namespace tk;

extern "C" {

size_t tk_knn_backward_workspace_size(int64_t nq, int k, int64_t n) {
    if (nq < 0 || k < 1 || n < 1) return 0;
    return bw_layout(nq, k, n).total;
}

int tk_knn_backward(const void* q, const void* ref, const int32_t* idx, const void* grad_dists, int64_t nq,
                    int64_t n, int k, int dims, int dtype, void* grad_q, void* grad_ref, void* workspace,
                    size_t workspace_bytes, void* stream) {
    clear_error();
    if (nq < 0 || nq >= (int64_t(1) << 31) || n < 1 || n >= (int64_t(1) << 31) || k < 1)
        return fail(TK_EINVAL, "bad sizes");
    if (nq * int64_t(k) >= (int64_t(1) << 31)) return fail(TK_EINVAL, "nq * k must be < 2^31");
    if (dims < 1 || dims > 128) return fail(TK_EINVAL, "dims must be in [1, 128]");
    if (dtype != TK_F32 && dtype != TK_F64) return fail(TK_EINVAL, "dtype must be TK_F32 or TK_F64");
    if (nq == 0 && !grad_ref) return TK_OK;
    if (!ref || (nq > 0 && (!q || !idx || !grad_dists))) return fail(TK_EINVAL, "null input pointer");
    if (grad_ref && (!workspace || workspace_bytes < bw_layout(nq, k, n).total))
        return fail(TK_EWORKSPACE, "workspace too small");
    if (ws_misaligned(workspace)) return fail(TK_EINVAL, "workspace must be 256-byte aligned");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    char* ws = static_cast<char*>(workspace);
    const int nq32 = int(nq), n32 = int(n);
#define TK_BW(TT, DD)                                                                                        \
    return run_backward<TT, DD>(static_cast<const TT*>(q), static_cast<const TT*>(ref), idx,                 \
                                static_cast<const TT*>(grad_dists), nq32, n32, k, dims,                      \
                                static_cast<TT*>(grad_q), static_cast<TT*>(grad_ref), ws, s)
#define TK_BW_ALL(TT)                   \
    if (dims == 1) TK_BW(TT, 1);        \
    if (dims == 2) TK_BW(TT, 2);        \
    if (dims == 3) TK_BW(TT, 3);        \
    if (dims <= 8) TK_BW(TT, 8);        \
    if (dims <= 16) TK_BW(TT, 16);      \
    if (dims <= 32) TK_BW(TT, 32);      \
    if (dims <= 64) TK_BW(TT, 64);      \
    TK_BW(TT, 128);
    if (dtype == TK_F32) {
        TK_BW_ALL(float)
    } else {
        TK_BW_ALL(double)
    }
#undef TK_BW_ALL
#undef TK_BW
}

}  // extern "C"
