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
// without float atomics, in one of two forms:
//  * float32, d <= 8: segments are built by counting (integer atomics, whose
//    returned ranks then place each pair), so the order inside a segment is
//    arbitrary; the segment's sum is made order-independent instead.  One
//    pass finds the
//    largest exponent of its terms per coordinate, a second adds every FP32
//    term exactly as a 64-bit fixed-point integer scaled to that exponent,
//    and the total is rounded once -- the same bits whatever the order, and
//    closer to the exact sum than a sequential FP32 sum;
//  * otherwise: the (idx, pair) list is sorted by a stable radix sort, so
//    each reference point sees its pairs in ascending pair order and one
//    thread sums them in that fixed order.
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

// keys: neighbour index (n for invalid entries, which sort last).
__global__ void k_make_keys(const int32_t* __restrict__ idx, long long npairs, int n, uint32_t* __restrict__ keys) {
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npairs) return;
    const int m = idx[p];
    keys[p] = (m < 0 || m >= n) ? uint32_t(n) : uint32_t(m);
}

// Segment bounds of every key present in the sorted list: seg_start[m] and
// seg_end[m] (one past the last position).  Keys absent from the list keep
// seg_end[m] = 0 (zeroed beforehand) and are skipped.
__global__ void k_segment_bounds(const uint32_t* __restrict__ keys, long long npairs, int n,
                                 int* __restrict__ seg_start, int* __restrict__ seg_end) {
    const long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= npairs) return;
    const uint32_t key = keys[s];
    if (key >= uint32_t(n)) return;
    if (s == 0 || keys[s - 1] != key) seg_start[key] = int(s);
    if (s == npairs - 1 || keys[s + 1] != key) seg_end[key] = int(s + 1);
}

// One thread per reference point walks its segment in sorted (ascending
// pair) order.
template <typename T, int D>
__global__ void k_grad_ref(const T* __restrict__ q, const T* __restrict__ ref, const T* __restrict__ g,
                           const uint32_t* __restrict__ pairs, const int* __restrict__ seg_start,
                           const int* __restrict__ seg_end, int n, int k, int d, T* __restrict__ grad_ref) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= n) return;
    T rm[D], acc[D];
#pragma unroll
    for (int c = 0; c < D; ++c) {
        rm[c] = c < d ? ref[(long long)m * d + c] : T(0);
        acc[c] = T(0);
    }
    const int end = seg_end[m];
    const int beg = end > 0 ? seg_start[m] : 0;  // seg_start is only written for keys present
    for (int s = beg; s < end; ++s) {
        const uint32_t p = pairs[s];
        const long long i = (long long)(p / uint32_t(k));
        const T w = T(2) * g[p];
#pragma unroll
        for (int c = 0; c < D; ++c)
            if (c < d) acc[c] += w * (rm[c] - q[i * d + c]);
    }
#pragma unroll
    for (int c = 0; c < D; ++c)
        if (c < d) grad_ref[(long long)m * d + c] = acc[c];
}

// Segments by counting (float32, d <= 8): counts of every key (then their
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
// D: compile-time bound of the runtime dimension d (d <= D <= 8).
template <int D>
__global__ void k_grad_ref_fixed(const float* __restrict__ q, const float* __restrict__ ref, const float* __restrict__ g,
                                 const uint32_t* __restrict__ list, const int* __restrict__ starts, int n, int k, int d,
                                 float* __restrict__ grad_ref) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= n) return;
    float rm[D];
#pragma unroll
    for (int c = 0; c < D; ++c) rm[c] = c < d ? ref[(long long)m * d + c] : 0.f;
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
                keep[u][c] = __fmul_rn(w, __fsub_rn(rm[c], (c < d ? q[i * d + c] : rm[c])));
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
            const int e = exp_field(__fmul_rn(w, __fsub_rn(rm[c], (c < d ? q[i * d + c] : rm[c]))));
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
            for (int c = 0; c < D; ++c) out[c] += __fmul_rn(w, __fsub_rn(rm[c], (c < d ? q[i * d + c] : rm[c])));
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
                acc[c] += to_fixed(__fmul_rn(w, __fsub_rn(rm[c], (c < d ? q[i * d + c] : rm[c]))), 187 - L - emax[c]);
        }
#pragma unroll
        for (int c = 0; c < D; ++c) out[c] = float(double(acc[c]) * pow2(emax[c] + L - 187));
    }
#pragma unroll
    for (int c = 0; c < D; ++c)
        if (c < d) grad_ref[(long long)m * d + c] = out[c];
}

struct BwLayout {
    size_t keys = 0, sorted_keys = 0, sorted_vals = 0, seg_end = 0, seg_start = 0, sort_ws = 0, scan_ws = 0,
           total = 0;
};

BwLayout bw_layout(int64_t nq, int k, int64_t n) {
    BwLayout w;
    const int64_t np = std::max<int64_t>(1, nq * k);
    size_t o = 0;
    w.keys = o;
    o += align256(4 * size_t(np));
    w.sorted_keys = o;
    o += align256(4 * size_t(np));
    w.sorted_vals = o;
    o += align256(4 * size_t(np));
    w.seg_end = o;  // also the n + 1 counts / starts of the counting path
    o += align256(4 * size_t(std::max<int64_t>(n, 1) + 1));
    w.seg_start = o;
    o += align256(4 * size_t(std::max<int64_t>(n, 1)));
    w.sort_ws = o;
    o += sort_workspace_bytes(np);
    w.scan_ws = o;
    o += scan_workspace_bytes(std::max<int64_t>(n, 1) + 1);
    w.total = o;
    return w;
}

int key_bits_for(int64_t n) {
    int b = 1;
    while ((int64_t(1) << b) <= n) ++b;  // keys 0..n inclusive (n marks invalid)
    return b;
}

template <typename T, int D>
int run_backward(const T* q, const T* ref, const int32_t* idx, const T* g, int nq, int n, int k, int d, T* grad_q,
                 T* grad_ref, char* ws, cudaStream_t s) {
    const int bs = D > 32 ? 64 : 256;
    if (grad_q && nq > 0) k_grad_q<T, D><<<(nq + bs - 1) / bs, bs, 0, s>>>(q, ref, idx, g, nq, n, k, d, grad_q);
    if (grad_ref && sizeof(T) == 4 && D <= 8) {
        const BwLayout w = bw_layout(nq, k, n);
        const long long np = (long long)nq * k;
        int* starts = reinterpret_cast<int*>(ws + w.seg_end);  // n + 1
        int* rank = reinterpret_cast<int*>(ws + w.keys);        // np
        uint32_t* list = reinterpret_cast<uint32_t*>(ws + w.sorted_vals);
        cudaError_t e = cudaMemsetAsync(starts, 0, sizeof(int) * (size_t(n) + 1), s);
        if (e != cudaSuccess) return fail(TK_ECUDA, std::string("memset: ") + cudaGetErrorString(e));
        if (np > 0) k_count_keys<<<unsigned((np + 255) / 256), 256, 0, s>>>(idx, np, n, starts, rank);
        e = exclusive_scan(starts, int64_t(n) + 1, ws + w.scan_ws, s);
        if (e != cudaSuccess) return fail(TK_ECUDA, std::string("backward scan: ") + cudaGetErrorString(e));
        if (np > 0) k_fill_segments<<<unsigned((np + 255) / 256), 256, 0, s>>>(idx, np, n, starts, rank, list);
        if constexpr (sizeof(T) == 4 && D <= 8)
            k_grad_ref_fixed<D><<<(n + 255) / 256, 256, 0, s>>>(reinterpret_cast<const float*>(q),
                                                                 reinterpret_cast<const float*>(ref),
                                                                 reinterpret_cast<const float*>(g), list, starts, n, k,
                                                                 d, reinterpret_cast<float*>(grad_ref));
    } else if (grad_ref) {
        const BwLayout w = bw_layout(nq, k, n);
        const long long np = (long long)nq * k;
        uint32_t* keys = reinterpret_cast<uint32_t*>(ws + w.keys);
        uint32_t* sk = reinterpret_cast<uint32_t*>(ws + w.sorted_keys);
        uint32_t* sv = reinterpret_cast<uint32_t*>(ws + w.sorted_vals);
        int* seg_end = reinterpret_cast<int*>(ws + w.seg_end);
        int* seg_start = reinterpret_cast<int*>(ws + w.seg_start);
        if (np > 0) {
            k_make_keys<<<unsigned((np + 255) / 256), 256, 0, s>>>(idx, np, n, keys);
            cudaError_t e = sort_pairs(keys, nullptr, sk, sv, np, key_bits_for(n), ws + w.sort_ws,
                                       sort_workspace_bytes(np), s);
            if (e != cudaSuccess) return fail(TK_ECUDA, std::string("backward sort: ") + cudaGetErrorString(e));
        }
        cudaError_t e = cudaMemsetAsync(seg_end, 0, sizeof(int) * size_t(n), s);
        if (e != cudaSuccess) return fail(TK_ECUDA, std::string("memset: ") + cudaGetErrorString(e));
        if (np > 0) k_segment_bounds<<<unsigned((np + 255) / 256), 256, 0, s>>>(sk, np, n, seg_start, seg_end);
        k_grad_ref<T, D><<<(n + bs - 1) / bs, bs, 0, s>>>(q, ref, g, sv, seg_start, seg_end, n, k, d, grad_ref);
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
