// Tensor-core brute force: candidate search with q.r on tensor cores, exact
// FP32 re-rank, and a per-query certificate that the answer equals the exact
// search; uncertified queries are recomputed by the exact kernel.
//
//   score(q, r) = |r|^2 - 2 q.r   (ranks like |q - r|^2 for a fixed query)
//
// 1. k_tc_pack: operands for the tensor cores (TF32 rounded to nearest, or a
//    BF16 hi/lo split x = hi + lo) and |x|^2 in FP32.
// 2. k_tc_select: a block owns 128 queries and one slice of the references;
//    tiles of 128 references are multiplied with mma.sync (TF32 m16n8k8 or
//    BF16 m16n8k16 with three products hi*hi + hi*lo + lo*hi, FP32 accumulate),
//    the score tile goes through shared memory, and one thread per query keeps
//    the C = over-fetch best scores of its row (C >= 2k) plus the row
//    threshold tau (the C-th score; +inf while fewer than C were seen).
// 3. k_tc_rerank: one warp per query recomputes the exact distance of every
//    candidate with the reference arithmetic (sqdist order, no fused
//    multiply-add), keeps the k best (distance, index) keys, and certifies:
//    with D = k-th exact distance, E = bound on |score_tc - score_exact| for
//    any reference that could reach D, and tau = min over slices, the answer
//    is the exact one if |q|^2 + tau - E > D / (1 - m).  (A reference outside
//    every list has score_tc >= tau, hence |q - r|^2 >= |q|^2 + tau - E.)
// 4. Uncertified queries are listed and recomputed by the exact kernel.
#include <cuda_bf16.h>

#include <algorithm>
#include <string>

#include "brute.cuh"
#include "brute_tc.cuh"
#include "tk_internal.h"

namespace tk {
namespace {

constexpr int kRows = 128;   // queries per block
constexpr int kCols = 128;   // references per tile
constexpr int kThreads = 256;

size_t align256(size_t v) { return (v + 255) / 256 * 256; }

__device__ __forceinline__ uint32_t to_tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}

// Row-major packed operands: TF32 -> one uint32 per element, BF16 split ->
// hi and lo bf16 planes.  Rows are zero-padded to KP elements.
template <int MODE>
__global__ void k_tc_pack(const float* __restrict__ x, int rows, int d, int KP, uint32_t* __restrict__ tf,
                          __nv_bfloat16* __restrict__ hi, __nv_bfloat16* __restrict__ lo, float* __restrict__ norm) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows) return;
    float s = 0.f;
    for (int c = 0; c < KP; ++c) {
        const float v = c < d ? x[(long long)r * d + c] : 0.f;
        s = fmaf(v, v, s);
        if (MODE == TK_BRUTE_TF32) {
            tf[(long long)r * KP + c] = to_tf32(v);
        } else {
            const __nv_bfloat16 h = __float2bfloat16_rn(v);
            hi[(long long)r * KP + c] = h;
            lo[(long long)r * KP + c] = __float2bfloat16_rn(v - __bfloat162float(h));
        }
    }
    norm[r] = s;
}

struct TcArgs {
    const uint32_t* a_tf;  // queries (TF32)
    const uint32_t* b_tf;  // references (TF32)
    const __nv_bfloat16 *a_hi, *a_lo, *b_hi, *b_lo;
    const float* rnorm;    // |r|^2
    int n, nq, KP, C;
    int nsplit;
    float* cand_s;         // [nq, nsplit, C] scores
    int32_t* cand_i;       // [nq, nsplit, C] indices (-1 = empty)
    float* tau;            // [nq, nsplit]
};

__device__ __forceinline__ void mma_tf32(float (&c)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ void mma_bf16(float (&c)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// KP: padded depth (TF32: multiple of 8; BF16: multiple of 16).  C: over-fetch.
template <int MODE, int KP, int C>
__global__ void __launch_bounds__(kThreads, 1) k_tc_select(const TcArgs a) {
    constexpr int KW = (MODE == TK_BRUTE_TF32) ? KP : KP / 2;  // 32-bit words per packed row
    constexpr int BS = KW + 4;                                  // smem row stride (bank-conflict free)
    constexpr int SS = kCols + 4;                               // score tile row stride
    constexpr int PLANES = (MODE == TK_BRUTE_TF32) ? 1 : 2;
    extern __shared__ __align__(16) unsigned char smem[];
    uint32_t* Bs = reinterpret_cast<uint32_t*>(smem);                        // [PLANES][kCols][BS]
    float* rn = reinterpret_cast<float*>(Bs + PLANES * kCols * BS);          // [kCols]
    float* S = rn + kCols;                                                   // [kRows][SS]
    float* Ls = S + kRows * SS;                                              // [C][kRows]
    int32_t* Li = reinterpret_cast<int32_t*>(Ls + C * kRows);                // [C][kRows]

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int g = lane >> 2, t = lane & 3;
    const int q0 = blockIdx.x * kRows;
    const long long per = ((long long)a.n + a.nsplit - 1) / a.nsplit;
    const int r0 = int(min((long long)a.n, per * blockIdx.y));
    const int r1 = int(min((long long)a.n, per * (blockIdx.y + 1)));

    // A fragments of this warp's 16 rows, all k-steps, kept in registers
    constexpr int KSTEPS = (MODE == TK_BRUTE_TF32) ? KP / 8 : KP / 16;
    uint32_t af[PLANES][KSTEPS][4];
    {
        const int ra = q0 + warp * 16 + g, rb = ra + 8;
#pragma unroll
        for (int p = 0; p < PLANES; ++p) {
#pragma unroll
            for (int ks = 0; ks < KSTEPS; ++ks) {
                if (MODE == TK_BRUTE_TF32) {
                    const uint32_t* A = a.a_tf;
                    const int c0 = ks * 8 + t, c1 = c0 + 4;
                    af[p][ks][0] = ra < a.nq ? A[(long long)ra * KP + c0] : 0u;
                    af[p][ks][1] = rb < a.nq ? A[(long long)rb * KP + c0] : 0u;
                    af[p][ks][2] = ra < a.nq ? A[(long long)ra * KP + c1] : 0u;
                    af[p][ks][3] = rb < a.nq ? A[(long long)rb * KP + c1] : 0u;
                } else {
                    const uint32_t* A = reinterpret_cast<const uint32_t*>(p == 0 ? a.a_hi : a.a_lo);
                    const int w0 = ks * 8 + t, w1 = w0 + 4;  // 32-bit words: element pairs
                    af[p][ks][0] = ra < a.nq ? A[(long long)ra * KW + w0] : 0u;
                    af[p][ks][1] = rb < a.nq ? A[(long long)rb * KW + w0] : 0u;
                    af[p][ks][2] = ra < a.nq ? A[(long long)ra * KW + w1] : 0u;
                    af[p][ks][3] = rb < a.nq ? A[(long long)rb * KW + w1] : 0u;
                }
            }
        }
    }

    // per-row candidate lists (threads 0..127 own one row each)
    int cnt = 0;
    float tau = __int_as_float(0x7f800000);
    for (int c = 0; c < C && tid < kRows; ++c) {
        Ls[c * kRows + tid] = tau;
        Li[c * kRows + tid] = -1;
    }

    for (int c0 = r0; c0 < r1; c0 += kCols) {
        const int len = min(kCols, r1 - c0);
        __syncthreads();
        // reference tile -> shared memory (zero rows past the slice end)
        for (int e = tid; e < PLANES * kCols * KW; e += kThreads) {
            const int p = e / (kCols * KW);
            const int rem = e - p * kCols * KW;
            const int j = rem / KW, w = rem - j * KW;
            uint32_t v = 0u;
            if (j < len) {
                const uint32_t* B = MODE == TK_BRUTE_TF32 ? a.b_tf
                                                          : reinterpret_cast<const uint32_t*>(p == 0 ? a.b_hi : a.b_lo);
                v = B[(long long)(c0 + j) * KW + w];
            }
            Bs[(p * kCols + j) * BS + w] = v;
        }
        for (int j = tid; j < kCols; j += kThreads) rn[j] = j < len ? a.rnorm[c0 + j] : __int_as_float(0x7f800000);
        __syncthreads();
        // 16 x 128 scores per warp
        float acc[kCols / 8][4];
#pragma unroll
        for (int nt = 0; nt < kCols / 8; ++nt)
#pragma unroll
            for (int i = 0; i < 4; ++i) acc[nt][i] = 0.f;
#pragma unroll
        for (int ks = 0; ks < KSTEPS; ++ks) {
#pragma unroll
            for (int nt = 0; nt < kCols / 8; ++nt) {
                const int j = nt * 8 + g;
                if (MODE == TK_BRUTE_TF32) {
                    const uint32_t b0 = Bs[j * BS + ks * 8 + t];
                    const uint32_t b1 = Bs[j * BS + ks * 8 + t + 4];
                    mma_tf32(acc[nt], af[0][ks], b0, b1);
                } else {
                    const uint32_t bh0 = Bs[j * BS + ks * 8 + t];
                    const uint32_t bh1 = Bs[j * BS + ks * 8 + t + 4];
                    const uint32_t bl0 = Bs[(kCols + j) * BS + ks * 8 + t];
                    const uint32_t bl1 = Bs[(kCols + j) * BS + ks * 8 + t + 4];
                    mma_bf16(acc[nt], af[0][ks], bh0, bh1);  // hi * hi
                    mma_bf16(acc[nt], af[0][ks], bl0, bl1);  // hi * lo
                    mma_bf16(acc[nt], af[PLANES - 1][ks], bh0, bh1);  // lo * hi
                }
            }
        }
        // scores -> shared memory
        {
            const int ra = warp * 16 + g;
#pragma unroll
            for (int nt = 0; nt < kCols / 8; ++nt) {
                const int cc = nt * 8 + 2 * t;
                S[ra * SS + cc] = acc[nt][0];
                S[ra * SS + cc + 1] = acc[nt][1];
                S[(ra + 8) * SS + cc] = acc[nt][2];
                S[(ra + 8) * SS + cc + 1] = acc[nt][3];
            }
        }
        __syncthreads();
        // one thread per row: filter by tau, insert the rare survivors
        if (tid < kRows) {
            const float* row = S + tid * SS;
            for (int j = 0; j < len; ++j) {
                const float sc = fmaf(-2.f, row[j], rn[j]);
                if (sc < tau) {
                    int pos = cnt < C ? cnt : C - 1;
                    while (pos > 0 && Ls[(pos - 1) * kRows + tid] > sc) {
                        Ls[pos * kRows + tid] = Ls[(pos - 1) * kRows + tid];
                        Li[pos * kRows + tid] = Li[(pos - 1) * kRows + tid];
                        --pos;
                    }
                    Ls[pos * kRows + tid] = sc;
                    Li[pos * kRows + tid] = c0 + j;
                    cnt = min(cnt + 1, C);
                    if (cnt == C) tau = Ls[(C - 1) * kRows + tid];
                }
            }
        }
    }
    // write the lists
    if (tid < kRows) {
        const int q = q0 + tid;
        if (q < a.nq) {
            const long long base = ((long long)q * a.nsplit + blockIdx.y) * C;
            for (int c = 0; c < C; ++c) {
                a.cand_s[base + c] = Ls[c * kRows + tid];
                a.cand_i[base + c] = Li[c * kRows + tid];
            }
            a.tau[(long long)q * a.nsplit + blockIdx.y] = cnt == C ? tau : __int_as_float(0x7f800000);
        }
    }
}

template <int MODE, int KP, int C>
size_t select_smem_bytes() {
    constexpr int KW = (MODE == TK_BRUTE_TF32) ? KP : KP / 2;
    constexpr int PLANES = (MODE == TK_BRUTE_TF32) ? 1 : 2;
    return sizeof(uint32_t) * PLANES * kCols * (KW + 4) + sizeof(float) * kCols +
           sizeof(float) * kRows * (kCols + 4) + (sizeof(float) + sizeof(int32_t)) * size_t(C) * kRows;
}

struct RerankArgs {
    const float* ref;     // [n, d] float32 originals
    const float* q;       // [nq, d]
    int n, nq, d, k, C, nsplit;
    const float* cand_s;
    const int32_t* cand_i;
    const float* tau;
    double eps_dot;       // relative error bound of the tensor-core dot product
    float* out_d;
    int32_t* out_i;
    int* fail_count;
    int* fail_list;
};

// One warp per query: exact distances of the candidates, top-k, certificate.
template <int R>
__global__ void __launch_bounds__(256) k_tc_rerank(const RerankArgs a) {
    const int lane = threadIdx.x & 31;
    const int qi = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
    if (qi >= a.nq) return;
    TopK<float, 32, R> list;
    list.init(a.k, lane);
    Key<float> worst = Key<float>::sentinel();
    const float* qrow = a.q + (long long)qi * a.d;
    const int total = a.C * a.nsplit;
    const long long base = (long long)qi * total;
    for (int e0 = 0; e0 < total; e0 += 32) {
        const int e = e0 + lane;
        Key<float> mine = Key<float>::sentinel();
        const int r = e < total ? a.cand_i[base + e] : -1;
        if (r >= 0) {
            const float* rr = a.ref + (long long)r * a.d;
            float d0 = __fsub_rn(qrow[0], rr[0]);
            float acc = __fmul_rn(d0, d0);
            for (int c = 1; c < a.d; ++c) {
                const float dc = __fsub_rn(qrow[c], rr[c]);
                acc = __fadd_rn(acc, __fmul_rn(dc, dc));
            }
            mine = Key<float>::make(acc, uint32_t(r));
        }
        worst = offer<float, 32, R>(list, mine, worst, 0xFFFFFFFFu, lane, 0);
    }
    list.store(a.k, lane, a.out_d, a.out_i, qi);
    // certificate (lane 0)
    if (lane == 0) {
        double tau = INFINITY;
        for (int s = 0; s < a.nsplit; ++s) tau = fmin(tau, (double)a.tau[(long long)qi * a.nsplit + s]);
        bool ok = true;
        if (!isinf(tau)) {
            const double D = (double)worst.dist();
            double qq = 0.0;
            for (int c = 0; c < a.d; ++c) qq += (double)qrow[c] * (double)qrow[c];
            const double u = 1.0 / 16777216.0;                  // 2^-24
            const double m = (a.d + 4) * u;                      // rounding of the exact FP32 distance
            const double Dp = D / (1.0 - m);                     // real |q-r|^2 of any r with dist(r) <= D
            const double qn = sqrt(qq);
            const double rho = qn + sqrt(Dp);                    // |r| of any such r
            const double eps = 2.0 * a.eps_dot + (a.d + 4) * u;  // score error, relative
            const double E = 2.0 * eps * (qn * rho + rho * rho + fmax(Dp, qq));  // x2 safety
            ok = !isnan(D) && (qq + tau - E > Dp);
        }
        if (!ok) {
            const int slot = atomicAdd(a.fail_count, 1);
            a.fail_list[slot] = qi;
        }
    }
}

struct TcWs {
    size_t a_pack, b_pack, a_lo, b_lo, rnorm, qnorm, cand_s, cand_i, tau, fail_count, fail_list, brute, total;
    int KP, C, nsplit;
};

int tc_kp(int d, int mode) {
    const int step = mode == TK_BRUTE_TF32 ? 8 : 16;
    int kp = (d + step - 1) / step * step;
    if (kp <= 16) return kp <= 8 && mode == TK_BRUTE_TF32 ? 8 : 16;
    if (kp <= 32) return 32;
    if (kp <= 64) return 64;
    return 128;
}

int tc_over(int k) {
    int c = 16;
    while (c < 2 * k) c <<= 1;
    return c;
}

TcWs tc_layout(int64_t n, int64_t nq, int d, int k, int mode, int sms) {
    TcWs w;
    w.KP = tc_kp(d, mode);
    w.C = tc_over(k);
    const int qblocks = int((nq + kRows - 1) / kRows);
    int ns = std::max(1, (2 * sms + qblocks - 1) / std::max(1, qblocks));
    ns = int(std::min<int64_t>(ns, std::max<int64_t>(1, n / (4 * kCols))));
    w.nsplit = ns;
    const size_t es = mode == TK_BRUTE_TF32 ? 4 : 2;
    size_t o = 0;
    w.a_pack = o; o += align256(es * size_t(nq) * w.KP);
    w.b_pack = o; o += align256(es * size_t(n) * w.KP);
    w.a_lo = o; o += mode == TK_BRUTE_TF32 ? 0 : align256(es * size_t(nq) * w.KP);
    w.b_lo = o; o += mode == TK_BRUTE_TF32 ? 0 : align256(es * size_t(n) * w.KP);
    w.rnorm = o; o += align256(4 * size_t(n));
    w.qnorm = o; o += align256(4 * size_t(nq));
    w.cand_s = o; o += align256(4 * size_t(nq) * w.nsplit * w.C);
    w.cand_i = o; o += align256(4 * size_t(nq) * w.nsplit * w.C);
    w.tau = o; o += align256(4 * size_t(nq) * w.nsplit);
    w.fail_count = o; o += 256;
    w.fail_list = o; o += align256(4 * size_t(nq));
    w.brute = o; o += brute_fallback_workspace_bytes(n, nq, d, k);
    w.total = o;
    return w;
}

int sm_count_now() {
    int dev = 0, v = 1;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v < 1) v = 1;
    return v;
}

template <int MODE, int KP, int C>
int launch_select(const TcArgs& a, int qblocks, cudaStream_t s) {
    const size_t smem = select_smem_bytes<MODE, KP, C>();
    const void* fn = reinterpret_cast<const void*>(&k_tc_select<MODE, KP, C>);
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return fail(TK_ECUDA, std::string("tc select smem: ") + cudaGetErrorString(e));
    k_tc_select<MODE, KP, C><<<dim3(qblocks, a.nsplit), kThreads, smem, s>>>(a);
    return TK_OK;
}

template <int MODE, int KP>
int dispatch_c(const TcArgs& a, int qblocks, cudaStream_t s) {
    switch (a.C) {
        case 16: return launch_select<MODE, KP, 16>(a, qblocks, s);
        case 32: return launch_select<MODE, KP, 32>(a, qblocks, s);
        case 64: return launch_select<MODE, KP, 64>(a, qblocks, s);
        case 128: return launch_select<MODE, KP, 128>(a, qblocks, s);
        default: return fail(TK_EUNSUPPORTED, "tensor-core modes support k <= 64");
    }
}

template <int MODE>
int dispatch_kp(const TcArgs& a, int qblocks, cudaStream_t s) {
    switch (a.KP) {
        case 8:
            if constexpr (MODE == TK_BRUTE_TF32) return dispatch_c<MODE, 8>(a, qblocks, s);
            break;
        case 16: return dispatch_c<MODE, 16>(a, qblocks, s);
        case 32: return dispatch_c<MODE, 32>(a, qblocks, s);
        case 64: return dispatch_c<MODE, 64>(a, qblocks, s);
        default: break;
    }
    return fail(TK_EUNSUPPORTED, "tensor-core modes support d <= 64");
}

}  // namespace

size_t brute_tc_workspace_bytes(int64_t n, int64_t nq, int d, int k, int mode) {
    return tc_layout(n, std::max<int64_t>(nq, 1), d, k, mode, sm_count_now()).total;
}

int run_brute_tc(const float* ref, int64_t n, const float* q, int64_t nq, int d, int k, int mode, float* dists,
                 int32_t* idx, void* ws, size_t ws_bytes, cudaStream_t s) {
    if (k > 64) return fail(TK_EUNSUPPORTED, "tensor-core modes support k <= 64 (use TK_BRUTE_EXACT)");
    if (d > 64) return fail(TK_EUNSUPPORTED, "tensor-core modes support d <= 64 (use TK_BRUTE_EXACT)");
    const TcWs w = tc_layout(n, nq, d, k, mode, sm_count_now());
    if (!ws || ws_bytes < w.total) return fail(TK_EWORKSPACE, "workspace too small");
    char* p = static_cast<char*>(ws);
    const int n32 = int(n), nq32 = int(nq);
    // 1. pack
    if (mode == TK_BRUTE_TF32) {
        k_tc_pack<TK_BRUTE_TF32><<<(nq32 + 255) / 256, 256, 0, s>>>(q, nq32, d, w.KP, reinterpret_cast<uint32_t*>(p + w.a_pack),
                                                                  nullptr, nullptr, reinterpret_cast<float*>(p + w.qnorm));
        k_tc_pack<TK_BRUTE_TF32><<<(n32 + 255) / 256, 256, 0, s>>>(ref, n32, d, w.KP, reinterpret_cast<uint32_t*>(p + w.b_pack),
                                                                 nullptr, nullptr, reinterpret_cast<float*>(p + w.rnorm));
    } else {
        k_tc_pack<TK_BRUTE_BF16_SPLIT><<<(nq32 + 255) / 256, 256, 0, s>>>(
            q, nq32, d, w.KP, nullptr, reinterpret_cast<__nv_bfloat16*>(p + w.a_pack),
            reinterpret_cast<__nv_bfloat16*>(p + w.a_lo), reinterpret_cast<float*>(p + w.qnorm));
        k_tc_pack<TK_BRUTE_BF16_SPLIT><<<(n32 + 255) / 256, 256, 0, s>>>(
            ref, n32, d, w.KP, nullptr, reinterpret_cast<__nv_bfloat16*>(p + w.b_pack),
            reinterpret_cast<__nv_bfloat16*>(p + w.b_lo), reinterpret_cast<float*>(p + w.rnorm));
    }
    // 2. candidates
    TcArgs a{};
    a.a_tf = reinterpret_cast<const uint32_t*>(p + w.a_pack);
    a.b_tf = reinterpret_cast<const uint32_t*>(p + w.b_pack);
    a.a_hi = reinterpret_cast<const __nv_bfloat16*>(p + w.a_pack);
    a.b_hi = reinterpret_cast<const __nv_bfloat16*>(p + w.b_pack);
    a.a_lo = reinterpret_cast<const __nv_bfloat16*>(p + w.a_lo);
    a.b_lo = reinterpret_cast<const __nv_bfloat16*>(p + w.b_lo);
    a.rnorm = reinterpret_cast<const float*>(p + w.rnorm);
    a.n = n32;
    a.nq = nq32;
    a.KP = w.KP;
    a.C = w.C;
    a.nsplit = w.nsplit;
    a.cand_s = reinterpret_cast<float*>(p + w.cand_s);
    a.cand_i = reinterpret_cast<int32_t*>(p + w.cand_i);
    a.tau = reinterpret_cast<float*>(p + w.tau);
    const int qblocks = (nq32 + kRows - 1) / kRows;
    int rc = mode == TK_BRUTE_TF32 ? dispatch_kp<TK_BRUTE_TF32>(a, qblocks, s)
                                   : dispatch_kp<TK_BRUTE_BF16_SPLIT>(a, qblocks, s);
    if (rc != TK_OK) return rc;
    // 3. exact re-rank + certificate
    cudaError_t e = cudaMemsetAsync(p + w.fail_count, 0, sizeof(int), s);
    if (e != cudaSuccess) return fail(TK_ECUDA, std::string("memset: ") + cudaGetErrorString(e));
    RerankArgs ra{};
    ra.ref = ref;
    ra.q = q;
    ra.n = n32;
    ra.nq = nq32;
    ra.d = d;
    ra.k = k;
    ra.C = w.C;
    ra.nsplit = w.nsplit;
    ra.cand_s = a.cand_s;
    ra.cand_i = a.cand_i;
    ra.tau = a.tau;
    const double u = 1.0 / 16777216.0;
    ra.eps_dot = mode == TK_BRUTE_TF32 ? (1.0 / 1024.0 + 1.0 / 4194304.0 + d * 2.0 * u)
                                       : (3.1 / 65536.0 + 3.0 * d * 2.0 * u);
    ra.out_d = dists;
    ra.out_i = idx;
    ra.fail_count = reinterpret_cast<int*>(p + w.fail_count);
    ra.fail_list = reinterpret_cast<int*>(p + w.fail_list);
    const int rb = (nq32 + 7) / 8;
    if (k <= 32) k_tc_rerank<1><<<rb, 256, 0, s>>>(ra);
    else k_tc_rerank<2><<<rb, 256, 0, s>>>(ra);
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(TK_ECUDA, std::string("tc launch: ") + cudaGetErrorString(e));
    // 4. exact recomputation of the uncertified queries
    return brute_fallback(ref, n, q, nq, d, k, dists, idx, ra.fail_list, ra.fail_count, p + w.brute,
                          brute_fallback_workspace_bytes(n, nq, d, k), s);
}

}  // namespace tk
