// Tensor-core brute force: kernels and launch templates, shared by the units
// that instantiate them (brute_tc5_tf32.cu, brute_tc5_tf32_deep.cu,
// brute_tc5_bf16.cu: the tcgen05 candidate search per operand mode and row
// depth; brute_tc_mma.cu: the mma.sync search for deeper rows or larger k;
// brute_tc.cu: packing, re-rank and the host side).
// The algorithm is described at the top of brute_tc.cu.
#pragma once

#include <cuda_bf16.h>

#include <string>

#include "brute.cuh"
#include "tc_sm100.cuh"
#include "tk_internal.h"

namespace tk {
namespace tcx {


constexpr int kRows = 128;   // queries per block
constexpr int kCols = 128;   // references per tile
constexpr int kThreads = 256;

inline size_t align256(size_t v) { return (v + 255) / 256 * 256; }

// The certificate below reasons about finite scores: a slice whose list never
// filled (tau = +inf) holds every reference of the slice.  NaN scores (from
// non-finite coordinates) enter no list, and overflowing ones break the error
// bound, so a query is certified only when |q|^2 < 2^125 and every reference
// has |r|^2 < 2^125 (the pack kernel flags any other reference in `err`,
// which certifies nothing).  Then every partial sum of a score is below
// |r|^2 + 2|q||r| <= 2 (|q|^2 + |r|^2) < 2^127: finite.  Uncertified queries
// are answered by the exact kernel.
constexpr float kTcNormLimit = 0x1p125f;
// Bits of the candidate search's error word (any bit: certify nothing, so
// the exact kernel recomputes every query and the answer stays exact).
constexpr int kTcErrTimeout = 1;  // a bounded wait of the tcgen05 kernel ran out
constexpr int kTcErrRange = 2;    // an input outside the certificate's range (kTcNormLimit)

__device__ __forceinline__ uint32_t to_tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}

// Row-major packed operands: TF32 -> one uint32 per element, BF16 split ->
// hi and lo bf16 planes.  Rows are zero-padded to KP elements.
template <int MODE>
__global__ void k_tc_pack(const float* __restrict__ x, int rows, int d, int KP, uint32_t* __restrict__ tf,
                          __nv_bfloat16* __restrict__ hi, __nv_bfloat16* __restrict__ lo, float* __restrict__ norm,
                          int* __restrict__ err) {
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
    if (err && !(s < kTcNormLimit)) atomicOr(err, kTcErrRange);  // see kTcNormLimit
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
    extern __shared__ __align__(1024) unsigned char smem[];  // one declaration per unit: k_tc5_select's alignment
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

// ---------------------------------------------------------------------------
// tcgen05 path (d <= 39 for TF32, d <= 47 for BF16 split; k <= 32).
//
// The score is produced by the MMA itself by augmenting K with one column:
//   A = [-2 q, 1, 0...],  B = [r, |r|^2, 0...]  =>  A.B = |r|^2 - 2 q.r.
// Operands are packed in global memory in the tensor core's canonical
// no-swizzle K-major layout (8-row x 16-byte core matrices; core matrices
// adjacent along K 128 bytes apart, 8-row groups 8*KB bytes apart), one
// contiguous block per 128 query rows / 256 reference rows, so each tile is
// a single bulk copy.  Reference padding rows carry a huge |r|^2 and never
// become candidates.
constexpr int kT5Rows = 128;   // M (queries per block)
constexpr int kT5Cols = 256;   // N (references per tile)
constexpr int kT5EpiWarps = 16; // 4 per 32-lane quarter of the accumulator when reading tensor memory
constexpr int kT5Chunk = 64;    // accumulator columns per phase (16 per column-group warp)
constexpr int kT5Buf = 48;      // hit buffer per row and tile parity (a redo phase: 32 columns)
constexpr int kT5BufStride = kT5Buf + 1;  // row stride of the hit buffer (keys), spreads rows over banks
// Row stride (words) of the sample's group minima (2C <= 128 per row); 132 = 4
// mod 32 puts the 32 lanes of a bisection read (8 rows x 4 interleaved lanes)
// on 32 different banks.
constexpr int kT5MinStride = 132;
constexpr int kT5Threads = 32 * (kT5EpiWarps + 1);
constexpr float kT5PadNorm = 1e30f;
constexpr uint32_t kT5MaxTries = 1u << 22;  // bounded mbarrier polls (default; Tc5Args::max_tries)

__device__ __forceinline__ uint32_t core_offset(int row, int kb, int KB) {
    return uint32_t((row >> 3) * (8 * KB) + (kb >> 4) * 128 + (row & 7) * 16 + (kb & 15));
}

// rows: logical rows; padded to a multiple of tile_rows.  is_query selects
// [-2q, 1] (queries) or [r, |r|^2] (references).
template <int MODE>
__global__ void k_tc5_pack(const float* __restrict__ x, int rows, int rows_pad, int d, int KP, int tile_rows,
                           int is_query, unsigned char* __restrict__ hi, unsigned char* __restrict__ lo,
                           int* __restrict__ err) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows_pad) return;
    constexpr int ESZ = MODE == TK_BRUTE_TF32 ? 4 : 2;
    const int KB = KP * ESZ;
    const bool real = r < rows;
    float nrm = 0.f;
    if (real && !is_query) {
        for (int c = 0; c < d; ++c) nrm = fmaf(x[(long long)r * d + c], x[(long long)r * d + c], nrm);
        if (!(nrm < kTcNormLimit)) atomicOr(err, kTcErrRange);  // see kTcNormLimit
    }
    const long long tile_base = (long long)(r / tile_rows) * tile_rows * KB;
    const int rr = r % tile_rows;
    for (int c = 0; c < KP; ++c) {
        float v = 0.f;
        if (c < d) {
            v = real ? x[(long long)r * d + c] : 0.f;
            if (is_query) v = -2.f * v;
        } else if (c == d) {
            v = is_query ? (real ? 1.f : 0.f) : (real ? nrm : kT5PadNorm);
        }
        const long long off = tile_base + core_offset(rr, c * ESZ, KB);
        if (MODE == TK_BRUTE_TF32) {
            *reinterpret_cast<uint32_t*>(hi + off) = to_tf32(v);
        } else {
            const __nv_bfloat16 h = __float2bfloat16_rn(v);
            *reinterpret_cast<__nv_bfloat16*>(hi + off) = h;
            *reinterpret_cast<__nv_bfloat16*>(lo + off) = __float2bfloat16_rn(v - __bfloat162float(h));
        }
    }
}

struct Tc5Args {
    const unsigned char* a_hi;  // packed queries, blocks of 128 rows
    const unsigned char* a_lo;
    const unsigned char* b_hi;  // packed references, tiles of 256 rows
    const unsigned char* b_lo;
    int n, nq, nsplit;
    float* cand_s;              // [nq, nsplit, 2 * CH]
    int32_t* cand_i;
    float* tau;                 // [nq, nsplit]
    int* err;                   // kTcErrTimeout set when a bounded wait ran out
    uint32_t max_tries;         // polls of each mbarrier wait before giving up
};

// Score keys: order-preserving uint32 image of the float score (negative
// scores included) in the high word, reference index in the low word.
__device__ __forceinline__ unsigned long long score_key(float sc, uint32_t idx) {
    uint32_t u = __float_as_uint(sc);
    u = (u & 0x80000000u) ? ~u : (u | 0x80000000u);
    return (static_cast<unsigned long long>(u) << 32) | idx;
}
__device__ __forceinline__ float key_score(unsigned long long key) {
    const uint32_t u = uint32_t(key >> 32);
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u);
}
constexpr unsigned long long kScoreSentinel = (0xFF800000ull << 32) | 0xFFFFFFFFull;  // score +inf
__device__ __forceinline__ uint32_t score_bits(float sc) {
    const uint32_t u = __float_as_uint(sc);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float bits_score(uint32_t u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u);
}

// A row's over-fetch list of up to 32 * R keys spread over a warp (slot s on
// lane s % 32, register s / 32; the first 32 R - C slots are padding below
// every key), as TopK in tk_device.cuh.
// The over-fetch list of one query row held by a group of 4 lanes: ascending
// score keys, lane g of the group holding ranks [RS g, RS g + RS) in its
// registers (RS = C / 4).  An insertion shifts every lane's run in registers
// and moves one key across each lane boundary with a single shuffle, so the 8
// groups of a warp insert into their 8 rows side by side.
template <int RS>
struct GroupList {
    unsigned long long slot[RS];
    __device__ __forceinline__ void init() {
#pragma unroll
        for (int i = 0; i < RS; ++i) slot[i] = kScoreSentinel;
    }
    // Insert c (the sentinel leaves the list as it is); every lane of the
    // warp calls it.  gl: this lane's place in its group.
    __device__ __forceinline__ void insert(unsigned long long c, int gl) {
        const unsigned long long before = __shfl_up_sync(0xFFFFFFFFu, slot[RS - 1], 1, 4);
#pragma unroll
        for (int i = RS - 1; i >= 0; --i) {  // top down: slot[i - 1] is still the old value
            const unsigned long long old = slot[i];
            const bool has_prev = i > 0 || gl > 0;
            const unsigned long long prev = i > 0 ? slot[i - 1] : before;
            slot[i] = old <= c ? old : ((!has_prev || prev <= c) ? c : prev);
        }
    }
    __device__ __forceinline__ unsigned long long worst() const {
        return __shfl_sync(0xFFFFFFFFu, slot[RS - 1], 3, 4);
    }
};


template <int MODE, int KP, int CH>
struct Tc5Shape {
    static constexpr int ESZ = MODE == TK_BRUTE_TF32 ? 4 : 2;
    static constexpr int KB = KP * ESZ;
    static constexpr int PL = MODE == TK_BRUTE_TF32 ? 1 : 2;
    static constexpr uint32_t A_BYTES = uint32_t(kT5Rows) * KB;
    static constexpr uint32_t B_BYTES = uint32_t(kT5Cols) * KB;
    static constexpr int KSTEPS = KB / 32;
    static constexpr size_t SMEM = size_t(PL) * A_BYTES + 2 * size_t(PL) * B_BYTES +
                                   2 * size_t(kT5Rows) * kT5BufStride * 8 +  // hit buffers by tile parity
                                   size_t(kT5Rows) * sizeof(float) +         // row thresholds
                                   2 * size_t(kT5Rows) * sizeof(int) +       // hit counts by tile parity
                                   40 * sizeof(int);                         // overflow / abort flags: block, per quarter
    static_assert(SMEM <= 232448, "shared memory of the select kernel");
    static_assert(size_t(kT5Rows) * kT5MinStride * 4 <= 2 * size_t(kT5Rows) * kT5BufStride * 8 && 4 * CH <= 128,
                  "the sample's minima fit the hit buffers");
};

// Candidate search of one block: 128 query rows against one slice of the
// references, C = 2 CH candidates per row.
//
// Sampled first threshold.  Before its slice a block runs PS = C / 2 full
// tiles spread over the slice (a sample); each epilogue thread takes the
// minimum of its 64 scores of a sample tile (a group of 64 references of its
// row), and the row's four list lanes find T0 = the C-th smallest of the
// row's 2C group minima (bisection on their order-preserving images).  At
// least C distinct references of the slice score <= T0 (the minima of C
// groups), so the slice's C-th best score is <= T0 and T0 is a valid
// threshold from the first tile on: the lists start empty, but only
// references scoring <= T0 enter them, instead of every score of the first
// tiles.  (The C-th of 2C minima of 64 scores sits near the 1% quantile of a
// row's scores; C / 4 sample tiles with minima of 32 scores, near 2%, were
// 2-5% slower, and the maximum of C minima, near 7%, slower still.)  The
// sample tiles are scanned again as part of the slice; slices of fewer than
// 2 PS full tiles skip the sample.
template <int MODE, int KP, int CH>
__global__ void __launch_bounds__(kT5Threads, 1) k_tc5_select(const Tc5Args a) {
    using Sh = Tc5Shape<MODE, KP, CH>;
    constexpr int PL = Sh::PL, KB = Sh::KB, KSTEPS = Sh::KSTEPS;
    constexpr uint32_t A_BYTES = Sh::A_BYTES, B_BYTES = Sh::B_BYTES;
    constexpr uint32_t LBO = 128, SBO = 8 * KB;
    constexpr int NPROD = MODE == TK_BRUTE_TF32 ? 1 : 3;
    constexpr uint32_t IDESC = sm100::instr_desc(MODE == TK_BRUTE_TF32 ? 2u : 1u, kT5Rows, kT5Cols);

    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char* sA = smem;                       // [PL][A_BYTES]
    unsigned char* sB = smem + PL * A_BYTES;        // [2 stages][PL][B_BYTES]
    unsigned long long* sBuf = reinterpret_cast<unsigned long long*>(sB + 2 * PL * B_BYTES);  // [2][kT5Rows][stride]
    float* sThr = reinterpret_cast<float*>(sBuf + 2 * kT5Rows * kT5BufStride);  // [kT5Rows] list threshold per row
    int* sCnt = reinterpret_cast<int*>(sThr + kT5Rows);                        // [2][kT5Rows] buffered hits per row
    // [0..7] the sample steps' flags (block-wide), then per quarter [8 + 8q ..]:
    // [0..3] overflow, [4..7] abort, by step mod 4
    int* sFlag = sCnt + 2 * kT5Rows;
    __shared__ __align__(8) uint64_t full_a, full_b[2], mma_done[2], epi_done[2];
    __shared__ uint32_t tmem_base_sh;
    __shared__ int abort_sh;
    constexpr int C = 2 * CH;                 // over-fetch per row and slice
    constexpr int RS = C / 4;                 // list keys per lane (4 lanes per row)
    constexpr int ROWS_PER_WARP = kT5Rows / kT5EpiWarps;
    static_assert(ROWS_PER_WARP * 4 == 32, "one row per group of 4 lanes");
    constexpr int NEPI = 32 * kT5EpiWarps;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const long long per0 = ((long long)a.n + a.nsplit - 1) / a.nsplit;
    const long long per = (per0 + kT5Cols - 1) / kT5Cols * kT5Cols;  // slices start on tile boundaries
    const int r0 = int(min((long long)a.n, per * blockIdx.y));
    const int r1 = int(min((long long)a.n, per * (blockIdx.y + 1)));
    const int ntiles = (r1 - r0 + kT5Cols - 1) / kT5Cols;
    const int tile0 = r0 / kT5Cols;
    constexpr int PS = (C + 1) / 2;             // sample tiles (4 group minima of a row per tile)
    const int nfull = (r1 - r0) / kT5Cols;
    const int npre = nfull >= 2 * PS ? PS : 0;  // sample tiles run before the slice
    const int pstride = npre ? nfull / PS : 1;
    const int nseq = npre + ntiles;             // tiles through the pipeline
    // slice tile of pipeline step t: the samples s * pstride, then 0 .. ntiles - 1
    auto tile_of = [&](int t) { return t < npre ? t * pstride : t - npre; };

    if (tid == 0) {
        sm100::mbar_init(&full_a, 1);
        sm100::mbar_init(&full_b[0], 1);
        sm100::mbar_init(&full_b[1], 1);
        sm100::mbar_init(&mma_done[0], 1);
        sm100::mbar_init(&mma_done[1], 1);
        sm100::mbar_init(&epi_done[0], kT5EpiWarps);
        sm100::mbar_init(&epi_done[1], kT5EpiWarps);
        abort_sh = 0;
        sm100::mbar_fence_init();
    }
    if (warp == kT5EpiWarps) sm100::tmem_alloc(&tmem_base_sh, 512);
    sm100::tc_fence_before();
    __syncthreads();
    sm100::tc_fence_after();
    const uint32_t tmem = tmem_base_sh;

    if (warp == kT5EpiWarps) {
        // ------------------------------------------------ producer / MMA issuer
        if (lane == 0 && nseq > 0) {
            bool ok = true;
            // what this thread started and has not yet seen complete, per
            // stage: the tile last copied in / waited for, last committed /
            // waited for (drained if it gives up, see below)
            bool a_pending = true;
            int b_issued[2] = {-1, -1}, b_waited[2] = {-1, -1};
            int m_issued[2] = {-1, -1}, m_waited[2] = {-1, -1};
            sm100::mbar_arrive_expect_tx(&full_a, PL * A_BYTES);
            sm100::bulk_g2s(sA, a.a_hi + (size_t)blockIdx.x * A_BYTES, A_BYTES, &full_a);
            if (PL == 2) sm100::bulk_g2s(sA + A_BYTES, a.a_lo + (size_t)blockIdx.x * A_BYTES, A_BYTES, &full_a);
            for (int t = 0; t < 2 && t < nseq; ++t) {
                const size_t tb = (size_t)(tile0 + tile_of(t)) * B_BYTES;
                sm100::mbar_arrive_expect_tx(&full_b[t], PL * B_BYTES);
                sm100::bulk_g2s(sB + (t * PL) * B_BYTES, a.b_hi + tb, B_BYTES, &full_b[t]);
                if (PL == 2) sm100::bulk_g2s(sB + (t * PL + 1) * B_BYTES, a.b_lo + tb, B_BYTES, &full_b[t]);
                b_issued[t] = t;
            }
            for (int t = 0; t < nseq; ++t) {
                const int st = t & 1;
                const uint32_t ph = (t >> 1) & 1;  // stage st serves tiles st, st + 2, ...: phase t / 2
                ok = sm100::mbar_wait(&full_b[st], ph, a.max_tries);
                if (!ok) break;
                b_waited[st] = t;
                if (t == 0) {
                    ok = sm100::mbar_wait(&full_a, 0, a.max_tries);
                    if (!ok) break;
                    a_pending = false;
                }
                if (t >= 2) {
                    ok = sm100::mbar_wait(&epi_done[st], ((t - 2) >> 1) & 1, a.max_tries);
                    if (!ok) break;
                }
                sm100::tc_fence_after();
                const uint32_t dtm = tmem + uint32_t(st * kT5Cols);
                const uint32_t a0 = sm100::smem_u32(sA);
                const uint32_t b0 = sm100::smem_u32(sB + (st * PL) * B_BYTES);
#pragma unroll
                for (int ks = 0; ks < KSTEPS; ++ks) {
#pragma unroll
                    for (int pr = 0; pr < NPROD; ++pr) {
                        const uint32_t pa = pr == 2 ? A_BYTES : 0u;  // lo(A) for lo*hi
                        const uint32_t pb = pr == 1 ? B_BYTES : 0u;  // lo(B) for hi*lo
                        const uint64_t ad = sm100::smem_desc(a0 + pa + uint32_t(ks) * 256u, LBO, SBO);
                        const uint64_t bd = sm100::smem_desc(b0 + pb + uint32_t(ks) * 256u, LBO, SBO);
                        const uint32_t acc = (ks | pr) != 0 ? 1u : 0u;
                        if (MODE == TK_BRUTE_TF32) sm100::mma_tf32(dtm, ad, bd, IDESC, acc);
                        else sm100::mma_bf16(dtm, ad, bd, IDESC, acc);
                    }
                }
                sm100::mma_commit(&mma_done[st]);
                m_issued[st] = t;
                if (t + 2 < nseq) {
                    ok = sm100::mbar_wait(&mma_done[st], ph, a.max_tries);  // stage st no longer read
                    if (!ok) break;
                    m_waited[st] = t;
                    const size_t tb = (size_t)(tile0 + tile_of(t + 2)) * B_BYTES;
                    sm100::mbar_arrive_expect_tx(&full_b[st], PL * B_BYTES);
                    sm100::bulk_g2s(sB + (st * PL) * B_BYTES, a.b_hi + tb, B_BYTES, &full_b[st]);
                    if (PL == 2) sm100::bulk_g2s(sB + (st * PL + 1) * B_BYTES, a.b_lo + tb, B_BYTES, &full_b[st]);
                    b_issued[st] = t + 2;
                }
            }
            if (!ok) {
                // A wait ran out: flag it (the re-rank then certifies nothing
                // and the exact kernel answers every query), then let this
                // thread's own copies and matrix products still in flight
                // land -- each wait bounded by the default poll count --
                // before the block frees its tensor memory and exits.
                atomicExch(&abort_sh, 1);
                atomicOr(a.err, kTcErrTimeout);
                if (a_pending) sm100::mbar_wait(&full_a, 0, kT5MaxTries);
                for (int s2 = 0; s2 < 2; ++s2) {
                    if (b_issued[s2] > b_waited[s2])
                        sm100::mbar_wait(&full_b[s2], (b_issued[s2] >> 1) & 1, kT5MaxTries);
                    if (m_issued[s2] > m_waited[s2])
                        sm100::mbar_wait(&mma_done[s2], (m_issued[s2] >> 1) & 1, kT5MaxTries);
                }
            }
        }
        __syncwarp();
    } else {
        // ------------------------------------------------------- epilogue warps
        // Thread (warp w, lane l) reads accumulator lane 32 (w & 3) + l, i.e.
        // query row `myrow`, and the 16-column group w >> 2 of every 64-column
        // phase.  Each score is compared with the row's threshold (the worst
        // key of its over-fetch list, possibly stale but never too small);
        // the rare hits are appended to the row's buffer of the tile's parity
        // in shared memory.  One barrier per tile and accumulator quarter:
        // after it the tile's accumulator is released to the MMA issuer, and
        // warp w merges the buffers of its quarter's rows 32 (w & 3) +
        // 8 (w >> 2) .. + 7 into their lists (kept in its registers, one row
        // per group of 4 lanes) while other warps may already be filtering
        // the next tile into the other parity's buffers.  A row can
        // take at most kT5Buf hits per tile on this path; a tile that
        // overflows a buffer (the first tiles of a slice, while the lists
        // fill) is done again from tensor memory in eight steps of 32
        // columns, merging after each, which cannot overflow.
        const int quarter = warp & 3, cgroup = warp >> 2;
        const int myrow = 32 * quarter + lane;
        // the row this lane's group keeps: the 4 warps of a quarter keep its 32 rows
        const int grow = 32 * quarter + ROWS_PER_WARP * cgroup + (lane >> 2);
        int* qFlag = sFlag + 8 + 8 * quarter;
        const int gl = lane & 3;
        GroupList<RS> glist;
        glist.init();
        unsigned long long gworst = kScoreSentinel;
        float t0g = __int_as_float(0x7f800000);   // T0 of row grow
        // the sample's group minima (images), 2C per row, in the hit buffers' space
        uint32_t* sMin = reinterpret_cast<uint32_t*>(sBuf);
        const uint32_t trow = tmem + (uint32_t(32 * quarter) << 16);
        constexpr int NPHASE = kT5Cols / kT5Chunk;
        if (tid < kT5Rows) {
            sThr[tid] = __int_as_float(0x7f800000);
            sCnt[tid] = 0;
            sCnt[kT5Rows + tid] = 0;
        }
        if (tid < 40) sFlag[tid] = 0;
        // The sample steps synchronise all epilogue warps (their minima share
        // the hit buffers' space across quarters); from the first tile of the
        // slice on, each quarter (its 4 warps filter and keep the same 32
        // rows) synchronises on its own named barrier, and the quarters meet
        // only through the accumulator stages (epi_done).
        auto bar_all = [&]() { asm volatile("bar.sync 1, %0;" ::"r"(NEPI) : "memory"); };
        auto bar_quarter = [&]() { asm volatile("bar.sync %0, 128;" ::"r"(2 + quarter) : "memory"); };
        bar_all();
        // compare 16 scores of columns col0 .. col0+15 with thr, append the hits
        // to buffer parity `par` (`edge`: the columns may run past the slice's
        // end, in its last tile)
        auto append16 = [&](const float (&v)[16], int col0, float thr, float pthr, int par, int* ovf, bool edge) {
            float m = v[0];
#pragma unroll
            for (int i = 1; i < 16; ++i) m = fminf(m, v[i]);
            if (!(m <= pthr)) return;  // no hit among the 16 (pthr = thr once hits are rare)
            unsigned long long* buf = sBuf + (par * kT5Rows + myrow) * kT5BufStride;
            int* cnt = sCnt + par * kT5Rows + myrow;
#pragma unroll
            for (int i = 0; i < 16; ++i) {
                if (v[i] <= thr && (!edge || col0 + i < r1)) {
                    const int pos = atomicAdd(cnt, 1);
                    if (pos < kT5Buf) buf[pos] = score_key(v[i], uint32_t(col0 + i));
                    else *ovf = 1;
                }
            }
        };
        // merge the buffered hits (parity par) of this warp's rows into their
        // lists: the 8 rows side by side, one hit of each row per step (a row
        // out of hits offers the sentinel); a step no row can use is skipped
        auto merge = [&](int par) {
            int* cnt = sCnt + par * kT5Rows + grow;
            const int n = min(*cnt, kT5Buf);  // the same on the 4 lanes of a group
            const unsigned long long* B = sBuf + (par * kT5Rows + grow) * kT5BufStride;
            const int nmax = __reduce_max_sync(0xFFFFFFFFu, n);
            // the last lane of a group holds the row's worst key: it alone
            // decides whether its row can use the step (no shuffle per step),
            // and the next hit is loaded while this one is inserted
            unsigned long long c = 0 < n ? B[0] : kScoreSentinel;
            for (int h = 0; h < nmax; ++h) {
                const unsigned long long cn = h + 1 < n ? B[h + 1] : kScoreSentinel;
                if (__any_sync(0xFFFFFFFFu, gl == 3 && c < glist.slot[RS - 1])) glist.insert(c, gl);
                c = cn;
            }
            gworst = glist.worst();
            if (gl == 0 && n > 0) {
                *cnt = 0;
                sThr[grow] = fminf(t0g, key_score(gworst));
            }
        };
        for (int t = 0; t < nseq; ++t) {
            const int st = t & 1, par = t & 1, f4 = t & 3;
            const uint32_t ph = (t >> 1) & 1;
            const bool pre = t < npre;
            const int tt = tile_of(t);
            const int base = r0 + tt * kT5Cols;
            const uint32_t tcol = trow + uint32_t(st * kT5Cols);
            int w_ok = 1;
            if (lane == 0) w_ok = sm100::mbar_wait(&mma_done[st], ph, a.max_tries);
            w_ok = __shfl_sync(0xFFFFFFFFu, w_ok, 0);
            int* F = pre ? sFlag : qFlag;  // this step's flags (block-wide while sampling)
            if (pre ? tid == 0 : (cgroup == 0 && lane == 0)) {
                // flags of step t + 2 (last read before the barrier of step t - 1)
                F[(f4 + 2) & 3] = 0;
                F[4 + ((f4 + 2) & 3)] = 0;
            }
            if (w_ok && pre) {
                // one group minimum (64 scores) of this thread's row per sample tile
                sm100::tc_fence_after();
                float m = __int_as_float(0x7f800000);
#pragma unroll 1
                for (int j = 0; j < NPHASE; ++j) {
                    float v0[16];
                    sm100::tmem_ld16(tcol + uint32_t(j * kT5Chunk + cgroup * 16), v0);
#pragma unroll
                    for (int i = 0; i < 16; ++i) m = fminf(m, v0[i]);
                }
                sMin[myrow * kT5MinStride + t * 4 + cgroup] = m == m ? score_bits(m) : 0xFFFFFFFFu;
            } else if (w_ok) {
                sm100::tc_fence_after();
                const float thr = sThr[myrow];
                // the 16-score pre-check pays once hits are rare (from the 16th tile of the slice on)
                const float pthr = tt >= 16 ? thr : __int_as_float(0x7f800000);
                const bool edge = base + kT5Cols > r1;
#pragma unroll
                for (int j = 0; j < NPHASE; j += 2) {
                    float v0[16], v1[16];
                    sm100::tmem_ld16x2(tcol + uint32_t(j * kT5Chunk + cgroup * 16),
                                       tcol + uint32_t((j + 1) * kT5Chunk + cgroup * 16), v0, v1);
                    append16(v0, base + j * kT5Chunk + cgroup * 16, thr, pthr, par, &F[f4], edge);
                    append16(v1, base + (j + 1) * kT5Chunk + cgroup * 16, thr, pthr, par, &F[f4], edge);
                }
            } else if (lane == 0) {
                F[4 + f4] = 1;
            }
            if (pre) bar_all();
            else bar_quarter();
            const int bad = F[4 + f4];   // agreed (block / quarter): written only before the barrier above
            const int ovf = F[f4];
            if (!bad && pre && t == npre - 1) {
                // T0 of row grow = the C-th smallest of its 2C group minima,
                // found by the row's 4 lanes by bisection on the order-
                // preserving image (C/2 minima per lane, interleaved so that
                // the 4 lanes read 4 different banks)
                const uint32_t* mins = sMin + grow * kT5MinStride + gl;
                uint32_t lo = 0u, hi = 0xFFFFFFFFu;
#pragma unroll 1
                for (int it = 0; it < 32; ++it) {
                    const uint32_t mid = lo + ((hi - lo) >> 1);
                    int cnt = 0;
#pragma unroll 8
                    for (int i = 0; i < C / 2; ++i) cnt += mins[4 * i] <= mid ? 1 : 0;
                    cnt += __shfl_xor_sync(0xFFFFFFFFu, cnt, 1);
                    cnt += __shfl_xor_sync(0xFFFFFFFFu, cnt, 2);
                    if (cnt >= C) hi = mid;
                    else lo = mid + 1u;
                }
                // images above +inf's are NaN minima (never certified): no threshold
                t0g = lo < 0xFF800000u ? bits_score(lo) : __int_as_float(0x7f800000);
                if (gl == 0) sThr[grow] = t0g;
                bar_all();  // no quarter appends hits over the sample's minima before all have read them
            }
            if (!bad && ovf) {
                // redo the tile in eight steps of 32 columns (two column groups each)
                if (cgroup == 0) sCnt[par * kT5Rows + myrow] = 0;  // the quarter's rows
                bar_quarter();
#pragma unroll 1
                for (int j = 0; j < 2 * NPHASE; ++j) {
                    if ((cgroup >> 1) == (j & 1)) {
                        const float thr = sThr[myrow];
                        float v[16];
                        sm100::tmem_ld16(tcol + uint32_t((j >> 1) * kT5Chunk + cgroup * 16), v);
                        int dummy = 0;
                        append16(v, base + (j >> 1) * kT5Chunk + cgroup * 16, thr, __int_as_float(0x7f800000), par,
                                 &dummy, true);  // <= 32 hits per row
                    }
                    bar_quarter();
                    merge(par);
                    bar_quarter();
                }
            }
            // this tile's accumulator is no longer read
            sm100::tc_fence_before();
            __syncwarp();
            if (lane == 0) sm100::mbar_arrive(&epi_done[st]);
            if (bad) {
                if (cgroup == 0 && lane == 0) atomicOr(a.err, kTcErrTimeout);
                break;
            }
            if (!ovf && !pre) merge(par);
        }
        // write the lists: C candidates per row and the row threshold
        {
            const int q = blockIdx.x * kT5Rows + grow;
            if (q < a.nq) {
                const long long base = ((long long)q * a.nsplit + blockIdx.y) * C + RS * gl;
#pragma unroll
                for (int i = 0; i < RS; ++i) {
                    const unsigned long long key = glist.slot[i];
                    const bool real = key != kScoreSentinel;
                    a.cand_s[base + i] = key_score(key);
                    a.cand_i[base + i] = real ? int32_t(uint32_t(key)) : -1;
                }
                if (gl == 0) a.tau[(long long)q * a.nsplit + blockIdx.y] = key_score(gworst);
            }
        }
    }
    // teardown: everyone done with tensor memory
    sm100::tc_fence_before();
    __syncthreads();
    sm100::tc_fence_after();
    if (warp == kT5EpiWarps) sm100::tmem_dealloc(tmem, 512);
}

// Shared memory of the mma.sync candidate search for (mode, KP, C).
inline size_t select_smem_bytes(int mode, int KP, int C) {
    const int KW = (mode == TK_BRUTE_TF32) ? KP : KP / 2;
    const int PLANES = (mode == TK_BRUTE_TF32) ? 1 : 2;
    return sizeof(uint32_t) * PLANES * kCols * (KW + 4) + sizeof(float) * kCols +
           sizeof(float) * kRows * (kCols + 4) + (sizeof(float) + sizeof(int32_t)) * size_t(C) * kRows;
}
template <int MODE, int KP, int C>
size_t select_smem_bytes() {
    return select_smem_bytes(MODE, KP, C);
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
    const int* err;       // candidate kernel gave up (bounded wait ran out): certify nothing
};

// Exact FP32 squared distance of reference row rr to the query (the
// reference's arithmetic: coordinate differences squared and summed in
// coordinate order); rows read 16 bytes at a time when `vec` (d % 4 == 0,
// 16-byte aligned rows), which cut the re-rank of the 262,144 x 65,536, d=32
// workload from 0.96 to ~0.45 ms.
__device__ __forceinline__ float rerank_dist(const float* __restrict__ qrow, const float* __restrict__ rr, int d,
                                             bool vec) {
    float acc;
    if (vec) {
        const float4* q4 = reinterpret_cast<const float4*>(qrow);
        const float4* r4 = reinterpret_cast<const float4*>(rr);
        float4 qv = __ldg(q4), rv = __ldg(r4);
        float t = __fsub_rn(qv.x, rv.x);
        acc = __fmul_rn(t, t);
        t = __fsub_rn(qv.y, rv.y);
        acc = __fadd_rn(acc, __fmul_rn(t, t));
        t = __fsub_rn(qv.z, rv.z);
        acc = __fadd_rn(acc, __fmul_rn(t, t));
        t = __fsub_rn(qv.w, rv.w);
        acc = __fadd_rn(acc, __fmul_rn(t, t));
        for (int c = 1; c < (d >> 2); ++c) {
            qv = __ldg(q4 + c);
            rv = __ldg(r4 + c);
            t = __fsub_rn(qv.x, rv.x);
            acc = __fadd_rn(acc, __fmul_rn(t, t));
            t = __fsub_rn(qv.y, rv.y);
            acc = __fadd_rn(acc, __fmul_rn(t, t));
            t = __fsub_rn(qv.z, rv.z);
            acc = __fadd_rn(acc, __fmul_rn(t, t));
            t = __fsub_rn(qv.w, rv.w);
            acc = __fadd_rn(acc, __fmul_rn(t, t));
        }
    } else {
        float t = __fsub_rn(qrow[0], rr[0]);
        acc = __fmul_rn(t, t);
        for (int c = 1; c < d; ++c) {
            t = __fsub_rn(qrow[c], rr[c]);
            acc = __fadd_rn(acc, __fmul_rn(t, t));
        }
    }
    return acc;
}

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
    const bool vec =
        (a.d & 3) == 0 && ((reinterpret_cast<uintptr_t>(a.ref) | reinterpret_cast<uintptr_t>(a.q)) & 15) == 0;
    for (int e0 = 0; e0 < total; e0 += 32) {
        const int e = e0 + lane;
        Key<float> mine = Key<float>::sentinel();
        const int r = e < total ? a.cand_i[base + e] : -1;
        if (r >= 0) mine = Key<float>::make(rerank_dist(qrow, a.ref + (long long)r * a.d, a.d, vec), uint32_t(r));
        worst = offer<float, 32, R>(list, mine, worst, 0xFFFFFFFFu, lane, 0);
    }
    list.store(a.k, lane, a.out_d, a.out_i, qi);
    // certificate (lane 0)
    if (lane == 0) {
        double tau = INFINITY;
        for (int s = 0; s < a.nsplit; ++s) tau = fmin(tau, (double)a.tau[(long long)qi * a.nsplit + s]);
        bool ok = !(a.err && *a.err);
        double qq = 0.0;
        for (int c = 0; c < a.d; ++c) qq += (double)qrow[c] * (double)qrow[c];
        ok = ok && qq < double(kTcNormLimit);  // see kTcNormLimit (false for NaN / inf coordinates)
        if (ok && !isinf(tau)) {
            const double D = (double)worst.dist();
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

template <int MODE, int KP, int CH>
int launch_tc5(const Tc5Args& a, int qblocks, cudaStream_t s) {
    using Sh = Tc5Shape<MODE, KP, CH>;
    const void* fn = reinterpret_cast<const void*>(&k_tc5_select<MODE, KP, CH>);
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(Sh::SMEM));
    if (e != cudaSuccess) return fail(TK_ECUDA, std::string("tcgen05 select smem: ") + cudaGetErrorString(e));
    k_tc5_select<MODE, KP, CH><<<dim3(qblocks, a.nsplit), kT5Threads, Sh::SMEM, s>>>(a);
    return TK_OK;
}

template <int MODE, int KP>
int tc5_dispatch_ch(const Tc5Args& a, int CH, int qblocks, cudaStream_t s) {
    switch (CH) {
        case 8: return launch_tc5<MODE, KP, 8>(a, qblocks, s);
        case 16: return launch_tc5<MODE, KP, 16>(a, qblocks, s);
        case 32: return launch_tc5<MODE, KP, 32>(a, qblocks, s);
        default: return fail(TK_EUNSUPPORTED, "tcgen05 path: k <= 32");
    }
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

// Entry points of the candidate kernels, one unit each.
int tc5_dispatch_tf32(const Tc5Args& a, int KP, int CH, int qblocks, cudaStream_t s);       // brute_tc5_tf32.cu
int tc5_dispatch_tf32_deep(const Tc5Args& a, int KP, int CH, int qblocks, cudaStream_t s);  // brute_tc5_tf32_deep.cu
int tc5_dispatch_bf16(const Tc5Args& a, int KP, int CH, int qblocks, cudaStream_t s);  // brute_tc5_bf16.cu
int tc_select_dispatch(const TcArgs& a, int mode, int qblocks, cudaStream_t s);          // brute_tc_mma.cu

}  // namespace tcx
}  // namespace tk
