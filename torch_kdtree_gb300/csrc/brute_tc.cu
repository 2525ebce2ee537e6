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
//
// Kernels and launch templates: brute_tc_kernels.cuh; the candidate kernels
// are instantiated in brute_tc5_tf32.cu, brute_tc5_tf32_deep.cu,
// brute_tc5_bf16.cu (tcgen05) and brute_tc_mma.cu (mma.sync), compiled in
// parallel.
#include <algorithm>
#include <atomic>
#include <string>

#include "brute_tc.cuh"
#include "brute_tc_kernels.cuh"

namespace tk {
using namespace tcx;
namespace {

struct TcWs {
    size_t a_pack, b_pack, a_lo, b_lo, rnorm, qnorm, cand_s, cand_i, tau, fail_count, fail_list, brute, err, total;
    int KP, C, nsplit;
    bool tc5;  // tcgen05 path
};

// tcgen05 path: K = d + 1 (augmented), padded to the MMA's K step.
bool tc5_eligible(int d, int k, int mode) {
    if (k > 32) return false;
    return mode == TK_BRUTE_TF32 ? (d + 1 <= 40) : (d + 1 <= 48);
}
int tc5_kp(int d, int mode) {
    const int step = mode == TK_BRUTE_TF32 ? 8 : 16;
    return (d + 1 + step - 1) / step * step;
}

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
    w.tc5 = tc5_eligible(d, k, mode);
    w.KP = w.tc5 ? tc5_kp(d, mode) : tc_kp(d, mode);
    w.C = tc_over(k);
    const size_t es = mode == TK_BRUTE_TF32 ? 4 : 2;
    size_t o = 0;
    if (w.tc5) {
        const int qblocks = int((nq + kT5Rows - 1) / kT5Rows);
        int ns = std::max(1, (8 * sms + qblocks / 2) / std::max(1, qblocks));
        ns = int(std::min<int64_t>({int64_t(ns), int64_t(8), std::max<int64_t>(1, n / (8 * kT5Cols))}));
        w.nsplit = ns;
        const size_t nq_pad = size_t(qblocks) * kT5Rows;
        const size_t n_pad = size_t((n + kT5Cols - 1) / kT5Cols) * kT5Cols;
        w.a_pack = o; o += align256(es * nq_pad * w.KP);
        w.b_pack = o; o += align256(es * n_pad * w.KP);
        w.a_lo = o; o += mode == TK_BRUTE_TF32 ? 0 : align256(es * nq_pad * w.KP);
        w.b_lo = o; o += mode == TK_BRUTE_TF32 ? 0 : align256(es * n_pad * w.KP);
        w.rnorm = w.qnorm = o;
    } else {
        const int qblocks = int((nq + kRows - 1) / kRows);
        int ns = std::max(1, (2 * sms + qblocks - 1) / std::max(1, qblocks));
        ns = int(std::min<int64_t>(ns, std::max<int64_t>(1, n / (4 * kCols))));
        w.nsplit = ns;
        w.a_pack = o; o += align256(es * size_t(nq) * w.KP);
        w.b_pack = o; o += align256(es * size_t(n) * w.KP);
        w.a_lo = o; o += mode == TK_BRUTE_TF32 ? 0 : align256(es * size_t(nq) * w.KP);
        w.b_lo = o; o += mode == TK_BRUTE_TF32 ? 0 : align256(es * size_t(n) * w.KP);
        w.rnorm = o; o += align256(4 * size_t(n));
        w.qnorm = o; o += align256(4 * size_t(nq));
    }
    w.err = o; o += 256;
    w.cand_s = o; o += align256(4 * size_t(nq) * w.nsplit * w.C);
    w.cand_i = o; o += align256(4 * size_t(nq) * w.nsplit * w.C);
    w.tau = o; o += align256(4 * size_t(nq) * w.nsplit);
    w.fail_count = o; o += 256;
    w.fail_list = o; o += align256(4 * size_t(nq));
    w.brute = o; o += brute_fallback_workspace_bytes(n, nq, d, k);
    w.total = o;
    return w;
}

// Every query on the fallback list: the tensor-core candidate search does
// not fit this shape (see run_brute_tc), the exact kernel answers them all.
__global__ void k_all_queries(int nq, int* list, int* count) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nq) list[i] = i;
    if (i == 0) *count = nq;
}

// Poll budget of the candidate kernel's bounded waits (0 = kT5MaxTries); set
// by tk_set_device_wait_limit.
std::atomic<uint32_t> g_wait_polls{0};

int sm_count_now() {
    int dev = 0, v = 1;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v < 1) v = 1;
    return v;
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
    cudaError_t e0 = cudaMemsetAsync(p + w.err, 0, sizeof(int), s);
    int* err = reinterpret_cast<int*>(p + w.err);  // no certificates when set (see kTcNormLimit)
    if (e0 != cudaSuccess) return fail(TK_ECUDA, std::string("memset: ") + cudaGetErrorString(e0));
    if (!w.tc5) {
        // The mma.sync candidate search keeps 128 rows' lists and a score tile
        // in shared memory; for k > 32 with d > 32 (C = 128, KP = 64) that is
        // more than a block may have.  The answer is exact either way, so the
        // exact kernel answers every query (tk_nn_distance_report: all
        // recomputed) instead of failing the call.
        int dev = 0, optin = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) optin = 0;
        if (select_smem_bytes(mode, w.KP, w.C) > size_t(optin)) {
            int* list = reinterpret_cast<int*>(p + w.fail_list);
            int* count = reinterpret_cast<int*>(p + w.fail_count);
            k_all_queries<<<(nq32 + 255) / 256, 256, 0, s>>>(nq32, list, count);
            const cudaError_t e1 = cudaGetLastError();
            if (e1 != cudaSuccess) return fail(TK_ECUDA, std::string("fallback list: ") + cudaGetErrorString(e1));
            return brute_fallback(ref, n, q, nq, d, k, dists, idx, list, count, p + w.brute,
                                  brute_fallback_workspace_bytes(n, nq, d, k), s);
        }
    }
    int crc = TK_OK;
    if (w.tc5) {
        // 1-2. pack into the core-matrix layout and run the tcgen05 candidate kernel
        const int qblocks = (nq32 + kT5Rows - 1) / kT5Rows;
        const int n_pad = int((n + kT5Cols - 1) / kT5Cols) * kT5Cols;
        unsigned char* ahi = reinterpret_cast<unsigned char*>(p + w.a_pack);
        unsigned char* alo = reinterpret_cast<unsigned char*>(p + w.a_lo);
        unsigned char* bhi = reinterpret_cast<unsigned char*>(p + w.b_pack);
        unsigned char* blo = reinterpret_cast<unsigned char*>(p + w.b_lo);
        const int nq_pad = qblocks * kT5Rows;
        if (mode == TK_BRUTE_TF32) {
            k_tc5_pack<TK_BRUTE_TF32><<<(nq_pad + 255) / 256, 256, 0, s>>>(q, nq32, nq_pad, d, w.KP, kT5Rows, 1, ahi, alo,
                                                                         err);
            k_tc5_pack<TK_BRUTE_TF32><<<(n_pad + 255) / 256, 256, 0, s>>>(ref, n32, n_pad, d, w.KP, kT5Cols, 0, bhi, blo,
                                                                        err);
        } else {
            k_tc5_pack<TK_BRUTE_BF16_SPLIT><<<(nq_pad + 255) / 256, 256, 0, s>>>(q, nq32, nq_pad, d, w.KP, kT5Rows, 1,
                                                                               ahi, alo, err);
            k_tc5_pack<TK_BRUTE_BF16_SPLIT><<<(n_pad + 255) / 256, 256, 0, s>>>(ref, n32, n_pad, d, w.KP, kT5Cols, 0,
                                                                              bhi, blo, err);
        }
        Tc5Args t5{};
        t5.a_hi = ahi;
        t5.a_lo = alo;
        t5.b_hi = bhi;
        t5.b_lo = blo;
        t5.n = n32;
        t5.nq = nq32;
        t5.nsplit = w.nsplit;
        t5.cand_s = reinterpret_cast<float*>(p + w.cand_s);
        t5.cand_i = reinterpret_cast<int32_t*>(p + w.cand_i);
        t5.tau = reinterpret_cast<float*>(p + w.tau);
        t5.err = reinterpret_cast<int*>(p + w.err);
        const uint32_t polls = g_wait_polls.load();
        t5.max_tries = polls ? polls : kT5MaxTries;
        crc = mode == TK_BRUTE_TF32 ? tc5_dispatch_tf32(t5, w.KP, w.C / 2, qblocks, s)
                                    : tc5_dispatch_bf16(t5, w.KP, w.C / 2, qblocks, s);
        if (crc != TK_OK) return crc;
    } else if (mode == TK_BRUTE_TF32) {
        k_tc_pack<TK_BRUTE_TF32><<<(nq32 + 255) / 256, 256, 0, s>>>(q, nq32, d, w.KP, reinterpret_cast<uint32_t*>(p + w.a_pack),
                                                                  nullptr, nullptr, reinterpret_cast<float*>(p + w.qnorm),
                                                                  nullptr);
        k_tc_pack<TK_BRUTE_TF32><<<(n32 + 255) / 256, 256, 0, s>>>(ref, n32, d, w.KP, reinterpret_cast<uint32_t*>(p + w.b_pack),
                                                                 nullptr, nullptr, reinterpret_cast<float*>(p + w.rnorm),
                                                                 err);
    } else {
        k_tc_pack<TK_BRUTE_BF16_SPLIT><<<(nq32 + 255) / 256, 256, 0, s>>>(
            q, nq32, d, w.KP, nullptr, reinterpret_cast<__nv_bfloat16*>(p + w.a_pack),
            reinterpret_cast<__nv_bfloat16*>(p + w.a_lo), reinterpret_cast<float*>(p + w.qnorm), nullptr);
        k_tc_pack<TK_BRUTE_BF16_SPLIT><<<(n32 + 255) / 256, 256, 0, s>>>(
            ref, n32, d, w.KP, nullptr, reinterpret_cast<__nv_bfloat16*>(p + w.b_pack),
            reinterpret_cast<__nv_bfloat16*>(p + w.b_lo), reinterpret_cast<float*>(p + w.rnorm), err);
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
    if (!w.tc5) {
        crc = tc_select_dispatch(a, mode, qblocks, s);
        if (crc != TK_OK) return crc;
    }
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
    ra.eps_dot = mode == TK_BRUTE_TF32 ? (1.0 / 1024.0 + 1.0 / 4194304.0 + (d + 2) * 2.0 * u)
                                       : (3.1 / 65536.0 + 3.0 * (d + 2) * 2.0 * u);
    ra.out_d = dists;
    ra.out_i = idx;
    ra.fail_count = reinterpret_cast<int*>(p + w.fail_count);
    ra.fail_list = reinterpret_cast<int*>(p + w.fail_list);
    ra.err = reinterpret_cast<const int*>(p + w.err);
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

extern "C" uint32_t tk_set_device_wait_limit(uint32_t polls) { return tk::g_wait_polls.exchange(polls); }

extern "C" int tk_nn_distance_report(const void* workspace, int64_t n, int64_t nq, int dims, int k, int dtype,
                                     int mode, int* flags, int* recomputed) {
    using namespace tk;
    using namespace tk::tcx;
    clear_error();
    if (!flags || !recomputed) return fail(TK_EINVAL, "null output pointer");
    *flags = 0;
    *recomputed = 0;
    if (mode != TK_BRUTE_TF32 && mode != TK_BRUTE_BF16_SPLIT) return TK_OK;  // the exact kernel has no certificate
    if (dtype != TK_F32) return fail(TK_EINVAL, "tensor-core modes take float32 inputs");
    if (!workspace || n < 1 || nq < 1 || k < 1 || dims < 1) return fail(TK_EINVAL, "bad shape or null workspace");
    const TcWs w = tc_layout(n, nq, dims, k, mode, sm_count_now());
    const char* p = static_cast<const char*>(workspace);
    cudaError_t e = cudaMemcpy(flags, p + w.err, sizeof(int), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(recomputed, p + w.fail_count, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return fail(TK_ECUDA, std::string("report: ") + cudaGetErrorString(e));
    if (*flags & kTcErrTimeout)
        return fail(TK_ETIMEOUT, "a bounded device wait ran out; the exact kernel recomputed every query");
    return TK_OK;
}
