// nn_distance: exhaustive exact KNN on CUDA cores (see brute.cuh), plus the
// C entry points for every brute-force mode.
#include <algorithm>
#include <mutex>
#include <string>
#include <vector>

#include "brute.cuh"
#include "brute_tc.cuh"

namespace tk {
namespace {

size_t align256(size_t v) { return (v + 255) / 256 * 256; }

int pow2_ceil(int v) {
    int p = 1;
    while (p < v) p <<= 1;
    return p;
}

int sm_count_dev() {
    static std::mutex mu;
    static std::vector<int> cache;
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lock(mu);
    if ((int)cache.size() <= dev) cache.resize(dev + 1, 0);
    if (!cache[dev]) {
        int v = 0;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) v = 1;
        cache[dev] = v;
    }
    return cache[dev];
}

// padded dimension for d
int padded_dims(int d) {
    if (d <= 4) return d;
    if (d <= 8) return 8;
    if (d <= 16) return 16;
    if (d <= 32) return 32;
    if (d <= 64) return 64;
    return 128;
}

BrutePlan plan_brute(int64_t n, int64_t nq, int d, int k, bool f32) {
    BrutePlan p;
    p.DP = padded_dims(d);
    if (f32 && p.DP % 4 == 0 && p.DP <= 32 && k <= 32) {
        // one lane per query with broadcast 16-byte row loads (brute.cuh)
        p.G = 1;
        p.R = k <= 1 ? 1 : (k <= 4 ? 4 : (k <= 16 ? 16 : 32));
    } else {
        p.G = std::max(1, pow2_ceil((k + 15) / 16));
        p.R = pow2_ceil((k + p.G - 1) / p.G);
        if (p.G == 1) p.R = p.R <= 1 ? 1 : (p.R <= 4 ? 4 : 16);
    }
    const int per_block = 256 / p.G;
    p.qtiles = int((nq + per_block - 1) / per_block);
    const int target = 8 * sm_count_dev();
    int ns = std::max(1, (target + p.qtiles - 1) / std::max(1, p.qtiles));
    ns = int(std::min<int64_t>(ns, std::max<int64_t>(1, n / 2048)));
    p.nsplit = ns;
    return p;
}

template <typename T>
size_t brute_ws_bytes(const BrutePlan& p, int64_t nq, int k) {
    if (p.nsplit <= 1) return 256;
    return align256(sizeof(Key<T>) * size_t(nq) * p.nsplit * k);
}

template <typename T>
int run_brute(const T* ref, int64_t n, const T* q, int64_t nq, int d, int k, T* dists, int32_t* idx, void* ws,
              size_t ws_bytes, cudaStream_t s) {
    const BrutePlan p = plan_brute(n, nq, d, k, sizeof(T) == 4);
    if (ws_bytes < brute_ws_bytes<T>(p, nq, k) || (p.nsplit > 1 && !ws))
        return fail(TK_EWORKSPACE, "workspace too small");
    BruteArgs<T> a;
    a.ref = ref;
    a.q = q;
    a.n = int(n);
    a.nq = int(nq);
    a.d = d;
    a.k = k;
    a.nsplit = p.nsplit;
    a.out_d = dists;
    a.out_i = idx;
    a.part = static_cast<Key<T>*>(ws);
    switch (p.DP) {
        case 1: return launch_dp<T, 1>(a, p, s);
        case 2: return launch_dp<T, 2>(a, p, s);
        case 3: return launch_dp<T, 3>(a, p, s);
        case 4: return launch_dp<T, 4>(a, p, s);
        default: break;
    }
    if constexpr (sizeof(T) == 4) {
        switch (p.DP) {
            case 8: return launch_dp<T, 8>(a, p, s);
            case 16: return launch_dp<T, 16>(a, p, s);
            case 32: return launch_dp<T, 32>(a, p, s);
            case 64: return launch_dp<T, 64>(a, p, s);
            case 128: return launch_dp<T, 128>(a, p, s);
            default: break;
        }
    } else {
        return launch_brute_f64_wide(a, p, s);  // brute_f64.cu: d = 5 .. 128
    }
    return fail(TK_EUNSUPPORTED, "no brute-force kernel for this dimension");
}

int check_common(const void* ref, int64_t n, const void* q, int64_t nq, int d, int k, int dtype, const void* dists,
                 const void* idx) {
    if (n < 1 || n >= (int64_t(1) << 31)) return fail(TK_EINVAL, "reference count must be in [1, 2^31)");
    if (nq < 0 || nq >= (int64_t(1) << 31)) return fail(TK_EINVAL, "query count must be in [0, 2^31)");
    if (d < 1 || d > 128) return fail(TK_EINVAL, "dims must be in [1, 128]");
    if (k < 1) return fail(TK_EINVAL, "k must be >= 1");
    if (k > n) return fail(TK_EINVAL, "You requested more nearest neighbors than there are reference points");
    if (k > kMaxK) return fail(TK_EINVAL, "k is limited to 128");
    if (dtype != TK_F32 && dtype != TK_F64) return fail(TK_EINVAL, "dtype must be TK_F32 or TK_F64");
    if (nq > 0 && (!ref || !q || !dists || !idx)) return fail(TK_EINVAL, "null pointer");
    return TK_OK;
}

}  // namespace

// The fallback expects few listed queries: it slices the references finely
// (as planned for 1,024 queries) and launches for the worst case of all nq;
// blocks past the device-side count exit at once.
size_t brute_fallback_workspace_bytes(int64_t n, int64_t nq, int d, int k) {
    BrutePlan p = plan_brute(n, std::min<int64_t>(std::max<int64_t>(nq, 1), 1024), d, k, true);
    if (p.nsplit <= 1) return 256;
    return align256(sizeof(Key<float>) * size_t(std::max<int64_t>(nq, 1)) * p.nsplit * k);
}

int brute_fallback(const float* ref, int64_t n, const float* q, int64_t nq, int d, int k, float* dists,
                   int32_t* idx, const int* qlist, const int* qcount, void* ws, size_t ws_bytes, cudaStream_t s) {
    BrutePlan p = plan_brute(n, std::min<int64_t>(std::max<int64_t>(nq, 1), 1024), d, k, true);
    const int per_block = 256 / p.G;
    p.qtiles = int((nq + per_block - 1) / per_block);
    if (ws_bytes < brute_fallback_workspace_bytes(n, nq, d, k)) return fail(TK_EWORKSPACE, "fallback workspace");
    BruteArgs<float> a;
    a.ref = ref;
    a.q = q;
    a.n = int(n);
    a.nq = int(nq);
    a.d = d;
    a.k = k;
    a.nsplit = p.nsplit;
    a.out_d = dists;
    a.out_i = idx;
    a.part = static_cast<Key<float>*>(ws);
    a.qlist = qlist;
    a.qcount = qcount;
    switch (p.DP) {
        case 1: return launch_dp<float, 1>(a, p, s);
        case 2: return launch_dp<float, 2>(a, p, s);
        case 3: return launch_dp<float, 3>(a, p, s);
        case 4: return launch_dp<float, 4>(a, p, s);
        case 8: return launch_dp<float, 8>(a, p, s);
        case 16: return launch_dp<float, 16>(a, p, s);
        case 32: return launch_dp<float, 32>(a, p, s);
        case 64: return launch_dp<float, 64>(a, p, s);
        default: return launch_dp<float, 128>(a, p, s);
    }
}

}  // namespace tk

using namespace tk;

extern "C" {

size_t tk_nn_distance_workspace_size(int64_t n, int64_t nq, int dims, int k, int dtype, int mode) {
    if (n < 1 || nq < 0 || k < 1 || dims < 1) return 0;
    if (mode == TK_BRUTE_TF32 || mode == TK_BRUTE_BF16_SPLIT) return brute_tc_workspace_bytes(n, nq, dims, k, mode);
    const BrutePlan p = plan_brute(n, std::max<int64_t>(nq, 1), dims, k, dtype != TK_F64);
    return dtype == TK_F64 ? brute_ws_bytes<double>(p, std::max<int64_t>(nq, 1), k)
                           : brute_ws_bytes<float>(p, std::max<int64_t>(nq, 1), k);
}

int tk_nn_distance(const void* ref, int64_t n, const void* q, int64_t nq, int dims, int k, int dtype, int mode,
                   void* dists, int32_t* idx, void* workspace, size_t workspace_bytes, void* stream) {
    clear_error();
    int rc = check_common(ref, n, q, nq, dims, k, dtype, dists, idx);
    if (rc != TK_OK) return rc;
    if (nq == 0) return TK_OK;
    if (ws_misaligned(workspace)) return fail(TK_EINVAL, "workspace must be 256-byte aligned");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (mode == TK_BRUTE_EXACT) {
        if (dtype == TK_F32)
            return run_brute<float>(static_cast<const float*>(ref), n, static_cast<const float*>(q), nq, dims, k,
                                    static_cast<float*>(dists), idx, workspace, workspace_bytes, s);
        return run_brute<double>(static_cast<const double*>(ref), n, static_cast<const double*>(q), nq, dims, k,
                                 static_cast<double*>(dists), idx, workspace, workspace_bytes, s);
    }
    if (mode == TK_BRUTE_TF32 || mode == TK_BRUTE_BF16_SPLIT) {
        if (dtype != TK_F32) return fail(TK_EINVAL, "tensor-core modes take float32 inputs");
        return run_brute_tc(static_cast<const float*>(ref), n, static_cast<const float*>(q), nq, dims, k, mode,
                            static_cast<float*>(dists), idx, workspace, workspace_bytes, s);
    }
    return fail(TK_EINVAL, "unknown brute-force mode");
}

}  // extern "C"
