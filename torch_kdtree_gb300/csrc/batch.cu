// Batched queries over many point clouds in one persistent launch.
//
// A batch plan references already-built trees (each with its own depth and
// its own k) and fixes the per-cloud query counts, so that everything the
// device needs -- a descriptor per cloud, query / output offsets, bin bases
// -- is uploaded once.  A batched query is then device work only (binning
// kernels + one persistent KD kernel), safe to capture in a CUDA graph.
//
//   1. k_batch_bin_count: each query finds its cloud (binary search over the
//      query prefix), descends B_c levels of that cloud's tree and counts
//      itself into the cloud's block of cells;
//   2. exclusive_scan over all cells; 3. k_bin_scatter -> processing order;
//   4. k_batch_query: warps pull chunks of the binned order from one global
//      counter (the work queue); every group looks up its query's cloud and
//      runs the same exact search as the single-cloud kernel with that
//      cloud's tree and k.
// Trees of 4-8 dimensions take the same steps with the wide trees' records
// and search (batch_wide.cuh); all clouds of a batch have one dims.
#include <algorithm>
#include <string>
#include <vector>

#include "batch_wide.cuh"
#include "kd_query.cuh"
#include "sort.cuh"
#include "tk_internal.h"

namespace tk {

template <typename T>
struct CloudDesc {
    const PointRec<T>* pts;
    const T* medians;
    const int32_t* leaf_off;
    const PointRec<T>* boxes;  // null: prune with split planes only
    long long out_off;  // element offset of the cloud's [nq_c, k_c] block in the outputs
    int levels;
    int k;
    int bins;       // 2^B_c cells used for binning
    int bin_base;   // first cell of this cloud in the global cell array
};

template <typename T>
struct BatchArgs {
    const CloudDesc<T>* desc;
    const long long* q_prefix;  // [n_clouds + 1] global query offsets
    int n_clouds;
    const T* q;                 // concatenated queries [total, D]
    int total;
    const int32_t* order;
    T* out_d;
    int32_t* out_i;
    int* work;
    int use_boxes;
};

__device__ __forceinline__ int cloud_of(const long long* prefix, int n_clouds, long long qi) {
    return batch_cloud_of(prefix, n_clouds, qi);
}

template <typename T, int D>
__global__ void k_batch_bin_count(const BatchArgs<T> a, int* counts, int* bin_of, int* pos_of) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.total) return;
    const int c = cloud_of(a.q_prefix, a.n_clouds, i);
    const CloudDesc<T> cd = a.desc[c];
    T p[D];
#pragma unroll
    for (int j = 0; j < D; ++j) p[j] = a.q[(long long)i * D + j];
    int B = 0;
    while ((1 << B) < cd.bins) ++B;
    int node = 0, ax = 0;
    for (int depth = 0; depth < B; ++depth) {
        const T m = __ldg(cd.medians + node);
        node = 2 * node + (pick<T, D>(p, ax) < m ? 1 : 2);
        ax = (ax + 1 == D) ? 0 : ax + 1;
    }
    const int bin = cd.bin_base + node - ((1 << B) - 1);
    bin_of[i] = bin;
    pos_of[i] = atomicAdd(counts + bin, 1);
}

template <typename T, int D, int G, int R>
__device__ __forceinline__ void batch_search(const CloudDesc<T>& cd, const T (&q)[D], long long local,
                                             const BatchArgs<T>& a, unsigned gmask, int gl, int gbase) {
    const TreeView<T> tv{cd.pts, cd.medians, cd.leaf_off, cd.levels, 0, nullptr, cd.boxes};
    const long long o = cd.out_off + local * cd.k;
    kd_search<T, D, G, R>(tv, q, cd.k, a.out_d + o, a.out_i + o, gmask, gl, gbase);
}

// G = 1: k <= 16 (registers per lane R in {1, 4, 16});
// G = 8: k <= 128 (R in {2, 4, 8, 16}).  Capped at 4 blocks of 256 per SM (64
// registers for float): left free the float kernels took 72-80 registers, 3
// blocks per SM, and ran the 256 ragged clouds 9-14% slower (a few bytes of
// spills cost less than a quarter of the resident warps).
template <typename T, int D, int G>
__global__ void __launch_bounds__(256, 4) k_batch_query(const BatchArgs<T> a) {
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
            const int c = cloud_of(a.q_prefix, a.n_clouds, qi);
            const CloudDesc<T> cd = a.desc[c];
            T q[D];
#pragma unroll
            for (int j = 0; j < D; ++j) q[j] = a.q[(long long)qi * D + j];
            const long long local = qi - a.q_prefix[c];
            if (G == 1) {
                if (cd.k <= 1) batch_search<T, D, G, 1>(cd, q, local, a, gmask, gl, gbase);
                else if (cd.k <= 4) batch_search<T, D, G, 4>(cd, q, local, a, gmask, gl, gbase);
                else batch_search<T, D, G, 16>(cd, q, local, a, gmask, gl, gbase);
            } else {
                if (cd.k <= 2 * G) batch_search<T, D, G, 2>(cd, q, local, a, gmask, gl, gbase);
                else if (cd.k <= 4 * G) batch_search<T, D, G, 4>(cd, q, local, a, gmask, gl, gbase);
                else if (cd.k <= 8 * G) batch_search<T, D, G, 8>(cd, q, local, a, gmask, gl, gbase);
                else batch_search<T, D, G, 16>(cd, q, local, a, gmask, gl, gbase);
            }
        }
        __syncwarp();
    }
}

__global__ void k_batch_scatter(int total, const int* bin_of, const int* pos_of, const int* offsets, int* order) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= total) return;
    order[offsets[bin_of[i]] + pos_of[i]] = i;
}

}  // namespace tk

using namespace tk;

struct tk_batch {
    int dtype = TK_F32, dims = 0, device = 0, n_clouds = 0;
    int max_k = 0;
    long long total_q = 0, total_out = 0;
    int total_bins = 0;
    void* d_desc = nullptr;
    long long* d_prefix = nullptr;
    std::vector<long long> q_prefix, out_off;
};

namespace {

size_t align256(size_t v) { return (v + 255) / 256 * 256; }

struct BatchWs {
    size_t counter, counts, bin_of, pos_of, order, scan, total;
};

BatchWs batch_ws(const tk_batch* b) {
    BatchWs w;
    size_t o = 0;
    w.counter = o;
    o += 256;
    w.counts = o;
    o += align256(sizeof(int) * size_t(std::max(1, b->total_bins)));
    w.bin_of = o;
    o += align256(sizeof(int) * size_t(std::max<long long>(1, b->total_q)));
    w.pos_of = o;
    o += align256(sizeof(int) * size_t(std::max<long long>(1, b->total_q)));
    w.order = o;
    o += align256(sizeof(int) * size_t(std::max<long long>(1, b->total_q)));
    w.scan = o;
    o += scan_workspace_bytes(std::max(1, b->total_bins));
    w.total = o;
    return w;
}

int batch_bin_levels(int L, long long nq) {
    int lg = 0;
    while ((1LL << (lg + 1)) <= nq) ++lg;
    return std::max(1, std::min({L, kMaxBinLevels, lg - 4}));
}

template <typename T>
void fill_desc(CloudDesc<T>& d, const tk_tree* t) {
    d.pts = static_cast<const PointRec<T>*>(t->d_pts);
    d.medians = static_cast<const T*>(t->d_medians);
    d.leaf_off = t->d_leaf_off;
    d.boxes = static_cast<const PointRec<T>*>(t->d_boxes);
}

template <typename T>
void fill_desc(WideCloudDesc<T>& d, const tk_tree* t) {
    d.pts = static_cast<const T*>(t->d_pts);
    d.perm = t->d_perm;
    d.medians = static_cast<const T*>(t->d_medians);
    d.leaf_off = t->d_leaf_off;
    d.boxes = static_cast<const T*>(t->d_boxes);
}

// Desc: CloudDesc<T> (trees of 1-3 dims) or WideCloudDesc<T> (4-8 dims).
template <typename T, typename Desc>
int upload_descs(tk_batch* b, const tk_tree* const* trees, const int64_t* q_counts, const int32_t* ks) {
    std::vector<Desc> h(b->n_clouds);
    int bin_base = 0;
    for (int c = 0; c < b->n_clouds; ++c) {
        const tk_tree* t = trees[c];
        Desc& d = h[c];
        fill_desc<T>(d, t);
        d.out_off = b->out_off[c];
        d.levels = t->levels;
        d.k = ks[c];
        const int B = batch_bin_levels(t->levels, std::max<int64_t>(q_counts[c], 1));
        d.bins = 1 << B;
        d.bin_base = bin_base;
        bin_base += d.bins;
    }
    b->total_bins = bin_base;
    cudaError_t e = cudaMalloc(&b->d_desc, sizeof(Desc) * h.size());
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&b->d_prefix), sizeof(long long) * b->q_prefix.size());
    if (e != cudaSuccess) return fail(TK_ENOMEM, std::string("batch allocation: ") + cudaGetErrorString(e));
    e = cudaMemcpy(b->d_desc, h.data(), sizeof(Desc) * h.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(b->d_prefix, b->q_prefix.data(), sizeof(long long) * b->q_prefix.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return fail(TK_ECUDA, std::string("batch upload: ") + cudaGetErrorString(e));
    return TK_OK;
}

template <typename T, int D>
int run_batch(const tk_batch* b, const T* q, T* dists, int32_t* idx, int G, int boxes, char* ws, cudaStream_t s) {
    const BatchWs w = batch_ws(b);
    BatchArgs<T> a;
    a.desc = static_cast<const CloudDesc<T>*>(b->d_desc);
    a.q_prefix = b->d_prefix;
    a.n_clouds = b->n_clouds;
    a.q = q;
    a.total = int(b->total_q);
    a.out_d = dists;
    a.out_i = idx;
    a.work = reinterpret_cast<int*>(ws + w.counter);
    a.use_boxes = boxes;
    int* counts = reinterpret_cast<int*>(ws + w.counts);
    int* bin_of = reinterpret_cast<int*>(ws + w.bin_of);
    int* pos_of = reinterpret_cast<int*>(ws + w.pos_of);
    int* order = reinterpret_cast<int*>(ws + w.order);
    a.order = order;
    cudaError_t e = cudaMemsetAsync(counts, 0, sizeof(int) * size_t(b->total_bins), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(a.work, 0, sizeof(int), s);
    if (e != cudaSuccess) return fail(TK_ECUDA, std::string("memset: ") + cudaGetErrorString(e));
    const int nb = (a.total + 255) / 256;
    k_batch_bin_count<T, D><<<nb, 256, 0, s>>>(a, counts, bin_of, pos_of);
    e = exclusive_scan(counts, b->total_bins, ws + w.scan, s);
    if (e != cudaSuccess) return fail(TK_ECUDA, std::string("batch scan: ") + cudaGetErrorString(e));
    k_batch_scatter<<<nb, 256, 0, s>>>(a.total, bin_of, pos_of, counts, order);
    const void* kfn = G == 1 ? reinterpret_cast<const void*>(&k_batch_query<T, D, 1>)
                             : reinterpret_cast<const void*>(&k_batch_query<T, D, 8>);
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kfn, 256, 0) != cudaSuccess || per_sm <= 0) per_sm = 1;
    int sms = 1;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device);
    const int need = (a.total + 256 / G - 1) / (256 / G);
    const int grid = std::max(1, std::min(need, per_sm * sms));
    if (G == 1) k_batch_query<T, D, 1><<<grid, 256, 0, s>>>(a);
    else k_batch_query<T, D, 8><<<grid, 256, 0, s>>>(a);
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(TK_ECUDA, std::string("batch launch: ") + cudaGetErrorString(e));
    return TK_OK;
}

template <typename T>
int run_batch_wide(const tk_batch* b, const T* q, T* dists, int32_t* idx, int G, char* ws, cudaStream_t s) {
    const BatchWs w = batch_ws(b);
    WideBatchArgs<T> a;
    a.desc = static_cast<const WideCloudDesc<T>*>(b->d_desc);
    a.q_prefix = b->d_prefix;
    a.n_clouds = b->n_clouds;
    a.dims = b->dims;
    a.q = q;
    a.total = int(b->total_q);
    a.out_d = dists;
    a.out_i = idx;
    a.work = reinterpret_cast<int*>(ws + w.counter);
    int* counts = reinterpret_cast<int*>(ws + w.counts);
    int* bin_of = reinterpret_cast<int*>(ws + w.bin_of);
    int* pos_of = reinterpret_cast<int*>(ws + w.pos_of);
    int* order = reinterpret_cast<int*>(ws + w.order);
    a.order = order;
    cudaError_t e = cudaMemsetAsync(counts, 0, sizeof(int) * size_t(b->total_bins), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(a.work, 0, sizeof(int), s);
    if (e != cudaSuccess) return fail(TK_ECUDA, std::string("memset: ") + cudaGetErrorString(e));
    const int nb = (a.total + 255) / 256;
    batch_wide_bin_launch<T>(a, counts, bin_of, pos_of, s);
    e = exclusive_scan(counts, b->total_bins, ws + w.scan, s);
    if (e != cudaSuccess) return fail(TK_ECUDA, std::string("batch scan: ") + cudaGetErrorString(e));
    k_batch_scatter<<<nb, 256, 0, s>>>(a.total, bin_of, pos_of, counts, order);
    const int W = record_width(b->dims);
    const void* kfn = batch_wide_kernel<T>(W, G);
    if (!kfn) return fail(TK_EUNSUPPORTED, "no batched kernel for this record width / lanes");
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kfn, 256, 0) != cudaSuccess || per_sm <= 0) per_sm = 1;
    int sms = 1;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device);
    const int need = (a.total + 256 / G - 1) / (256 / G);
    const int grid = std::max(1, std::min(need, per_sm * sms));
    return batch_wide_launch<T>(a, W, G, grid, s);
}

}  // namespace

extern "C" {

int tk_batch_create(const tk_tree* const* trees, int n_trees, const int64_t* q_counts, const int32_t* ks,
                    tk_batch** out) {
    clear_error();
    if (!out) return fail(TK_EINVAL, "out is null");
    *out = nullptr;
    if (!trees || n_trees < 1 || !q_counts || !ks) return fail(TK_EINVAL, "empty batch");
    tk_batch* b = new (std::nothrow) tk_batch();
    if (!b) return fail(TK_ENOMEM, "host allocation failed");
    b->n_clouds = n_trees;
    b->dtype = trees[0] ? trees[0]->dtype : TK_F32;
    b->dims = trees[0] ? trees[0]->dims : 0;
    b->device = trees[0] ? trees[0]->device : 0;
    b->q_prefix.assign(n_trees + 1, 0);
    b->out_off.assign(n_trees, 0);
    long long out_elems = 0;
    for (int c = 0; c < n_trees; ++c) {
        const tk_tree* t = trees[c];
        if (!t || !t->d_pts || t->dtype != b->dtype || t->dims != b->dims || t->device != b->device) {
            delete b;
            return fail(TK_EINVAL, "batch trees must be device trees of one dtype, dims and device");
        }
        if (q_counts[c] < 0 || ks[c] < 1 || ks[c] > kMaxK || ks[c] > t->n) {
            delete b;
            return fail(TK_EINVAL, "cloud " + std::to_string(c) + ": need 0 <= queries and 1 <= k <= min(n, 128)");
        }
        b->q_prefix[c + 1] = b->q_prefix[c] + q_counts[c];
        b->out_off[c] = out_elems;
        out_elems += q_counts[c] * int64_t(ks[c]);
        b->max_k = std::max<int>(b->max_k, ks[c]);
    }
    b->total_q = b->q_prefix[n_trees];
    b->total_out = out_elems;
    if (b->total_q >= (1LL << 31) || out_elems >= (1LL << 40)) {
        delete b;
        return fail(TK_EINVAL, "batch too large");
    }
    int prev = -1;
    cudaGetDevice(&prev);
    cudaSetDevice(b->device);
    int rc;
    if (b->dims <= 3)
        rc = b->dtype == TK_F32 ? upload_descs<float, CloudDesc<float>>(b, trees, q_counts, ks)
                                : upload_descs<double, CloudDesc<double>>(b, trees, q_counts, ks);
    else
        rc = b->dtype == TK_F32 ? upload_descs<float, WideCloudDesc<float>>(b, trees, q_counts, ks)
                                : upload_descs<double, WideCloudDesc<double>>(b, trees, q_counts, ks);
    if (prev >= 0) cudaSetDevice(prev);
    if (rc != TK_OK) {
        if (b->d_desc) cudaFree(b->d_desc);
        if (b->d_prefix) cudaFree(b->d_prefix);
        delete b;
        return rc;
    }
    *out = b;
    return TK_OK;
}

int tk_batch_destroy(tk_batch* b) {
    if (!b) return TK_OK;
    if (b->d_desc) cudaFree(b->d_desc);
    if (b->d_prefix) cudaFree(b->d_prefix);
    delete b;
    return TK_OK;
}

size_t tk_batch_workspace_size(const tk_batch* b) { return b ? batch_ws(b).total : 0; }

int64_t tk_batch_output_size(const tk_batch* b) { return b ? b->total_out : 0; }

int tk_batch_query(const tk_batch* b, const void* q, void* dists, int32_t* idx, int threads_per_query,
                   int prune_boxes, void* workspace, size_t workspace_bytes, void* stream) {
    clear_error();
    if (!b) return fail(TK_EINVAL, "batch is null");
    if (b->total_q == 0) return TK_OK;
    if (!q || !dists || !idx) return fail(TK_EINVAL, "null pointer");
    if (!workspace || workspace_bytes < batch_ws(b).total) return fail(TK_EWORKSPACE, "workspace too small");
    if (ws_misaligned(workspace)) return fail(TK_EINVAL, "workspace must be 256-byte aligned");
    int G = threads_per_query;
    if (G <= 0) G = b->max_k <= 16 ? 1 : 8;
    if (G != 1 && G != 8 && G != 32) return fail(TK_EINVAL, "batched queries run 1, 8 or 32 lanes per query");
    if (G == 1 && b->max_k > 16) return fail(TK_EINVAL, "1 lane per query supports k <= 16 in a batch");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    char* ws = static_cast<char*>(workspace);
    if (b->dims > 3) {  // trees of 4-8 dims: 1 or 32 lanes per query (the wide kernels' shapes)
        const int Gw = G == 1 ? 1 : 32;
        if (b->dtype == TK_F32)
            return run_batch_wide<float>(b, static_cast<const float*>(q), static_cast<float*>(dists), idx, Gw, ws, s);
        return run_batch_wide<double>(b, static_cast<const double*>(q), static_cast<double*>(dists), idx, Gw, ws, s);
    }
    if (G == 32) G = 8;  // trees of 1-3 dims: 8-lane groups serve every k <= 128
    if (b->dtype == TK_F32) {
        switch (b->dims) {
            case 1: return run_batch<float, 1>(b, static_cast<const float*>(q), static_cast<float*>(dists), idx, G, prune_boxes != 0, ws, s);
            case 2: return run_batch<float, 2>(b, static_cast<const float*>(q), static_cast<float*>(dists), idx, G, prune_boxes != 0, ws, s);
            default: return run_batch<float, 3>(b, static_cast<const float*>(q), static_cast<float*>(dists), idx, G, prune_boxes != 0, ws, s);
        }
    }
    switch (b->dims) {
        case 1: return run_batch<double, 1>(b, static_cast<const double*>(q), static_cast<double*>(dists), idx, G, prune_boxes != 0, ws, s);
        case 2: return run_batch<double, 2>(b, static_cast<const double*>(q), static_cast<double*>(dists), idx, G, prune_boxes != 0, ws, s);
        default: return run_batch<double, 3>(b, static_cast<const double*>(q), static_cast<double*>(dists), idx, G, prune_boxes != 0, ws, s);
    }
}

}  // extern "C"
