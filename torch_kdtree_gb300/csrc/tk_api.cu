// C ABI of the engine (include/tk_knn.h): error reporting, tree life cycle,
// and the KD query pipeline (query binning + KD kernel launch).
#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "kd_query.cuh"
#include "kd_wide.cuh"
#include "sort.cuh"
#include "tk_internal.h"

namespace tk {

namespace {
thread_local std::string g_err;

struct DeviceGuard {
    int prev = -1;
    bool changed = false;
    explicit DeviceGuard(int dev) {
        if (cudaGetDevice(&prev) == cudaSuccess && prev != dev) {
            changed = cudaSetDevice(dev) == cudaSuccess;
        }
    }
    ~DeviceGuard() {
        if (changed) cudaSetDevice(prev);
    }
};

int sm_count(int dev) {
    static std::mutex mu;
    static std::vector<int> cache;
    std::lock_guard<std::mutex> lock(mu);
    if (dev < 0) dev = 0;
    if ((int)cache.size() <= dev) cache.resize(dev + 1, 0);
    if (cache[dev] == 0) {
        int v = 0;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) v = 1;
        cache[dev] = v;
    }
    return cache[dev];
}

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }
}  // namespace

int fail(int status, const std::string& msg) {
    g_err = msg;
    return status;
}
void clear_error() { g_err.clear(); }

// ------------------------------------------------------------ binning --

// Queries in cell order; with `classes`, each one's cost class (bits 16-23
// of bin_of, see k_bin_count) goes to the same position.
__global__ void k_bin_scatter(int nq, const int* bin_of, const int* pos_of, const int* offsets, int* order,
                              uint32_t* classes) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nq) return;
    const int b = bin_of[i];
    const int dst = offsets[b & 0xFFFF] + pos_of[i];
    order[dst] = i;
    if (classes) classes[dst] = uint32_t(b) >> 16;
}

// ------------------------------------------------------------ planning --

namespace {

int bin_levels(int L, int64_t nq) {
    int lg = 0;
    while ((int64_t(1) << (lg + 1)) <= nq) ++lg;
    return std::max(1, std::min({L, kMaxBinLevels, lg - 4}));
}

// Query workspace: work counter, cell counts, per query its cell, rank,
// place in cell order and cost class, then the scratch of the cell-count
// scan or (used after it) of the cost-class pass.  After the cell scatter
// bin_of and pos_of are free again and receive the class pass's output.
struct WsLayout {
    size_t counter = 0, counts = 0, bin_of = 0, pos_of = 0, order = 0, classes = 0, scan = 0, total = 0;
};

WsLayout ws_layout(int L, int64_t nq) {
    WsLayout w;
    const int B = bin_levels(L, nq);
    size_t o = 0;
    w.counter = o;
    o += 256;
    w.counts = o;
    o += align_up(sizeof(int) * (size_t(1) << B), 256);
    w.bin_of = o;
    o += align_up(sizeof(int) * size_t(nq), 256);
    w.pos_of = o;
    o += align_up(sizeof(int) * size_t(nq), 256);
    w.order = o;
    o += align_up(sizeof(int) * size_t(nq), 256);
    w.classes = o;
    o += align_up(sizeof(uint32_t) * size_t(nq), 256);
    w.scan = o;
    o += std::max(scan_workspace_bytes(int64_t(1) << B), sort_pass8_workspace_bytes(nq));
    w.total = o;
    return w;
}

bool gr_available(int dtype, int dims, int G, int R) {
    const bool full = dtype == TK_F32 && dims == 3;
    if (!full && !(G == 1 || G == 4 || G == 32)) return false;
    if (R < 1 || R > 16 || (R & (R - 1))) return false;
    if (G * R > 128) return false;
    if (G == 16 && R > 8) return false;
    if (G == 32 && R > 4) return false;
    return true;
}

// Lanes per query when the caller leaves it to the library (measured on the
// large workloads): one lane per query up to ~192 points per leaf and k <= 16
// (its list fits one lane's registers); 32 lanes for larger leaves or k > 16,
// which spread both the leaf scan and the list (k = 100: 21 ms on 32 lanes,
// 35 ms on 8).  Calls with fewer queries than half a wave (SMs x 512) spread
// each query over 4, 8, 16 or 32 lanes until queries x lanes fill a wave of
// SMs x 1024 threads: 10,000 queries on one lane each fill 40 of 152 SMs and
// ran 1.6x slower than on 16 lanes; at 32,768 (65,536) queries 8 (4) lanes
// beat one by 25% (6%), while at 131,072 one lane beat two by 20%.  Two-lane
// groups were the slowest shape in every measurement and are skipped.  Trees
// of 4-8 dimensions (1M refs x 262k queries N(0,1), depth 12-13): one lane
// only for k = 1 up to 6 dimensions (d=4: 0.40 vs 0.70 ms), 32 otherwise
// (d=8, k=16: 21.4 vs 38.3 ms; d=8, k=1: 8.5 vs 9.1 ms).
int auto_lanes(const tk_tree* t, int64_t nq, int k) {
    const double avg_leaf = double(t->n) / double(int64_t(1) << t->levels);
    int g = (k > 16 || avg_leaf > 192) ? 32 : 1;
    if (t->dims > 3) g = (k == 1 && t->dims <= 6) ? 1 : 32;
    const int64_t wave = int64_t(sm_count(t->device)) * 1024;  // resident threads
    if (g == 1 && 2 * nq < wave) {
        g = 4;
        while (g < 32 && nq * g < wave) g <<= 1;
    }
    return g;
}

int pow2_ceil(int v) {
    int p = 1;
    while (p < v) p <<= 1;
    return p;
}

// Zero the work counter and, when binning is on, order the queries by the
// tree cell at depth B they fall into (count, exclusive scan, scatter).
// `count(B, counts, bin_of, pos_of)` launches the counting kernel.  With
// `classes` (the counting kernel wrote cost classes), one stable radix pass
// then puts the costliest class first, cell order kept within a class: the
// persistent search takes its work in that order, so the expensive queries
// do not end up in the last chunks (the launch's tail), and a warp's 32
// queries have similar costs (a warp runs as long as its slowest lane).
template <typename CountFn>
int prepare_order(const tk_tree* t, int nq, const tk_query_opts& o, char* ws, cudaStream_t s, int** counter,
                  const int32_t** order, bool classes, CountFn count) {
    const int L = t->levels;
    const WsLayout w = ws_layout(L, nq);
    *counter = reinterpret_cast<int*>(ws + w.counter);
    *order = nullptr;
    // Automatic binning from one wave of queries (SMs x 1024) on: below that
    // each thread takes about one query, the cell order gains little leaf
    // sharing, and grouping a region's expensive queries into the same warps
    // lengthens the slowest warp, which then sets the launch time (131,072
    // queries: 1.33 ms binned vs 1.17 ms in input order; 1,048,576: 3.53 vs
    // 5.84 ms on the cube-and-sphere workload).
    const bool bin = o.bin_queries == 1 ||
                     (o.bin_queries < 0 && L >= 2 && int64_t(nq) >= int64_t(sm_count(t->device)) * 1024);
    cudaError_t e;
    if (bin) {
        const int B = bin_levels(L, nq);
        const int nbins = 1 << B;
        int* counts = reinterpret_cast<int*>(ws + w.counts);
        int* bin_of = reinterpret_cast<int*>(ws + w.bin_of);
        int* pos_of = reinterpret_cast<int*>(ws + w.pos_of);
        int* ord = reinterpret_cast<int*>(ws + w.order);
        e = cudaMemsetAsync(counts, 0, sizeof(int) * nbins, s);
        if (e == cudaSuccess) e = cudaMemsetAsync(*counter, 0, sizeof(int), s);
        if (e != cudaSuccess) return fail(TK_ECUDA, std::string("memset: ") + cudaGetErrorString(e));
        count(B, counts, bin_of, pos_of);
        e = exclusive_scan(counts, nbins, ws + w.scan, s);
        if (e != cudaSuccess) return fail(TK_ECUDA, std::string("bin scan: ") + cudaGetErrorString(e));
        uint32_t* cls = classes ? reinterpret_cast<uint32_t*>(ws + w.classes) : nullptr;
        k_bin_scatter<<<(nq + 255) / 256, 256, 0, s>>>(nq, bin_of, pos_of, counts, ord, cls);
        e = cudaGetLastError();
        if (e != cudaSuccess) return fail(TK_ECUDA, std::string("binning launch: ") + cudaGetErrorString(e));
        *order = ord;
        if (classes) {
            uint32_t* final_order = reinterpret_cast<uint32_t*>(pos_of);
            e = sort_pass8(cls, reinterpret_cast<const uint32_t*>(ord), reinterpret_cast<uint32_t*>(bin_of),
                           final_order, nq, ws + w.scan, w.total - w.scan, s);
            if (e != cudaSuccess) return fail(TK_ECUDA, std::string("cost-class pass: ") + cudaGetErrorString(e));
            *order = reinterpret_cast<const int32_t*>(final_order);
        }
    } else {
        e = cudaMemsetAsync(*counter, 0, sizeof(int), s);
        if (e != cudaSuccess) return fail(TK_ECUDA, std::string("memset: ") + cudaGetErrorString(e));
    }
    return TK_OK;
}

template <typename T, int D>
int run_query(const tk_tree* t, const T* q, int nq, int k, T* dists, int32_t* idx, const tk_query_opts& o,
              char* ws, cudaStream_t s) {
    if (o.traversal < 0 || o.traversal > 2) return fail(TK_EINVAL, "traversal must be 0, 1 or 2");
    // warp packets: one lane per query, the warp walks the tree together
    const bool packet = o.traversal == 2 && k <= 16 && t->d_boxes != nullptr;
    // lanes per query and registers per lane
    int G = 1, R = pow2_ceil(k);
    if (!packet) {
        G = o.threads_per_query > 0 ? o.threads_per_query : auto_lanes(t, nq, k);
        if (G != 1 && G != 2 && G != 4 && G != 8 && G != 16 && G != 32)
            return fail(TK_EINVAL, "threads_per_query must be 1, 2, 4, 8, 16 or 32");
        G = std::max(G, pow2_ceil((k + 15) / 16));
        R = pow2_ceil((k + G - 1) / G);
        while (!gr_available(t->dtype, D, G, R) && G < 32) {
            G <<= 1;
            R = pow2_ceil((k + G - 1) / G);
        }
        if (!gr_available(t->dtype, D, G, R)) return fail(TK_EUNSUPPORTED, "no kernel shape for this k");
    }

    const int L = t->levels;
    // 10 levels (4 KiB for float): deeper staging measured no faster, and at
    // 12 levels (16 KiB) only 3 of the 4 blocks the registers allow stayed
    // resident per SM on the one-lane shape.
    int S = o.smem_levels >= 0 ? o.smem_levels : 10;
    S = std::max(0, std::min({S, L, sizeof(T) == 4 ? 15 : 14}));  // <= 128 KiB of shared memory
    const int block = kKdBlock;
    const size_t smem = kd_smem_bytes<T>(S);
    const void* kfn = packet ? kd_packet_kernel<T, D>(R) : kd_query_kernel<T, D>(G, R);
    if (!kfn) return fail(TK_EUNSUPPORTED, "KD query kernel shape not compiled");
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
        if (e != cudaSuccess) return fail(TK_ECUDA, std::string("smem attribute: ") + cudaGetErrorString(e));
    }
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kfn, block, smem);
    if (e != cudaSuccess || per_sm <= 0) per_sm = 1;
    if (o.blocks_per_sm > 0) per_sm = std::min(per_sm, int(o.blocks_per_sm));
    const int groups_per_block = block / G;
    const int need = (nq + groups_per_block - 1) / groups_per_block;
    const int grid = std::max(1, std::min(need, per_sm * sm_count(t->device)));

    int* counter = nullptr;
    const int32_t* order = nullptr;
    const PointRec<T>* boxes = static_cast<const PointRec<T>*>(t->d_boxes);
    int rc0 = prepare_order(t, nq, o, ws, s, &counter, &order, true, [&](int B, int* counts, int* bin_of, int* pos_of) {
        bin_count_launch<T, D>(q, nq, static_cast<const T*>(t->d_medians), B, L, boxes, counts, bin_of, pos_of, s);
    });
    if (rc0 != TK_OK) return rc0;

    KdArgs<T> a;
    a.pts = static_cast<const PointRec<T>*>(t->d_pts);
    a.medians = static_cast<const T*>(t->d_medians);
    a.leaf_off = t->d_leaf_off;
    a.boxes = static_cast<const PointRec<T>*>(t->d_boxes);  // the 1-3-D searches always prune with node boxes
    a.levels = L;
    a.smem_levels = S;
    a.q = q;
    a.nq = nq;
    a.k = k;
    a.order = order;
    a.out_d = dists;
    a.out_i = idx;
    a.work = counter;
    KdLaunch l{G, R, block, grid, smem};
    if (o.kernel_start_event) cudaEventRecord(static_cast<cudaEvent_t>(o.kernel_start_event), s);
    const int rc = packet ? kd_packet_launch<T, D>(a, l, s) : kd_query_launch<T, D>(a, l, s);
    if (rc == TK_OK && o.kernel_stop_event) cudaEventRecord(static_cast<cudaEvent_t>(o.kernel_stop_event), s);
    return rc;
}

// KD query of a tree of 4-8 dimensions (kd_wide.cuh): one lane per query
// for k <= 16 when the automatic / requested shape is one lane, else a
// 32-lane group per query; binning and options as run_query (warp packets do
// not apply: traversal 2 runs as 1).
template <typename T>
int run_query_wide(const tk_tree* t, const T* q, int nq, int k, T* dists, int32_t* idx, const tk_query_opts& o,
                   char* ws, cudaStream_t s) {
    if (o.traversal < 0 || o.traversal > 2) return fail(TK_EINVAL, "traversal must be 0, 1 or 2");
    int G = o.threads_per_query > 0 ? o.threads_per_query : auto_lanes(t, nq, k);
    if (G != 1 && G != 2 && G != 4 && G != 8 && G != 16 && G != 32)
        return fail(TK_EINVAL, "threads_per_query must be 1, 2, 4, 8, 16 or 32");
    if (G != 1 || k > 16) G = 32;  // kernels of wide trees: 1 (k <= 16) or 32 lanes per query
    const int R = pow2_ceil((k + G - 1) / G);
    const int W = record_width(t->dims);
    const int L = t->levels;
    int S = o.smem_levels >= 0 ? o.smem_levels : 10;
    S = std::max(0, std::min({S, L, sizeof(T) == 4 ? 15 : 14}));
    const int block = kKdBlock;
    const size_t smem = kd_smem_bytes<T>(S);
    const void* kfn = kd_wide_kernel<T>(W, G, R);
    if (!kfn) return fail(TK_EUNSUPPORTED, "KD query kernel shape not compiled");
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
        if (e != cudaSuccess) return fail(TK_ECUDA, std::string("smem attribute: ") + cudaGetErrorString(e));
    }
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kfn, block, smem);
    if (e != cudaSuccess || per_sm <= 0) per_sm = 1;
    if (o.blocks_per_sm > 0) per_sm = std::min(per_sm, int(o.blocks_per_sm));
    const int groups_per_block = block / G;
    const int need = (nq + groups_per_block - 1) / groups_per_block;
    const int grid = std::max(1, std::min(need, per_sm * sm_count(t->device)));

    int* counter = nullptr;
    const int32_t* order = nullptr;
    const int rc0 = prepare_order(t, nq, o, ws, s, &counter, &order, true, [&](int B, int* counts, int* bin_of, int* pos_of) {
        bin_count_wide_launch<T>(q, nq, t->dims, static_cast<const T*>(t->d_medians), B, L,
                                 static_cast<const T*>(t->d_boxes), W, counts, bin_of, pos_of, s);
    });
    if (rc0 != TK_OK) return rc0;

    KdWideArgs<T> a;
    a.pts = static_cast<const T*>(t->d_pts);
    a.perm = t->d_perm;
    a.medians = static_cast<const T*>(t->d_medians);
    a.leaf_off = t->d_leaf_off;
    a.boxes = o.prune_boxes == 0 ? nullptr : static_cast<const T*>(t->d_boxes);
    a.levels = L;
    a.smem_levels = S;
    a.dims = t->dims;
    a.q = q;
    a.nq = nq;
    a.k = k;
    a.order = order;
    a.out_d = dists;
    a.out_i = idx;
    a.work = counter;
    if (o.kernel_start_event) cudaEventRecord(static_cast<cudaEvent_t>(o.kernel_start_event), s);
    const int rc = kd_wide_launch<T>(a, W, G, R, grid, block, smem, s);
    if (rc == TK_OK && o.kernel_stop_event) cudaEventRecord(static_cast<cudaEvent_t>(o.kernel_stop_event), s);
    return rc;
}

// The 4th slot of a point record holds an index as raw bits: the original
// index of a point, or the begin / end offset of a leaf in its box records.
template <typename T>
void set_rec_index(PointRec<T>& r, uint32_t v) {
    if (sizeof(T) == 4) {
        std::memcpy(&r.w, &v, 4);
    } else {
        const uint64_t bits = v;
        std::memcpy(&r.w, &bits, 8);
    }
}

// Device image of a tree of 4-8 dimensions: zero-padded coordinate rows of
// record_width(dims), the original indices, and node boxes as lo / hi rows.
template <typename T>
int upload_wide(tk_tree* t, const HostTree<T>& h) {
    const int64_t n = h.n;
    const int W = record_width(h.dims);
    std::vector<T> rows(static_cast<size_t>(n) * W, T(0));
    for (int64_t i = 0; i < n; ++i)
        for (int d = 0; d < h.dims; ++d) rows[size_t(i) * W + d] = h.structured[i * h.dims + d];
    const size_t nnodes = h.box_lo.size() / W;
    std::vector<T> boxes(2 * nnodes * W);
    for (size_t i = 0; i < nnodes; ++i)
        for (int c = 0; c < W; ++c) {
            boxes[(2 * i) * W + c] = h.box_lo[i * W + c];
            boxes[(2 * i + 1) * W + c] = h.box_hi[i * W + c];
        }
    const size_t b_pts = sizeof(T) * rows.size();
    const size_t b_perm = sizeof(int32_t) * size_t(n);
    const size_t b_med = sizeof(T) * h.medians.size();
    const size_t b_off = sizeof(int32_t) * h.leaf_off.size();
    const size_t b_box = sizeof(T) * boxes.size();
    cudaError_t e = cudaMalloc(&t->d_pts, b_pts);
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&t->d_perm), b_perm);
    if (e == cudaSuccess) e = cudaMalloc(&t->d_medians, std::max<size_t>(b_med, sizeof(T)));
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&t->d_leaf_off), b_off);
    if (e == cudaSuccess) e = cudaMalloc(&t->d_boxes, b_box);
    if (e != cudaSuccess) return fail(TK_ENOMEM, std::string("device allocation: ") + cudaGetErrorString(e));
    e = cudaMemcpy(t->d_pts, rows.data(), b_pts, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(t->d_perm, h.perm.data(), b_perm, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && b_med) e = cudaMemcpy(t->d_medians, h.medians.data(), b_med, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(t->d_leaf_off, h.leaf_off.data(), b_off, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(t->d_boxes, boxes.data(), b_box, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return fail(TK_ECUDA, std::string("tree upload: ") + cudaGetErrorString(e));
    t->device_bytes = int64_t(b_pts + b_perm + b_med + b_off + b_box);
    return TK_OK;
}

template <typename T>
int upload_tree(tk_tree* t, const HostTree<T>& h) {
    if (h.dims > 3) return upload_wide(t, h);
    const int64_t n = h.n;
    std::vector<PointRec<T>> recs(static_cast<size_t>(n));
    for (int64_t i = 0; i < n; ++i) {
        T c[3] = {T(0), T(0), T(0)};
        for (int d = 0; d < h.dims; ++d) c[d] = h.structured[i * h.dims + d];
        recs[i].x = c[0];
        recs[i].y = c[1];
        recs[i].z = c[2];
        set_rec_index(recs[i], uint32_t(h.perm[i]));
    }
    const size_t b_pts = sizeof(PointRec<T>) * size_t(n);
    const size_t b_med = sizeof(T) * h.medians.size();
    const size_t b_off = sizeof(int32_t) * h.leaf_off.size();
    const size_t nnodes = h.box_lo.size() / 3;
    std::vector<PointRec<T>> boxes(2 * nnodes);
    const size_t first_leaf = nnodes / 2;  // nnodes = 2^(L+1) - 1
    for (size_t i = 0; i < nnodes; ++i) {
        boxes[2 * i] = PointRec<T>{h.box_lo[3 * i], h.box_lo[3 * i + 1], h.box_lo[3 * i + 2], T(0)};
        boxes[2 * i + 1] = PointRec<T>{h.box_hi[3 * i], h.box_hi[3 * i + 1], h.box_hi[3 * i + 2], T(0)};
        if (i >= first_leaf) {  // a leaf's box also carries its point range [begin, end)
            set_rec_index(boxes[2 * i], uint32_t(h.leaf_off[i - first_leaf]));
            set_rec_index(boxes[2 * i + 1], uint32_t(h.leaf_off[i - first_leaf + 1]));
        }
    }
    const size_t b_box = sizeof(PointRec<T>) * boxes.size();
    cudaError_t e = cudaMalloc(&t->d_pts, b_pts);
    if (e == cudaSuccess) e = cudaMalloc(&t->d_medians, std::max<size_t>(b_med, sizeof(T)));
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&t->d_leaf_off), b_off);
    if (e == cudaSuccess) e = cudaMalloc(&t->d_boxes, b_box);
    if (e != cudaSuccess) return fail(TK_ENOMEM, std::string("device allocation: ") + cudaGetErrorString(e));
    e = cudaMemcpy(t->d_pts, recs.data(), b_pts, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && b_med) e = cudaMemcpy(t->d_medians, h.medians.data(), b_med, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(t->d_leaf_off, h.leaf_off.data(), b_off, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(t->d_boxes, boxes.data(), b_box, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return fail(TK_ECUDA, std::string("tree upload: ") + cudaGetErrorString(e));
    t->device_bytes = int64_t(b_pts + b_med + b_off + b_box);
    return TK_OK;
}

void free_tree_device(tk_tree* t) {
    if (t->d_pts) cudaFree(t->d_pts);
    if (t->d_perm) cudaFree(t->d_perm);
    t->d_perm = nullptr;
    if (t->d_medians) cudaFree(t->d_medians);
    if (t->d_leaf_off) cudaFree(t->d_leaf_off);
    if (t->d_boxes) cudaFree(t->d_boxes);
    t->d_pts = t->d_medians = t->d_boxes = nullptr;
    t->d_leaf_off = nullptr;
}

// Layout of a tree built on the GPU: points (T[n*dims]) and / or the
// permutation (int32[n]) copied out of its device point records.
template <typename T>
int device_layout(const tk_tree* t, T* points, int32_t* perm) {
    DeviceGuard g(t->device);
    if (t->dims > 3) {  // coordinate rows + separate indices
        const int W = record_width(t->dims);
        cudaError_t e = cudaSuccess;
        if (points) {
            std::vector<T> rows(static_cast<size_t>(t->n) * W);
            e = cudaMemcpy(rows.data(), t->d_pts, sizeof(T) * rows.size(), cudaMemcpyDeviceToHost);
            if (e == cudaSuccess)
                for (int64_t i = 0; i < t->n; ++i)
                    for (int d = 0; d < t->dims; ++d) points[i * t->dims + d] = rows[size_t(i) * W + d];
        }
        if (e == cudaSuccess && perm)
            e = cudaMemcpy(perm, t->d_perm, sizeof(int32_t) * size_t(t->n), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return fail(TK_ECUDA, std::string("layout copy: ") + cudaGetErrorString(e));
        return TK_OK;
    }
    std::vector<PointRec<T>> recs(static_cast<size_t>(t->n));
    const cudaError_t e = cudaMemcpy(recs.data(), t->d_pts, sizeof(PointRec<T>) * recs.size(), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return fail(TK_ECUDA, std::string("layout copy: ") + cudaGetErrorString(e));
    for (int64_t i = 0; i < t->n; ++i) {
        const PointRec<T>& r = recs[size_t(i)];
        if (points) {
            const T c[3] = {r.x, r.y, r.z};
            for (int d = 0; d < t->dims; ++d) points[i * t->dims + d] = c[d];
        }
        if (perm) {
            if (sizeof(T) == 4) {
                uint32_t bits;
                std::memcpy(&bits, &r.w, 4);
                perm[i] = int32_t(bits);
            } else {
                uint64_t bits;
                std::memcpy(&bits, &r.w, 8);
                perm[i] = int32_t(bits);
            }
        }
    }
    return TK_OK;
}

}  // namespace
}  // namespace tk

using namespace tk;

extern "C" {

const char* tk_last_error(void) { return g_err.c_str(); }

int tk_version(void) { return 1; }

int tk_cuda_available(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n > 0 ? 1 : 0;
}

int tk_tree_create(const void* host_points, int64_t n, int dims, int dtype, int levels, int device,
                   int n_threads, tk_tree** out) {
    clear_error();
    if (!out) return fail(TK_EINVAL, "out is null");
    *out = nullptr;
    if (dtype != TK_F32 && dtype != TK_F64) return fail(TK_EINVAL, "dtype must be TK_F32 or TK_F64");
    tk_tree* t = new (std::nothrow) tk_tree();
    if (!t) return fail(TK_ENOMEM, "host allocation failed");
    t->dtype = dtype;
    t->dims = dims;
    t->levels = levels;
    t->device = device;
    t->n = n;
    int rc = dtype == TK_F32
                 ? build_host_tree<float>(static_cast<const float*>(host_points), n, dims, levels, n_threads, t->h32)
                 : build_host_tree<double>(static_cast<const double*>(host_points), n, dims, levels, n_threads,
                                           t->h64);
    if (rc != TK_OK) {
        delete t;
        return rc;
    }
    if (device < 0) {  // host-only tree: layout getters work, queries are refused
        *out = t;
        return TK_OK;
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device >= ndev) {
        cudaGetLastError();
        delete t;
        return fail(TK_EINVAL, "CUDA device " + std::to_string(device) + " is not available");
    }
    {
        DeviceGuard g(device);
        rc = dtype == TK_F32 ? upload_tree<float>(t, t->h32) : upload_tree<double>(t, t->h64);
    }
    if (rc != TK_OK) {
        DeviceGuard g(device);
        free_tree_device(t);
        delete t;
        return rc;
    }
    *out = t;
    return TK_OK;
}

int tk_tree_create_from_layout(const void* structured_points, const int32_t* perm, const void* medians,
                               const int32_t* leaf_offsets, int64_t n, int dims, int dtype, int levels, int device,
                               tk_tree** out) {
    clear_error();
    if (!out) return fail(TK_EINVAL, "out is null");
    *out = nullptr;
    if (dtype != TK_F32 && dtype != TK_F64) return fail(TK_EINVAL, "dtype must be TK_F32 or TK_F64");
    tk_tree* t = new (std::nothrow) tk_tree();
    if (!t) return fail(TK_ENOMEM, "host allocation failed");
    t->dtype = dtype;
    t->dims = dims;
    t->levels = levels;
    t->device = device;
    t->n = n;
    int rc = dtype == TK_F32
                 ? tree_from_layout<float>(static_cast<const float*>(structured_points), perm,
                                           static_cast<const float*>(medians), leaf_offsets, n, dims, levels, t->h32)
                 : tree_from_layout<double>(static_cast<const double*>(structured_points), perm,
                                            static_cast<const double*>(medians), leaf_offsets, n, dims, levels, t->h64);
    if (rc == TK_OK && device >= 0) {
        int ndev = 0;
        if (cudaGetDeviceCount(&ndev) != cudaSuccess || device >= ndev) {
            cudaGetLastError();
            rc = fail(TK_EINVAL, "CUDA device " + std::to_string(device) + " is not available");
        } else {
            DeviceGuard g(device);
            rc = dtype == TK_F32 ? upload_tree<float>(t, t->h32) : upload_tree<double>(t, t->h64);
            if (rc != TK_OK) free_tree_device(t);
        }
    }
    if (rc != TK_OK) {
        delete t;
        return rc;
    }
    *out = t;
    return TK_OK;
}

int tk_tree_create_device(const void* dev_points, int64_t n, int dims, int dtype, int levels, int device,
                          void* stream, tk_tree** out) {
    clear_error();
    if (!out) return fail(TK_EINVAL, "out is null");
    *out = nullptr;
    if (dtype != TK_F32 && dtype != TK_F64) return fail(TK_EINVAL, "dtype must be TK_F32 or TK_F64");
    if (!dev_points) return fail(TK_EINVAL, "points pointer is null");
    if (dims < 1 || dims > kMaxDims)
        return fail(TK_EINVAL, "KD-tree supports dims 1 to " + std::to_string(kMaxDims) + " (got " +
                                   std::to_string(dims) + ")");
    if (n < 1) return fail(TK_EINVAL, "the reference point cloud is empty");
    if (n >= (int64_t(1) << 31)) return fail(TK_EINVAL, "only 32 bit signed indexing implemented (n < 2^31)");
    if (levels < 1 || levels > kMaxLevels)
        return fail(TK_EINVAL, "levels must be in [1, " + std::to_string(kMaxLevels) + "]");
    // node sizes at depth t are floor / ceil of n / 2^t: a leaf parent gets no
    // point exactly when n < 2^(levels-1)
    if (n < (int64_t(1) << (levels - 1)))
        return fail(TK_EINVAL,
                    "Ran out of points while building KD-Tree. Either you required too many levels, "
                    "or you used a lot of coplanar points");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
        cudaGetLastError();
        return fail(TK_EINVAL, "CUDA device " + std::to_string(device) + " is not available");
    }
    cudaPointerAttributes attr;
    if (cudaPointerGetAttributes(&attr, dev_points) != cudaSuccess ||
        (attr.type != cudaMemoryTypeDevice && attr.type != cudaMemoryTypeManaged) || attr.device != device) {
        cudaGetLastError();
        return fail(TK_EINVAL, "points must be device memory on CUDA device " + std::to_string(device));
    }
    tk_tree* t = new (std::nothrow) tk_tree();
    if (!t) return fail(TK_ENOMEM, "host allocation failed");
    t->dtype = dtype;
    t->dims = dims;
    t->levels = levels;
    t->device = device;
    t->n = n;
    t->host_layout = false;
    DeviceGuard g(device);
    const int rc = dtype == TK_F32
                       ? build_device_tree<float>(static_cast<const float*>(dev_points), n, dims, levels, stream, t)
                       : build_device_tree<double>(static_cast<const double*>(dev_points), n, dims, levels, stream, t);
    if (rc != TK_OK) {
        cudaStreamSynchronize(static_cast<cudaStream_t>(stream));
        free_tree_device(t);
        delete t;
        return rc;
    }
    *out = t;
    return TK_OK;
}

int tk_tree_destroy(tk_tree* t) {
    clear_error();
    if (!t) return TK_OK;
    if (t->device >= 0) {
        DeviceGuard g(t->device);
        free_tree_device(t);
        tk::free_host_pipe(t->pipe);
        t->pipe = nullptr;
    }
    delete t;
    return TK_OK;
}

int tk_tree_get_info(const tk_tree* t, tk_tree_info* out) {
    if (!t || !out) return fail(TK_EINVAL, "null argument");
    out->n_points = t->n;
    out->dims = t->dims;
    out->dtype = t->dtype;
    out->levels = t->levels;
    out->device = t->device;
    out->n_leaves = int64_t(1) << t->levels;
    out->device_bytes = t->device_bytes;
    return TK_OK;
}

int tk_tree_get_perm(const tk_tree* t, int32_t* out) {
    if (!t || !out) return fail(TK_EINVAL, "null argument");
    if (!t->host_layout)
        return t->dtype == TK_F32 ? device_layout<float>(t, nullptr, out) : device_layout<double>(t, nullptr, out);
    const auto& p = t->dtype == TK_F32 ? t->h32.perm : t->h64.perm;
    std::memcpy(out, p.data(), sizeof(int32_t) * p.size());
    return TK_OK;
}

int tk_tree_get_points(const tk_tree* t, void* out) {
    if (!t || !out) return fail(TK_EINVAL, "null argument");
    if (!t->host_layout)
        return t->dtype == TK_F32 ? device_layout<float>(t, static_cast<float*>(out), nullptr)
                                  : device_layout<double>(t, static_cast<double*>(out), nullptr);
    if (t->dtype == TK_F32)
        std::memcpy(out, t->h32.structured.data(), sizeof(float) * t->h32.structured.size());
    else
        std::memcpy(out, t->h64.structured.data(), sizeof(double) * t->h64.structured.size());
    return TK_OK;
}

int tk_tree_get_splits(const tk_tree* t, void* medians, int32_t* leaf_offsets) {
    if (!t) return fail(TK_EINVAL, "null argument");
    if (!t->host_layout) {
        DeviceGuard g(t->device);
        const size_t nparts = (size_t(1) << t->levels) - 1;
        cudaError_t e = cudaSuccess;
        if (medians)
            e = cudaMemcpy(medians, t->d_medians, (t->dtype == TK_F32 ? 4 : 8) * nparts, cudaMemcpyDeviceToHost);
        if (e == cudaSuccess && leaf_offsets)
            e = cudaMemcpy(leaf_offsets, t->d_leaf_off, sizeof(int32_t) * (nparts + 2), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return fail(TK_ECUDA, std::string("split copy: ") + cudaGetErrorString(e));
        return TK_OK;
    }
    if (medians) {
        if (t->dtype == TK_F32)
            std::memcpy(medians, t->h32.medians.data(), sizeof(float) * t->h32.medians.size());
        else
            std::memcpy(medians, t->h64.medians.data(), sizeof(double) * t->h64.medians.size());
    }
    if (leaf_offsets) {
        const auto& o = t->dtype == TK_F32 ? t->h32.leaf_off : t->h64.leaf_off;
        std::memcpy(leaf_offsets, o.data(), sizeof(int32_t) * o.size());
    }
    return TK_OK;
}

size_t tk_tree_query_workspace_size(const tk_tree* t, int64_t nq) {
    if (!t || nq < 0) return 0;
    return ws_layout(t->levels, std::max<int64_t>(nq, 1)).total;
}

int tk_tree_query(const tk_tree* t, const void* q, int64_t nq, int k, void* dists, int32_t* idx,
                  const tk_query_opts* opts, void* workspace, size_t workspace_bytes, void* stream) {
    clear_error();
    if (!t) return fail(TK_EINVAL, "tree is null");
    if (nq < 0 || nq >= (int64_t(1) << 31)) return fail(TK_EINVAL, "number of queries must be in [0, 2^31)");
    if (k < 1) return fail(TK_EINVAL, "k must be >= 1");
    if (k > t->n) return fail(TK_EINVAL, "You requested more nearest neighbors than there are in the KD-Tree");
    if (k > kMaxK) return fail(TK_EINVAL, "k is limited to 128 on the GPU");
    if (t->device < 0 || !t->d_pts) return fail(TK_EINVAL, "tree was built host-only (device < 0); it has no device image");
    if (nq == 0) return TK_OK;
    if (!q || !dists || !idx) return fail(TK_EINVAL, "null query or output pointer");
    const size_t need = ws_layout(t->levels, nq).total;
    if (!workspace || workspace_bytes < need)
        return fail(TK_EWORKSPACE, "workspace too small: need " + std::to_string(need) + " bytes");
    if (ws_misaligned(workspace)) return fail(TK_EINVAL, "workspace must be 256-byte aligned");
    tk_query_opts o{0, -1, -1, 0, 0, nullptr, nullptr, -1, 0};
    if (opts) o = *opts;
    DeviceGuard g(t->device);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    char* ws = static_cast<char*>(workspace);
    const int n32 = int(nq);
    if (t->dtype == TK_F32) {
        auto* qq = static_cast<const float*>(q);
        auto* dd = static_cast<float*>(dists);
        switch (t->dims) {
            case 1: return run_query<float, 1>(t, qq, n32, k, dd, idx, o, ws, s);
            case 2: return run_query<float, 2>(t, qq, n32, k, dd, idx, o, ws, s);
            case 3: return run_query<float, 3>(t, qq, n32, k, dd, idx, o, ws, s);
            default: return run_query_wide<float>(t, qq, n32, k, dd, idx, o, ws, s);
        }
    } else {
        auto* qq = static_cast<const double*>(q);
        auto* dd = static_cast<double*>(dists);
        switch (t->dims) {
            case 1: return run_query<double, 1>(t, qq, n32, k, dd, idx, o, ws, s);
            case 2: return run_query<double, 2>(t, qq, n32, k, dd, idx, o, ws, s);
            case 3: return run_query<double, 3>(t, qq, n32, k, dd, idx, o, ws, s);
            default: return run_query_wide<double>(t, qq, n32, k, dd, idx, o, ws, s);
        }
    }
}

}  // extern "C"

// ------------------------------------------------ allocation-free query --
//
// Scratch of tk_tree_query_noalloc: one static device array, sized for
// TK_NOALLOC_MAX_QUERIES queries (counter + 2^16 cell counts + four 32-bit
// arrays of that many queries + the scratch of the cost-class radix pass:
// 256 counts per tile of 2,048 queries and their scan's tile sums, laid out
// as ws_layout() lays out a caller's workspace; the call checks the layout
// against this size before any launch).  Every GPU that loads the library
// holds it until the process exits, and every call on a device shares it.
namespace tk {
namespace {

constexpr size_t kNoAllocScratchBytes = 256 + sizeof(int) * (size_t(1) << kMaxBinLevels) +
                                        4 * sizeof(int) * size_t(TK_NOALLOC_MAX_QUERIES) +
                                        sizeof(int) * 256 * ((size_t(TK_NOALLOC_MAX_QUERIES) + 2047) / 2048) + 1024;
static_assert(TK_NOALLOC_MAX_QUERIES % 64 == 0, "each scratch array must stay 256-byte aligned");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
void* g_noalloc_ptr[kNoAllocMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device (looked up once
// per device; in host code the symbol itself is only a host-side stand-in).
int noalloc_scratch(int dev, void** out) {
    if (dev < 0 || dev >= kNoAllocMaxDevices) return fail(TK_EINVAL, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return fail(TK_ECUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
        g_noalloc_ptr[dev] = p;
    }
    *out = g_noalloc_ptr[dev];
    return TK_OK;
}

}  // namespace
}  // namespace tk

extern "C" int tk_tree_query_noalloc(const tk_tree* t, const void* q, int64_t nq, int k, void* dists, int32_t* idx,
                                     const tk_query_opts* opts, void* stream) {
    clear_error();
    if (!t) return fail(TK_EINVAL, "tree is null");
    if (nq < 0 || nq > TK_NOALLOC_MAX_QUERIES)
        return fail(TK_EINVAL, "tk_tree_query_noalloc takes at most " + std::to_string(TK_NOALLOC_MAX_QUERIES) +
                                   " queries per call (got " + std::to_string(nq) + "); split the batch");
    if (k < 1) return fail(TK_EINVAL, "k must be >= 1");
    if (k > t->n) return fail(TK_EINVAL, "You requested more nearest neighbors than there are in the KD-Tree");
    if (k > kMaxK) return fail(TK_EINVAL, "k is limited to 128 on the GPU");
    if (t->device < 0 || !t->d_pts) return fail(TK_EINVAL, "tree was built host-only (device < 0); it has no device image");
    if (nq == 0) return TK_OK;
    if (!q || !dists || !idx) return fail(TK_EINVAL, "null query or output pointer");
    DeviceGuard g(t->device);
    void* scratch = nullptr;
    int rc = noalloc_scratch(t->device, &scratch);
    if (rc != TK_OK) return rc;
    if (ws_layout(t->levels, nq).total > kNoAllocScratchBytes)
        return fail(TK_EINVAL, "query needs more scratch than the static array holds");
    tk_query_opts o{0, -1, -1, 0, 0, nullptr, nullptr, -1, 0};
    if (opts) o = *opts;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    char* ws = static_cast<char*>(scratch);
    const int n32 = int(nq);
    if (t->dtype == TK_F32) {
        auto* qq = static_cast<const float*>(q);
        auto* dd = static_cast<float*>(dists);
        switch (t->dims) {
            case 1: return run_query<float, 1>(t, qq, n32, k, dd, idx, o, ws, s);
            case 2: return run_query<float, 2>(t, qq, n32, k, dd, idx, o, ws, s);
            case 3: return run_query<float, 3>(t, qq, n32, k, dd, idx, o, ws, s);
            default: return run_query_wide<float>(t, qq, n32, k, dd, idx, o, ws, s);
        }
    }
    auto* qq = static_cast<const double*>(q);
    auto* dd = static_cast<double*>(dists);
    switch (t->dims) {
        case 1: return run_query<double, 1>(t, qq, n32, k, dd, idx, o, ws, s);
        case 2: return run_query<double, 2>(t, qq, n32, k, dd, idx, o, ws, s);
        case 3: return run_query<double, 3>(t, qq, n32, k, dd, idx, o, ws, s);
        default: return run_query_wide<double>(t, qq, n32, k, dd, idx, o, ws, s);
    }
}

// ------------------------------------------------- host-buffer query --
//
// tk_tree_query_host: queries and results in host memory.  The queries are
// uploaded into device staging with one copy (the search reads each query
// more than once; host reads at link latency slowed it down), then:
//  * direct: the result buffers are registered (pinned) memory that the GPU
//    can address, so the query kernel writes the results into host memory
//    itself (over NVLink-C2C on Grace-Blackwell), spread over the search
//    instead of a download after it;
//  * staged: the results go to device staging and are downloaded after the
//    search.
// Device staging and workspace are kept per tree (grown as needed) and freed
// with it; calls on one tree are serialised by its mutex.

namespace tk {

struct HostPipe {
    std::mutex mu;
    char* buf = nullptr;
    size_t cap = 0;
};

void free_host_pipe(HostPipe* p) {
    if (!p) return;
    if (p->buf) cudaFree(p->buf);
    delete p;
}

namespace {

std::mutex g_pipe_create_mu;

HostPipe* host_pipe(const tk_tree* t) {
    std::lock_guard<std::mutex> lk(g_pipe_create_mu);
    if (!t->pipe) t->pipe = new HostPipe();
    return t->pipe;
}

// Device address of registered host memory, or null when the GPU cannot
// address it (pageable memory, or not host memory at all).
void* mapped_host(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

int pipe_buffer(HostPipe* p, size_t need, char** out) {
    if (p->cap < need) {
        if (p->buf) cudaFree(p->buf);
        p->buf = nullptr;
        p->cap = 0;
        const cudaError_t e = cudaMalloc(&p->buf, need);
        if (e != cudaSuccess) return fail(TK_ECUDA, std::string("host query staging: ") + cudaGetErrorString(e));
        p->cap = need;
    }
    *out = p->buf;
    return TK_OK;
}

}  // namespace
}  // namespace tk

extern "C" int tk_tree_query_host(const tk_tree* t, const void* q, int64_t nq, int k, void* dists, int32_t* idx,
                                  const tk_query_opts* opts, int transfer, void* stream) {
    using namespace tk;
    clear_error();
    if (!t) return fail(TK_EINVAL, "tree is null");
    if (nq < 0 || nq >= (int64_t(1) << 31)) return fail(TK_EINVAL, "number of queries must be in [0, 2^31)");
    if (k < 1) return fail(TK_EINVAL, "k must be >= 1");
    if (k > t->n) return fail(TK_EINVAL, "You requested more nearest neighbors than there are in the KD-Tree");
    if (k > kMaxK) return fail(TK_EINVAL, "k is limited to 128 on the GPU");
    if (t->device < 0 || !t->d_pts) return fail(TK_EINVAL, "tree was built host-only (device < 0); it has no device image");
    if (transfer != TK_HOST_AUTO && transfer != TK_HOST_DIRECT && transfer != TK_HOST_STAGED)
        return fail(TK_EINVAL, "transfer must be TK_HOST_AUTO, TK_HOST_DIRECT or TK_HOST_STAGED");
    if (nq == 0) return TK_OK;
    if (!q || !dists || !idx) return fail(TK_EINVAL, "null query or output pointer");

    DeviceGuard g(t->device);
    void* md = nullptr;
    void* mi = nullptr;
    if (transfer != TK_HOST_STAGED) {
        md = mapped_host(dists);
        mi = mapped_host(idx);
    }
    const bool direct = md && mi;
    if (transfer == TK_HOST_DIRECT && !direct)
        return fail(TK_EINVAL, "direct transfer needs registered (pinned) result buffers the GPU can address");

    HostPipe* p = host_pipe(t);
    std::lock_guard<std::mutex> lk(p->mu);
    const size_t es = t->dtype == TK_F32 ? 4 : 8;
    const size_t qb = es * size_t(t->dims) * size_t(nq), db = es * size_t(k) * size_t(nq),
                 ib = 4 * size_t(k) * size_t(nq);
    const size_t wsb = align_up(ws_layout(t->levels, nq).total, 256);
    const size_t need = wsb + align_up(qb, 256) + (direct ? 0 : align_up(db, 256) + align_up(ib, 256));
    char* buf = nullptr;
    int rc = pipe_buffer(p, need, &buf);
    if (rc != TK_OK) return rc;
    tk_query_opts o{0, -1, -1, 0, 0, nullptr, nullptr, -1, 0};
    if (opts) o = *opts;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaError_t e = cudaSuccess;
    char* dq = buf + wsb;
    e = cudaMemcpyAsync(dq, q, qb, cudaMemcpyDefault, s);  // unified addressing: any kind of buffer
    if (direct) {
        if (e == cudaSuccess) rc = tk_tree_query(t, dq, nq, k, md, static_cast<int32_t*>(mi), &o, buf, wsb, s);
    } else {
        char* dd = dq + align_up(qb, 256);
        char* di = dd + align_up(db, 256);
        if (e == cudaSuccess) rc = tk_tree_query(t, dq, nq, k, dd, reinterpret_cast<int32_t*>(di), &o, buf, wsb, s);
        if (e == cudaSuccess && rc == TK_OK) e = cudaMemcpyAsync(dists, dd, db, cudaMemcpyDefault, s);
        if (e == cudaSuccess && rc == TK_OK) e = cudaMemcpyAsync(idx, di, ib, cudaMemcpyDefault, s);
    }
    const cudaError_t se = cudaStreamSynchronize(s);  // whatever was queued completes, also on failure
    if (rc != TK_OK) return rc;
    if (e == cudaSuccess) e = se;
    if (e != cudaSuccess) return fail(TK_ECUDA, std::string("host query: ") + cudaGetErrorString(e));
    return TK_OK;
}
