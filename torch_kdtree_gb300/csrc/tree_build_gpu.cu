// KD-tree construction on the GPU, in exactly the layout build_host_tree
// produces (the reference's createKDTree, src/kdtree.hpp:392-534): node at
// depth t splits on axis t % dims, its points ordered along that axis by
// (coordinate, original index) send the first floor(n/2) left, split value =
// middle element or 0.5 * (a + b) of the two middle ones, leaves contiguous,
// points inside a leaf ordered along the leaf parent's axis.
//
// Presorted-axes construction instead of per-node sorting:
//   1. for every axis a, P_a = all point ids stably radix-sorted by the
//      coordinate's order-preserving key (ties keep ascending ids);
//   2. level by level, every node's points occupy the same range [lo, lo+n)
//      in every P_a, sorted along that axis.  The split axis's array gives
//      the split value (ranks h-1, h) and each point's side; every other
//      axis's array is stably partitioned by side within its node (one
//      global exclusive scan of the "goes left" flags and one scatter), which
//      keeps both children's ranges sorted;
//   3. node sizes depend only on n (left = floor(n/2)), so the node ranges of
//      the next level come from the current ones without looking at data;
//   4. after the last split, the leaf parents' axis array is the final point
//      order; point records, split values, leaf offsets and node bounding
//      boxes are written straight into the tree's device image.
// Work per level is a few coalesced passes over n ids, with no per-node
// selection or sort: dims radix sorts plus about 4 (dims - 1) + 2 passes per
// level.
#include <algorithm>
#include <cstring>
#include <limits>
#include <string>
#include <vector>

#include "sort.cuh"
#include "tk_device.cuh"
#include "tk_internal.h"

namespace tk {
namespace {

constexpr int kThreads = 256;

unsigned blocks_for(int64_t n) { return unsigned((n + kThreads - 1) / kThreads); }

// Order-preserving unsigned keys; -0 and +0 get the same key (they compare
// equal on the host, so their order falls to the original index).
__device__ __forceinline__ uint32_t coord_key32(float v) {
    uint32_t b = __float_as_uint(v == 0.0f ? 0.0f : v);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ unsigned long long coord_key64(double v) {
    unsigned long long b = (unsigned long long)__double_as_longlong(v == 0.0 ? 0.0 : v);
    return (b & 0x8000000000000000ull) ? ~b : (b | 0x8000000000000000ull);
}

template <typename T>
__global__ void k_axis_keys(const T* __restrict__ pts, int64_t n, int dims, int ax, uint32_t* __restrict__ key_lo,
                            uint32_t* __restrict__ key_hi, int* __restrict__ nan_flag) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const T v = pts[i * dims + ax];
    if (v != v) *nan_flag = 1;
    if constexpr (sizeof(T) == 4) {
        key_lo[i] = coord_key32(float(v));
    } else {
        const unsigned long long k = coord_key64(double(v));
        key_lo[i] = uint32_t(k);
        key_hi[i] = uint32_t(k >> 32);
    }
}

__global__ void k_gather_u32(const uint32_t* __restrict__ src, const uint32_t* __restrict__ idx, int64_t n,
                             uint32_t* __restrict__ dst) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = src[idx[i]];
}

__device__ __forceinline__ float add_t(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_t(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float half_t(float s) { return __double2float_rn(__dmul_rn(0.5, double(s))); }
__device__ __forceinline__ double half_t(double s) { return __dmul_rn(0.5, s); }

// Split values of the 2^t nodes of level t (and, at the leaf parents, the
// leaf offsets).  compMedian (src/kdtree.hpp:392-401): odd n -> element h,
// even n -> 0.5 * (element h-1 + element h), the sum rounded in T and the
// product taken in double.
template <typename T>
__global__ void k_level_split(const T* __restrict__ pts, int dims, int ax, const uint32_t* __restrict__ pa,
                              const int32_t* __restrict__ off, int nodes, T* __restrict__ medians,
                              int32_t* __restrict__ leaf_off, bool last) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nodes) return;
    const int32_t lo = off[j], cnt = off[j + 1] - lo, h = cnt / 2;
    const T upper = pts[int64_t(pa[lo + h]) * dims + ax];
    const T lower = h > 0 ? pts[int64_t(pa[lo + h - 1]) * dims + ax] : upper;
    medians[nodes - 1 + j] = (cnt & 1) ? upper : half_t(add_t(lower, upper));
    if (last) {
        leaf_off[2 * j] = lo;
        leaf_off[2 * j + 1] = lo + h;
    }
}

// side[id] = 1 if point id goes to the right child of its node.
__global__ void k_mark_side(const uint32_t* __restrict__ pa, int64_t n, const int32_t* __restrict__ node_of,
                            const int32_t* __restrict__ off, uint8_t* __restrict__ side) {
    const int64_t p = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const int j = node_of[p];
    const int32_t lo = off[j], h = (off[j + 1] - lo) / 2;
    side[pa[p]] = uint8_t(int32_t(p) - lo >= h);
}

__global__ void k_left_flags(const uint32_t* __restrict__ pb, int64_t n, const uint8_t* __restrict__ side,
                             int* __restrict__ flags) {
    const int64_t p = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (p < n) flags[p] = side[pb[p]] ^ 1;
}

// Stable partition of every node's range of pb by side: lefts first.  pre is
// the exclusive prefix sum of the left flags over the whole array.
__global__ void k_partition(const uint32_t* __restrict__ pb, int64_t n, const uint8_t* __restrict__ side,
                            const int32_t* __restrict__ node_of, const int32_t* __restrict__ off,
                            const int* __restrict__ pre, uint32_t* __restrict__ out) {
    const int64_t p = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const int j = node_of[p];
    const int32_t lo = off[j], h = (off[j + 1] - lo) / 2;
    const uint32_t id = pb[p];
    const int32_t left_before = pre[p] - pre[lo];
    const int32_t dst = side[id] == 0 ? lo + left_before : lo + h + (int32_t(p) - lo - left_before);
    out[dst] = id;
}

// Node of every position at the next level, and the next level's ranges.
__global__ void k_next_nodes(int64_t n, const int32_t* __restrict__ off, int32_t* __restrict__ node_of) {
    const int64_t p = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const int j = node_of[p];
    const int32_t lo = off[j], h = (off[j + 1] - lo) / 2;
    node_of[p] = 2 * j + (int32_t(p) - lo >= h ? 1 : 0);
}

__global__ void k_child_offsets(const int32_t* __restrict__ off, int nodes, int32_t* __restrict__ next) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j > nodes) return;
    if (j == nodes) {
        next[2 * nodes] = off[nodes];
        return;
    }
    const int32_t lo = off[j];
    next[2 * j] = lo;
    next[2 * j + 1] = lo + (off[j + 1] - lo) / 2;
}

template <typename T>
__global__ void k_make_records(const T* __restrict__ pts, int dims, const uint32_t* __restrict__ order, int64_t n,
                               PointRec<T>* __restrict__ recs) {
    const int64_t p = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const uint32_t id = order[p];
    T c[3] = {T(0), T(0), T(0)};
    for (int d = 0; d < dims; ++d) c[d] = pts[int64_t(id) * dims + d];
    PointRec<T> r;
    r.x = c[0];
    r.y = c[1];
    r.z = c[2];
    if constexpr (sizeof(T) == 4) {
        r.w = __uint_as_float(id);
    } else {
        r.w = __longlong_as_double((long long)id);
    }
    recs[p] = r;
}

// Box of every leaf (one warp per leaf), stored at node 2^L - 1 + leaf, with
// the leaf's point range in the records' 4th slots.
template <typename T>
__global__ void k_leaf_boxes(const PointRec<T>* __restrict__ recs, const int32_t* __restrict__ leaf_off,
                             int64_t nleaves, PointRec<T>* __restrict__ boxes) {
    const int64_t leaf = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (leaf >= nleaves) return;
    const T inf = std::numeric_limits<T>::infinity();
    T lo[3] = {inf, inf, inf}, hi[3] = {-inf, -inf, -inf};
    for (int32_t i = leaf_off[leaf] + lane; i < leaf_off[leaf + 1]; i += 32) {
        const PointRec<T> r = recs[i];
        const T c[3] = {r.x, r.y, r.z};
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            lo[d] = c[d] < lo[d] ? c[d] : lo[d];
            hi[d] = hi[d] < c[d] ? c[d] : hi[d];
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const T l = __shfl_xor_sync(0xFFFFFFFFu, lo[d], o);
            const T h = __shfl_xor_sync(0xFFFFFFFFu, hi[d], o);
            lo[d] = l < lo[d] ? l : lo[d];
            hi[d] = hi[d] < h ? h : hi[d];
        }
    }
    if (lane == 0) {  // the box records also carry the leaf's point range [begin, end)
        const int64_t node = nleaves - 1 + leaf;
        PointRec<T> a{lo[0], lo[1], lo[2], T(0)}, b{hi[0], hi[1], hi[2], T(0)};
        if constexpr (sizeof(T) == 4) {
            a.w = __uint_as_float(uint32_t(leaf_off[leaf]));
            b.w = __uint_as_float(uint32_t(leaf_off[leaf + 1]));
        } else {
            a.w = __longlong_as_double((long long)uint32_t(leaf_off[leaf]));
            b.w = __longlong_as_double((long long)uint32_t(leaf_off[leaf + 1]));
        }
        boxes[2 * node] = a;
        boxes[2 * node + 1] = b;
    }
}

// Boxes of the 2^t inner nodes of level t from their children.
template <typename T>
__global__ void k_inner_boxes(int nodes, PointRec<T>* __restrict__ boxes) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nodes) return;
    const int64_t id = int64_t(nodes) - 1 + j;
    const PointRec<T> al = boxes[2 * (2 * id + 1)], ah = boxes[2 * (2 * id + 1) + 1];
    const PointRec<T> bl = boxes[2 * (2 * id + 2)], bh = boxes[2 * (2 * id + 2) + 1];
    PointRec<T> lo, hi;
    lo.x = bl.x < al.x ? bl.x : al.x;
    lo.y = bl.y < al.y ? bl.y : al.y;
    lo.z = bl.z < al.z ? bl.z : al.z;
    lo.w = T(0);
    hi.x = ah.x < bh.x ? bh.x : ah.x;
    hi.y = ah.y < bh.y ? bh.y : ah.y;
    hi.z = ah.z < bh.z ? bh.z : ah.z;
    hi.w = T(0);
    boxes[2 * id] = lo;
    boxes[2 * id + 1] = hi;
}

// Trees of 4-8 dimensions: coordinate rows of W (zero padded) and the
// original indices, in leaf order.
template <typename T>
__global__ void k_make_rows(const T* __restrict__ pts, int dims, int W, const uint32_t* __restrict__ order,
                            int64_t n, T* __restrict__ rows, int32_t* __restrict__ perm) {
    const int64_t p = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const uint32_t id = order[p];
    for (int d = 0; d < W; ++d) rows[p * W + d] = d < dims ? pts[int64_t(id) * dims + d] : T(0);
    perm[p] = int32_t(id);
}

// Leaf boxes of such a tree (one warp per leaf): lo row at node 2i, hi at 2i+1.
template <typename T>
__global__ void k_leaf_boxes_wide(const T* __restrict__ rows, int W, const int32_t* __restrict__ leaf_off,
                                  int64_t nleaves, T* __restrict__ boxes) {
    const int64_t leaf = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (leaf >= nleaves) return;
    const T inf = std::numeric_limits<T>::infinity();
    T lo[kMaxDims], hi[kMaxDims];
#pragma unroll
    for (int d = 0; d < kMaxDims; ++d) {
        lo[d] = inf;
        hi[d] = -inf;
    }
    for (int32_t i = leaf_off[leaf] + lane; i < leaf_off[leaf + 1]; i += 32) {
#pragma unroll
        for (int d = 0; d < kMaxDims; ++d) {
            if (d < W) {
                const T c = rows[int64_t(i) * W + d];
                lo[d] = c < lo[d] ? c : lo[d];
                hi[d] = hi[d] < c ? c : hi[d];
            }
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
        for (int d = 0; d < kMaxDims; ++d) {
            const T l = __shfl_xor_sync(0xFFFFFFFFu, lo[d], o);
            const T h = __shfl_xor_sync(0xFFFFFFFFu, hi[d], o);
            lo[d] = l < lo[d] ? l : lo[d];
            hi[d] = hi[d] < h ? h : hi[d];
        }
    }
    if (lane == 0) {
        const int64_t node = nleaves - 1 + leaf;
        for (int d = 0; d < W; ++d) {
            boxes[(2 * node) * W + d] = lo[d];
            boxes[(2 * node + 1) * W + d] = hi[d];
        }
    }
}

template <typename T>
__global__ void k_inner_boxes_wide(int nodes, int W, T* __restrict__ boxes) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nodes) return;
    const int64_t id = int64_t(nodes) - 1 + j, a = 2 * id + 1, b = 2 * id + 2;
    for (int d = 0; d < W; ++d) {
        const T al = boxes[(2 * a) * W + d], ah = boxes[(2 * a + 1) * W + d];
        const T bl = boxes[(2 * b) * W + d], bh = boxes[(2 * b + 1) * W + d];
        boxes[(2 * id) * W + d] = bl < al ? bl : al;
        boxes[(2 * id + 1) * W + d] = ah < bh ? bh : ah;
    }
}

// Device scratch of one build, freed on every exit path.
struct Scratch {
    std::vector<void*> ptrs;
    cudaError_t err = cudaSuccess;
    template <typename X>
    X* get(size_t count) {
        void* p = nullptr;
        if (err == cudaSuccess) err = cudaMalloc(&p, std::max<size_t>(count * sizeof(X), 16));
        if (err == cudaSuccess) ptrs.push_back(p);
        return static_cast<X*>(p);
    }
    ~Scratch() {
        for (void* p : ptrs) cudaFree(p);
    }
};

#define TK_TRY(expr)                                                                          \
    do {                                                                                      \
        cudaError_t e_ = (expr);                                                              \
        if (e_ != cudaSuccess) return fail(TK_ECUDA, std::string("device build: ") + cudaGetErrorString(e_)); \
    } while (0)

}  // namespace

template <typename T>
int build_device_tree(const T* pts, int64_t n, int dims, int levels, void* stream, tk_tree* t) {
    const cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int L = levels;
    const int64_t nleaves = int64_t(1) << L;
    const int64_t nparts = nleaves - 1;
    const int64_t nnodes = 2 * nleaves - 1;

    Scratch sc;
    uint32_t* P[kMaxDims] = {};
    for (int a = 0; a < dims; ++a) P[a] = sc.get<uint32_t>(n);
    uint32_t* spare = sc.get<uint32_t>(n);
    uint32_t* key_lo = sc.get<uint32_t>(n);
    uint32_t* key_hi = sizeof(T) == 8 ? sc.get<uint32_t>(n) : nullptr;
    uint32_t* tmp_k = sc.get<uint32_t>(n);
    uint32_t* tmp_v = sizeof(T) == 8 ? sc.get<uint32_t>(n) : nullptr;
    uint8_t* side = sc.get<uint8_t>(n);
    int32_t* node_of = sc.get<int32_t>(n);
    int* flags = sc.get<int>(n);
    int32_t* off_a = sc.get<int32_t>(nleaves + 1);
    int32_t* off_b = sc.get<int32_t>(nleaves + 1);
    int* nan_flag = sc.get<int>(1);
    const size_t sort_ws_bytes = sort_workspace_bytes(n);
    void* sort_ws = sc.get<unsigned char>(sort_ws_bytes);
    void* scan_ws = sc.get<unsigned char>(scan_workspace_bytes(n));
    if (sc.err != cudaSuccess) return fail(TK_ENOMEM, std::string("device build scratch: ") + cudaGetErrorString(sc.err));

    // the tree's device image (wide trees: coordinate rows, indices, box rows)
    const bool wide = dims > 3;
    const int W = record_width(dims);
    const size_t b_pts = wide ? sizeof(T) * W * size_t(n) : sizeof(PointRec<T>) * size_t(n);
    const size_t b_perm = wide ? sizeof(int32_t) * size_t(n) : 0;
    const size_t b_med = sizeof(T) * size_t(nparts);
    const size_t b_off = sizeof(int32_t) * size_t(nleaves + 1);
    const size_t b_box = wide ? sizeof(T) * W * 2 * size_t(nnodes) : sizeof(PointRec<T>) * 2 * size_t(nnodes);
    TK_TRY(cudaMalloc(&t->d_pts, b_pts));
    if (wide) TK_TRY(cudaMalloc(reinterpret_cast<void**>(&t->d_perm), b_perm));
    TK_TRY(cudaMalloc(&t->d_medians, std::max<size_t>(b_med, 16)));
    TK_TRY(cudaMalloc(reinterpret_cast<void**>(&t->d_leaf_off), b_off));
    TK_TRY(cudaMalloc(&t->d_boxes, b_box));
    t->device_bytes = int64_t(b_pts + b_perm + b_med + b_off + b_box);
    T* medians = static_cast<T*>(t->d_medians);
    PointRec<T>* recs = static_cast<PointRec<T>*>(t->d_pts);
    PointRec<T>* boxes = static_cast<PointRec<T>*>(t->d_boxes);

    // 1. presorted axes
    TK_TRY(cudaMemsetAsync(nan_flag, 0, sizeof(int), s));
    for (int a = 0; a < dims; ++a) {
        k_axis_keys<T><<<blocks_for(n), kThreads, 0, s>>>(pts, n, dims, a, key_lo, key_hi, nan_flag);
        TK_TRY(cudaGetLastError());
        if constexpr (sizeof(T) == 4) {
            TK_TRY(sort_pairs(key_lo, nullptr, tmp_k, P[a], n, 32, sort_ws, sort_ws_bytes, s));
        } else {
            TK_TRY(sort_pairs(key_lo, nullptr, tmp_k, tmp_v, n, 32, sort_ws, sort_ws_bytes, s));
            k_gather_u32<<<blocks_for(n), kThreads, 0, s>>>(key_hi, tmp_v, n, key_lo);
            TK_TRY(cudaGetLastError());
            TK_TRY(sort_pairs(key_lo, tmp_v, tmp_k, P[a], n, 32, sort_ws, sort_ws_bytes, s));
        }
    }

    // 2./3. level by level
    const int32_t init_off[2] = {0, int32_t(n)};
    TK_TRY(cudaMemcpyAsync(off_a, init_off, sizeof(init_off), cudaMemcpyHostToDevice, s));
    TK_TRY(cudaMemsetAsync(node_of, 0, sizeof(int32_t) * size_t(n), s));
    int32_t* off = off_a;
    int32_t* off_next = off_b;
    for (int lev = 0; lev < L; ++lev) {
        const int ax = lev % dims;
        const int nodes = 1 << lev;
        const bool last = lev == L - 1;
        k_level_split<T><<<blocks_for(nodes), kThreads, 0, s>>>(pts, dims, ax, P[ax], off, nodes, medians,
                                                                t->d_leaf_off, last);
        TK_TRY(cudaGetLastError());
        if (last) break;
        k_mark_side<<<blocks_for(n), kThreads, 0, s>>>(P[ax], n, node_of, off, side);
        TK_TRY(cudaGetLastError());
        for (int b = 0; b < dims; ++b) {
            if (b == ax) continue;
            k_left_flags<<<blocks_for(n), kThreads, 0, s>>>(P[b], n, side, flags);
            TK_TRY(cudaGetLastError());
            TK_TRY(exclusive_scan(flags, n, scan_ws, s));
            k_partition<<<blocks_for(n), kThreads, 0, s>>>(P[b], n, side, node_of, off, flags, spare);
            TK_TRY(cudaGetLastError());
            std::swap(P[b], spare);
        }
        k_next_nodes<<<blocks_for(n), kThreads, 0, s>>>(n, off, node_of);
        k_child_offsets<<<blocks_for(nodes + 1), kThreads, 0, s>>>(off, nodes, off_next);
        TK_TRY(cudaGetLastError());
        std::swap(off, off_next);
    }
    const int32_t n32 = int32_t(n);
    TK_TRY(cudaMemcpyAsync(t->d_leaf_off + nleaves, &n32, sizeof(int32_t), cudaMemcpyHostToDevice, s));

    // 4. records in leaf order, node boxes bottom-up
    if (wide) {
        T* rows = static_cast<T*>(t->d_pts);
        T* wboxes = static_cast<T*>(t->d_boxes);
        k_make_rows<T><<<blocks_for(n), kThreads, 0, s>>>(pts, dims, W, P[(L - 1) % dims], n, rows, t->d_perm);
        k_leaf_boxes_wide<T><<<unsigned((nleaves * 32 + kThreads - 1) / kThreads), kThreads, 0, s>>>(
            rows, W, t->d_leaf_off, nleaves, wboxes);
        TK_TRY(cudaGetLastError());
        for (int lev = L - 1; lev >= 0; --lev) {
            k_inner_boxes_wide<T><<<blocks_for(int64_t(1) << lev), kThreads, 0, s>>>(1 << lev, W, wboxes);
            TK_TRY(cudaGetLastError());
        }
    } else {
        k_make_records<T><<<blocks_for(n), kThreads, 0, s>>>(pts, dims, P[(L - 1) % dims], n, recs);
        k_leaf_boxes<T><<<unsigned((nleaves * 32 + kThreads - 1) / kThreads), kThreads, 0, s>>>(recs, t->d_leaf_off,
                                                                                                nleaves, boxes);
        TK_TRY(cudaGetLastError());
        for (int lev = L - 1; lev >= 0; --lev) {
            k_inner_boxes<T><<<blocks_for(int64_t(1) << lev), kThreads, 0, s>>>(1 << lev, boxes);
            TK_TRY(cudaGetLastError());
        }
    }
    int nan_host = 0;
    TK_TRY(cudaMemcpyAsync(&nan_host, nan_flag, sizeof(int), cudaMemcpyDeviceToHost, s));
    TK_TRY(cudaStreamSynchronize(s));
    if (nan_host) return fail(TK_EINVAL, "reference points contain NaN");
    return TK_OK;
}

template int build_device_tree<float>(const float*, int64_t, int, int, void*, tk_tree*);
template int build_device_tree<double>(const double*, int64_t, int, int, void*, tk_tree*);

}  // namespace tk
