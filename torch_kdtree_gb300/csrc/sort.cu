// Exclusive scan and stable LSD radix sort (see sort.cuh).
//
// Radix pass over 8-bit digits, tiles of kTile = 256 threads x kRounds items:
//   1. k_digit_hist: per-tile digit histogram, stored digit-major
//      (hist[digit * ntiles + tile]) so that one exclusive scan of the whole
//      array yields every (digit, tile) output start in stable order;
//   2. exclusive_scan over that array;
//   3. k_digit_scatter: the tile is walked in rounds of 256 consecutive
//      items; within a round each warp ranks equal digits with
//      __match_any_sync, warps are ordered through a shared table, and a
//      running per-digit count carries across rounds -- so every item's rank
//      equals its rank in input order among equal digits (stability).
#include <algorithm>

#include "sort.cuh"

namespace tk {

namespace {

constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;  // per thread
constexpr int kScanTile = kScanThreads * kScanItems;

constexpr int kSortThreads = 256;
constexpr int kRounds = 8;
constexpr int kTile = kSortThreads * kRounds;
constexpr int kWarps = kSortThreads / 32;

size_t align256(size_t v) { return (v + 255) / 256 * 256; }

__device__ __forceinline__ int block_exclusive_sum(int v, int* warp_sums, int* total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xFFFFFFFFu, x, o);
        if (lane >= o) x += t;
    }
    if (lane == 31) warp_sums[wid] = x;
    __syncthreads();
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
        int w = lane < nw ? warp_sums[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xFFFFFFFFu, w, o);
            if (lane >= o) w += t;
        }
        warp_sums[lane] = w;
    }
    __syncthreads();
    const int excl = x - v + (wid > 0 ? warp_sums[wid - 1] : 0);
    if (total) *total = warp_sums[(blockDim.x >> 5) - 1];
    __syncthreads();
    return excl;
}

// Tile-local exclusive scan; writes the tile total to sums[blockIdx.x].
__global__ void k_scan_tiles(int* data, int64_t n, int* sums) {
    __shared__ int warp_sums[32];
    const int64_t base = int64_t(blockIdx.x) * kScanTile + int64_t(threadIdx.x) * kScanItems;
    int v[kScanItems];
    int s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        v[i] = base + i < n ? data[base + i] : 0;
        s += v[i];
    }
    int total = 0;
    int run = block_exclusive_sum(s, warp_sums, &total);
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        if (base + i < n) data[base + i] = run;
        run += v[i];
    }
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// One block: exclusive scan of sums[0..m) in place, any m (chunked).
__global__ void k_scan_single(int* sums, int m) {
    __shared__ int warp_sums[32];
    const int per = (m + blockDim.x - 1) / blockDim.x;
    const int beg = min(m, int(threadIdx.x) * per), end = min(m, beg + per);
    int s = 0;
    for (int i = beg; i < end; ++i) s += sums[i];
    int run = block_exclusive_sum(s, warp_sums, nullptr);
    for (int i = beg; i < end; ++i) {
        const int c = sums[i];
        sums[i] = run;
        run += c;
    }
}

__global__ void k_scan_add(int* data, int64_t n, const int* sums) {
    const int64_t base = int64_t(blockIdx.x) * kScanTile;
    const int add = sums[blockIdx.x];
    for (int i = threadIdx.x; i < kScanTile; i += blockDim.x)
        if (base + i < n) data[base + i] += add;
}

__global__ void k_digit_hist(const uint32_t* keys, int64_t n, int shift, int ntiles, int* hist) {
    __shared__ int h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const int64_t base = int64_t(blockIdx.x) * kTile;
#pragma unroll
    for (int r = 0; r < kRounds; ++r) {
        const int64_t e = base + int64_t(r) * kSortThreads + threadIdx.x;
        if (e < n) atomicAdd(&h[(keys[e] >> shift) & 255u], 1);
    }
    __syncthreads();
    hist[int64_t(threadIdx.x) * ntiles + blockIdx.x] = h[threadIdx.x];
}

__global__ void k_digit_scatter(const uint32_t* keys, const uint32_t* vals, int64_t n, int shift, int ntiles,
                                const int* offs, uint32_t* keys_out, uint32_t* vals_out) {
    __shared__ int warp_cnt[kWarps][256];
    __shared__ int run_cnt[256];
    const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
    run_cnt[t] = 0;
    const unsigned lt_mask = (1u << lane) - 1u;
    const int64_t base = int64_t(blockIdx.x) * kTile;
    for (int r = 0; r < kRounds; ++r) {
#pragma unroll
        for (int w = 0; w < kWarps; ++w) warp_cnt[w][t] = 0;
        __syncthreads();
        const int64_t e = base + int64_t(r) * kSortThreads + t;
        const bool valid = e < n;
        uint32_t key = 0, val = 0;
        int digit = 0;
        if (valid) {
            key = keys[e];
            val = vals ? vals[e] : uint32_t(e);
            digit = int((key >> shift) & 255u);
        }
        const unsigned peers = __match_any_sync(0xFFFFFFFFu, valid ? digit : 256 + lane);
        const int rank = __popc(peers & lt_mask);
        if (valid && rank == 0) warp_cnt[wid][digit] = __popc(peers);
        __syncthreads();
        {
            int run = run_cnt[t];
#pragma unroll
            for (int w = 0; w < kWarps; ++w) {
                const int c = warp_cnt[w][t];
                warp_cnt[w][t] = run;
                run += c;
            }
            run_cnt[t] = run;
        }
        __syncthreads();
        if (valid) {
            const int64_t pos = int64_t(offs[int64_t(digit) * ntiles + blockIdx.x]) + warp_cnt[wid][digit] + rank;
            keys_out[pos] = key;
            vals_out[pos] = val;
        }
        __syncthreads();
    }
}

}  // namespace

size_t scan_workspace_bytes(int64_t n) {
    const int64_t tiles = (n + kScanTile - 1) / kScanTile;
    return align256(sizeof(int) * size_t(std::max<int64_t>(tiles, 1)));
}

cudaError_t exclusive_scan(int* data, int64_t n, void* ws, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    const int64_t tiles = (n + kScanTile - 1) / kScanTile;
    int* sums = static_cast<int*>(ws);
    k_scan_tiles<<<unsigned(tiles), kScanThreads, 0, s>>>(data, n, sums);
    k_scan_single<<<1, kScanThreads, 0, s>>>(sums, int(tiles));
    k_scan_add<<<unsigned(tiles), 256, 0, s>>>(data, n, sums);
    return cudaGetLastError();
}

size_t sort_workspace_bytes(int64_t n) {
    const int64_t ntiles = std::max<int64_t>(1, (n + kTile - 1) / kTile);
    const int64_t hist = 256 * ntiles;
    return align256(sizeof(int) * size_t(hist)) + scan_workspace_bytes(hist) +
           2 * align256(sizeof(uint32_t) * size_t(std::max<int64_t>(n, 1)));
}

size_t sort_pass8_workspace_bytes(int64_t n) {
    const int64_t ntiles = std::max<int64_t>(1, (n + kTile - 1) / kTile);
    const int64_t hist = 256 * ntiles;
    return align256(sizeof(int) * size_t(hist)) + scan_workspace_bytes(hist);
}

cudaError_t sort_pass8(const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out, uint32_t* vals_out,
                       int64_t n, void* ws, size_t ws_bytes, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    if (ws_bytes < sort_pass8_workspace_bytes(n)) return cudaErrorInvalidValue;
    const int64_t ntiles = (n + kTile - 1) / kTile;
    const int64_t hist_n = 256 * ntiles;
    int* hist = static_cast<int*>(ws);
    void* scan_ws = static_cast<char*>(ws) + align256(sizeof(int) * size_t(hist_n));
    k_digit_hist<<<unsigned(ntiles), kSortThreads, 0, s>>>(keys_in, n, 0, int(ntiles), hist);
    cudaError_t e = exclusive_scan(hist, hist_n, scan_ws, s);
    if (e != cudaSuccess) return e;
    k_digit_scatter<<<unsigned(ntiles), kSortThreads, 0, s>>>(keys_in, vals_in, n, 0, int(ntiles), hist, keys_out,
                                                             vals_out);
    return cudaGetLastError();
}

cudaError_t sort_pairs(const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out, uint32_t* vals_out,
                       int64_t n, int key_bits, void* ws, size_t ws_bytes, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    if (ws_bytes < sort_workspace_bytes(n)) return cudaErrorInvalidValue;
    const int64_t ntiles = (n + kTile - 1) / kTile;
    const int64_t hist_n = 256 * ntiles;
    char* p = static_cast<char*>(ws);
    int* hist = reinterpret_cast<int*>(p);
    p += align256(sizeof(int) * size_t(hist_n));
    void* scan_ws = p;
    p += scan_workspace_bytes(hist_n);
    uint32_t* tmp_k = reinterpret_cast<uint32_t*>(p);
    p += align256(sizeof(uint32_t) * size_t(n));
    uint32_t* tmp_v = reinterpret_cast<uint32_t*>(p);

    const int passes = std::max(1, (key_bits + 7) / 8);
    // Ping-pong so that the last pass lands in keys_out / vals_out.
    const uint32_t* src_k = keys_in;
    const uint32_t* src_v = vals_in;
    for (int pass = 0; pass < passes; ++pass) {
        const bool to_out = ((passes - 1 - pass) % 2) == 0;
        uint32_t* dk = to_out ? keys_out : tmp_k;
        uint32_t* dv = to_out ? vals_out : tmp_v;
        const int shift = 8 * pass;
        k_digit_hist<<<unsigned(ntiles), kSortThreads, 0, s>>>(src_k, n, shift, int(ntiles), hist);
        cudaError_t e = exclusive_scan(hist, hist_n, scan_ws, s);
        if (e != cudaSuccess) return e;
        k_digit_scatter<<<unsigned(ntiles), kSortThreads, 0, s>>>(src_k, src_v, n, shift, int(ntiles), hist, dk, dv);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        src_k = dk;
        src_v = dv;
    }
    return cudaSuccess;
}

}  // namespace tk
