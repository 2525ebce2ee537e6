/*
 * tk_knn.h -- C ABI of the GB300 KNN engine (libtkknn.so).
 *
 * Drop-in boundary for torch_kdtree's query path.  Every entry point takes
 * plain pointers and sizes, returns a tk_status, never exits the process and
 * never allocates device memory on a query path (tk_tree_query_host, whose
 * device staging is kept per tree, excepted): scratch memory is passed in by
 * the caller (sizes from the *_workspace_size functions; 256-byte aligned, as
 * cudaMalloc returns it -- a misaligned workspace fails with TK_EINVAL before
 * any device work).  Device work is
 * enqueued on the caller's CUDA stream (a cudaStream_t passed as void*; NULL
 * = the legacy default stream, which is what the reference used) and is
 * asynchronous, like the reference's KDTreeKNNGPUSearch.
 *
 * Index results are ORIGINAL point indices (the reference returned indices in
 * tree order and remapped them in Python, torch_kdtree/nn_distance.py:109).
 * Among neighbours at exactly equal distance the lower original index wins.
 */
#ifndef TK_KNN_H
#define TK_KNN_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum tk_status {
    TK_OK = 0,
    TK_EINVAL = 1,       /* bad argument (k > n, unsupported dims, null pointer ...) */
    TK_ENOMEM = 2,       /* allocation failed (tree construction only) */
    TK_EUNSUPPORTED = 3, /* valid request this build does not implement */
    TK_ETIMEOUT = 4,     /* a bounded device-side wait ran out */
    TK_ECUDA = 5,        /* CUDA runtime error; tk_last_error() has the text */
    TK_EWORKSPACE = 6    /* workspace missing or too small */
} tk_status;

typedef enum tk_dtype { TK_F32 = 0, TK_F64 = 1 } tk_dtype;

/* Text of the last error on the calling thread ("" if none). */
const char* tk_last_error(void);
/* ABI version of this library. */
int tk_version(void);
/* 1 if the library can see a CUDA device, else 0.
 * Replaces check_for_gpu (src/interface.cpp:105-112), which reported a
 * compile-time flag rather than a device. */
int tk_cuda_available(void);

/* ------------------------------------------------------------ KD-tree -- */

typedef struct tk_tree tk_tree;

typedef struct tk_tree_info {
    int64_t n_points;
    int32_t dims;
    int32_t dtype;     /* tk_dtype */
    int32_t levels;    /* split levels L: 2^L - 1 split planes, 2^L leaves */
    int32_t device;    /* CUDA ordinal holding the tree */
    int64_t n_leaves;
    int64_t device_bytes;
} tk_tree_info;

/* Build a KD-tree on the host in the reference's layout and upload it.
 * host_points: [n, dims] C-contiguous, float or double per dtype; dims
 * 1..8 (1-3 as the reference compiles, 4-8 as its README's extra template
 * instantiations add).  levels: 1..24 (the reference's default heuristic is applied by the Python
 * layer).  device: CUDA ordinal, or -1 for a host-only tree (layout getters
 * only; queries on it fail with TK_EINVAL).  n_threads: host build threads
 * (0 = all hardware threads).  Fails with TK_EINVAL when a split node would receive no point
 * ("ran out of points"), like the reference.
 * Replaces the constructor of the pybind class KDTree<T,dims,use_gpu>
 * (src/interface.cpp:25-43): createKDTree (src/kdtree.hpp:494-534) +
 * copyPartitionToGPU (src/kdtree_g.cu:63-98). */
int tk_tree_create(const void* host_points, int64_t n, int dims, int dtype, int levels, int device,
                   int n_threads, tk_tree** out);

/* Re-create a tree from a saved layout (the arrays the getters below
 * return: structured points T[n*dims], perm int32[n], split values
 * T[2^L-1], leaf offsets int32[2^L+1]; all host memory) without rebuilding
 * it.  The layout is validated -- offsets from 0 to n and non-decreasing,
 * perm a permutation, no NaN, every split value separating its children's
 * points along its axis -- and TK_EINVAL is returned otherwise, so a
 * corrupt file cannot make queries silently inexact.  device: CUDA ordinal
 * or -1 (host-only).  No reference counterpart: the reference always
 * rebuilt the tree (src/interface.cpp:25-43). */
int tk_tree_create_from_layout(const void* structured_points, const int32_t* perm, const void* medians,
                               const int32_t* leaf_offsets, int64_t n, int dims, int dtype, int levels, int device,
                               tk_tree** out);

/* Build the same tree ON THE GPU from device-resident points: dev_points is
 * device memory on `device`, [n, dims] C-contiguous, float or double per
 * dtype.  The result is identical to tk_tree_create's (split values, leaf
 * offsets, point order, original indices; ties on a coordinate ordered by
 * original index), built level by level from one stable radix sort per axis
 * instead of per-node sorts, with no host copy of the points.  Runs on
 * `stream` and synchronises it before returning.  The layout getters below
 * copy from the device for such a tree.  Same errors as tk_tree_create
 * (NaN points, too many levels for n).  Replaces the host-side
 * createKDTree (src/kdtree.hpp:494-534) + copyPartitionToGPU
 * (src/kdtree_g.cu:63-98) that the reference runs after copying the points
 * to the host (torch_kdtree/nn_distance.py:26-31). */
int tk_tree_create_device(const void* dev_points, int64_t n, int dims, int dtype, int levels, int device,
                          void* stream, tk_tree** out);

/* Free the tree and its device memory.  Replaces ~KDTree
 * (src/interface.cpp:88-94) + freePartitionFromGPU (src/kdtree_g.cu:140-157). */
int tk_tree_destroy(tk_tree* tree);

int tk_tree_get_info(const tk_tree* tree, tk_tree_info* out);

/* Host copies of the layout.  Replace get_shuffled_inds / get_structured_points
 * (src/interface.cpp:45-58). perm: int32[n]; points: T[n*dims]. */
int tk_tree_get_perm(const tk_tree* tree, int32_t* out);
int tk_tree_get_points(const tk_tree* tree, void* out);
/* Split planes in heap order (T[2^L-1]; axis of node i is depth(i) % dims)
 * and leaf start offsets (int32[2^L + 1]).  Partition / PartitionLeaf
 * (src/kdtree.hpp:126-152). */
int tk_tree_get_splits(const tk_tree* tree, void* medians, int32_t* leaf_offsets);

/* Launch-shape options for a query.  Zero-initialise and set what you need;
 * NULL means all defaults. */
typedef struct tk_query_opts {
    int32_t threads_per_query; /* 0 = auto, else 1, 2, 4, 8, 16 or 32 lanes per query */
    int32_t bin_queries;       /* -1 = auto (on from one wave of queries, SMs x 1024), 0 = off,
                                  1 = on: queries ordered by tree cell (1-3-D trees: costliest
                                  cost class first, cell order within a class) */
    int32_t smem_levels;       /* -1 = auto, else top split levels staged in shared memory */
    int32_t block_threads;     /* reserved, 0 (the KD kernel runs 256-thread blocks) */
    int32_t blocks_per_sm;     /* 0 = as many as fit */
    void* kernel_start_event;  /* optional cudaEvent_t recorded right before the KD kernel */
    void* kernel_stop_event;   /* optional cudaEvent_t recorded right after it */
    int32_t prune_boxes;       /* trees of 4-8 dims: -1 = auto (on), 0 = split planes only, 1 = also
                                  node bounding boxes; trees of 1-3 dims always prune with both */
    int32_t traversal;         /* 0 = auto (per-query), 1 = per-query search (G lanes per query),
                                  2 = warp packets: the 32 queries of a warp walk the tree together,
                                  one lane each, pruning with node boxes (k <= 16; larger k falls
                                  back to 1; threads_per_query and prune_boxes are then ignored) */
} tk_query_opts;

/* Bytes of device scratch tk_tree_query needs for nq queries. */
size_t tk_tree_query_workspace_size(const tk_tree* tree, int64_t nq);

/* Exact k nearest neighbours of nq device-resident query points.
 * q: device [nq, dims] (tree dtype); dists: device [nq, k] squared
 * distances (tree dtype); idx: device int32 [nq, k] original indices.
 * 1 <= k <= min(n, 128).  Asynchronous on `stream`.
 * Replaces KDTree::query (src/interface.cpp:60-86) ->
 * KDTreeKNNGPUSearch (src/kdtree_g.cu:410-457). */
int tk_tree_query(const tk_tree* tree, const void* q, int64_t nq, int k, void* dists, int32_t* idx,
                  const tk_query_opts* opts, void* workspace, size_t workspace_bytes, void* stream);

/* Transfers of tk_tree_query_host. */
#define TK_HOST_AUTO 0   /* direct when both result buffers are registered host memory, else staged */
#define TK_HOST_DIRECT 1 /* the query kernel writes the results into the host buffers itself */
#define TK_HOST_STAGED 2 /* results to device staging, downloaded after the search */

/* Exact k nearest neighbours with the queries and results in HOST memory:
 * q host [nq, dims] (tree dtype), dists host [nq, k], idx host int32
 * [nq, k].  The queries are uploaded into device staging with one copy.
 * When the result buffers are registered (pinned: cudaHostAlloc /
 * cudaHostRegister) memory the GPU addresses, the query kernel writes the
 * results straight into them over the host link while it searches
 * (TK_HOST_DIRECT; TK_EINVAL when they are not registered); otherwise they
 * are downloaded from device staging after the search (TK_HOST_STAGED).
 * Synchronous on `stream`: returns when the results are in host memory.
 * Device staging and workspace are allocated on first use and kept, grown as
 * needed, until tk_tree_destroy; calls on one tree are serialised.  Results
 * are identical to tk_tree_query's; device or mixed buffers work too (the
 * copies take their direction from the pointers).  Replaces the host-tensor use of
 * TorchKDTree.query (torch_kdtree/nn_distance.py:80 copies the queries to
 * the device; the caller copies the results back). */
int tk_tree_query_host(const tk_tree* tree, const void* q, int64_t nq, int k, void* dists, int32_t* idx,
                       const tk_query_opts* opts, int transfer, void* stream);

/* Exact KNN computed on the host, for a tree built on the host
 * (tk_tree_create, any device ordinal including -1; a tree built with
 * tk_tree_create_device keeps no host layout: TK_EINVAL).  q host
 * [nq, dims], dists host [nq, k], idx host int32 [nq, k]: the same results,
 * bit for bit, as tk_tree_query of the same tree (reference distance
 * arithmetic, original indices, lower index among equal distances).  Any
 * 1 <= k <= n.  n_threads: host threads (0 = all hardware threads).
 * Blocking; no CUDA call.  Replaces the query of the pybind class
 * KDTreeCPU<dims>[F] (src/interface.cpp:60-86 -> KDTreeKNNSearch,
 * src/kdtree.cpp:164-194). */
int tk_tree_query_cpu(const tk_tree* tree, const void* q, int64_t nq, int k, void* dists, int32_t* idx,
                      int n_threads);

/* Largest query count tk_tree_query_noalloc accepts in one call. */
#define TK_NOALLOC_MAX_QUERIES 262144

/* tk_tree_query without a caller workspace and without any allocation.
 * No counterpart in the reference: it exists for callers that cannot call
 * cudaMalloc on their query path -- hosts whose device memory belongs to
 * another allocator, plain C/FFI callers with no device allocator of their
 * own, and latency-critical code where cudaMalloc (which synchronises the
 * device) is not acceptable.  Scratch comes from a static device array of
 * about 4.4 MiB built into the library (held on every GPU that loads it until
 * the process exits).  At most TK_NOALLOC_MAX_QUERIES queries per call; more
 * fails with TK_EINVAL.  Every call on a device shares that array: calls that
 * may overlap on the GPU (different streams, or threads without ordering)
 * race and must be serialised by the caller.  The first call on a device
 * looks up the array's device address; make that first call before any
 * stream capture.  Results are identical to tk_tree_query's. */
int tk_tree_query_noalloc(const tk_tree* tree, const void* q, int64_t nq, int k, void* dists, int32_t* idx,
                          const tk_query_opts* opts, void* stream);

/* ------------------------------------------------------------ batches -- */

typedef struct tk_batch tk_batch;

/* Plan a batched query over n_trees clouds, each with its own tree (same
 * dtype, dims and device; dims 1..8) and its own k (ks[c], 1..min(n_c,
 * 128)); query
 * counts per cloud are fixed by q_counts.  The trees must outlive the batch.
 * Queries are passed concatenated cloud after cloud ([sum q_counts, dims]);
 * results come back concatenated the same way, cloud c occupying a
 * [q_counts[c], ks[c]] block.  No reference counterpart: the reference
 * queried one cloud per call (src/interface.cpp:79-86). */
int tk_batch_create(const tk_tree* const* trees, int n_trees, const int64_t* q_counts, const int32_t* ks,
                    tk_batch** out);
int tk_batch_destroy(tk_batch* batch);
size_t tk_batch_workspace_size(const tk_batch* batch);
/* Number of output elements (sum of q_counts[c] * ks[c]). */
int64_t tk_batch_output_size(const tk_batch* batch);
/* All clouds in one persistent launch fed by a global work counter (plus
 * the binning kernels).  Device work only, no host synchronisation and no
 * allocation: it can be captured in a CUDA graph.  threads_per_query: 0 =
 * auto, 1 (max k <= 16), or 8 / 32 (any k): trees of 1-3 dims run groups
 * of 8 lanes, trees of 4-8 dims groups of 32 (their kernels' shapes).
 * prune_boxes: trees of 1-3 dims always prune with node bounding boxes
 * (the argument is kept for binary compatibility); trees of 4-8 dims too. */
int tk_batch_query(const tk_batch* batch, const void* q, void* dists, int32_t* idx, int threads_per_query,
                   int prune_boxes, void* workspace, size_t workspace_bytes, void* stream);

/* -------------------------------------------------------- brute force -- */

typedef enum tk_brute_mode {
    TK_BRUTE_EXACT = 0,      /* CUDA cores, the reference's distance arithmetic (float or double) */
    TK_BRUTE_TF32 = 1,       /* q.r on tensor cores in TF32, over-fetch, exact FP32 re-rank */
    TK_BRUTE_BF16_SPLIT = 2  /* q.r as BF16 hi/lo split products with FP32 accumulation, then exact re-rank */
} tk_brute_mode;

/* Bytes of device scratch tk_nn_distance needs. */
size_t tk_nn_distance_workspace_size(int64_t n, int64_t nq, int dims, int k, int dtype, int mode);

/* Exhaustive exact k nearest neighbours (the nn_distance op).
 * ref: device [n, dims]; q: device [nq, dims]; dists [nq, k] squared
 * distances, idx int32 [nq, k]; 1 <= dims <= 128 (float32 or float64),
 * 1 <= k <= min(n, 128).  Every mode returns the same answer as the KD-tree
 * query: ordered by (distance computed as the reference does, index).
 * Replaces NmDistanceKernelLauncherDynamic (src/nndistance_g.cu:191-220),
 * which had no Python binding, ran one thread block and only d = 3. */
int tk_nn_distance(const void* ref, int64_t n, const void* q, int64_t nq, int dims, int k, int dtype, int mode,
                   void* dists, int32_t* idx, void* workspace, size_t workspace_bytes, void* stream);

/* What the last tk_nn_distance call made with `workspace` met on the
 * device, read back from that workspace after the call has completed
 * (synchronise its stream first); pass the same shape arguments as that
 * call.  *flags: bit 0 = a bounded device-side wait of the tensor-core
 * kernel ran out, bit 1 = an input lay outside the tensor-core
 * certificate's range; *recomputed = queries the exact kernel recomputed
 * (all of them for k > 32 with dims > 32, where the candidate search's
 * shared memory would not fit a block).
 * The answer is exact in every case: an unfinished or uncertifiable
 * candidate search only sends its queries to the exact kernel.  Returns
 * TK_ETIMEOUT when bit 0 is set, else TK_OK; TK_BRUTE_EXACT calls report
 * zeros.  Replaces the reference's exit() on a device error
 * (src/cutils.cuh:34-43), which left the caller nothing to inspect. */
int tk_nn_distance_report(const void* workspace, int64_t n, int64_t nq, int dims, int k, int dtype, int mode,
                          int* flags, int* recomputed);

/* Poll budget of every bounded device-side wait (the mbarrier waits of the
 * tensor-core brute force); 0 = the default (2^22 polls, far beyond any
 * wait that completes).  A small budget makes the waits run out on purpose:
 * host-side fault injection for tests of the time-out path, whose answers
 * stay exact (see tk_nn_distance_report).  Process-wide, for later calls;
 * returns the previous value.  No counterpart in the reference. */
uint32_t tk_set_device_wait_limit(uint32_t polls);

/* ----------------------------------------------------------- backward -- */

/* Bytes of device scratch tk_knn_backward needs when grad_ref is requested. */
size_t tk_knn_backward_workspace_size(int64_t nq, int k, int64_t n);

/* Gradient of squared KNN distances dist[i,j] = |q[i] - ref[idx[i,j]]|^2:
 *   grad_q[i]   = sum_j 2 g[i,j] (q[i] - ref[idx[i,j]])
 *   grad_ref[m] = sum over pairs with idx[i,j] == m of 2 g[i,j] (ref[m] - q[i])
 * q [nq,dims], ref [n,dims] (1 <= dims <= 128), idx int32 [nq,k] (original indices; entries
 * outside [0,n) are skipped), grad_dists [nq,k]; grad_q [nq,dims] and
 * grad_ref [n,dims] are overwritten; either may be NULL to skip it.  The ref
 * gradient is a segmented reduction over idx, bitwise identical run to run
 * without float atomics: for float32 with dims <= 8 each segment's terms are
 * summed exactly as 64-bit fixed-point integers scaled to the segment's
 * largest exponent (order-independent, one final rounding); otherwise the
 * segments come from a stable sort and are summed in pair order.
 * nq * k < 2^31.
 * Replaces the torch re-gather + autograd of torch_kdtree/nn_distance.py:111-112
 * (index_put_ with accumulate, float atomics). */
int tk_knn_backward(const void* q, const void* ref, const int32_t* idx, const void* grad_dists, int64_t nq,
                    int64_t n, int k, int dims, int dtype, void* grad_q, void* grad_ref, void* workspace,
                    size_t workspace_bytes, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* TK_KNN_H */
