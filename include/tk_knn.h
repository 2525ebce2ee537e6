/*
 * tk_knn.h -- C ABI of the GB300 KNN engine (libtkknn.so).
 *
 * Drop-in boundary for torch_kdtree's query path.  Every entry point takes
 * plain pointers and sizes, returns a tk_status, never exits the process and
 * never allocates device memory on a query path: scratch memory is passed in
 * by the caller (sizes from the *_workspace_size functions).  Device work is
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
 * host_points: [n, dims] C-contiguous, float or double per dtype.
 * levels: 1..24 (the reference's default heuristic is applied by the Python
 * layer).  device: CUDA ordinal, or -1 for a host-only tree (layout getters
 * only; queries on it fail with TK_EINVAL).  n_threads: host build threads
 * (0 = all hardware threads).  Fails with TK_EINVAL when a split node would receive no point
 * ("ran out of points"), like the reference.
 * Replaces the constructor of the pybind class KDTree<T,dims,use_gpu>
 * (src/interface.cpp:25-43): createKDTree (src/kdtree.hpp:494-534) +
 * copyPartitionToGPU (src/kdtree_g.cu:63-98). */
int tk_tree_create(const void* host_points, int64_t n, int dims, int dtype, int levels, int device,
                   int n_threads, tk_tree** out);

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
    int32_t bin_queries;       /* -1 = auto, 0 = off, 1 = reorder queries by tree cell */
    int32_t smem_levels;       /* -1 = auto, else top split levels staged in shared memory */
    int32_t block_threads;     /* reserved, 0 (the KD kernel runs 256-thread blocks) */
    int32_t blocks_per_sm;     /* 0 = as many as fit */
    void* kernel_start_event;  /* optional cudaEvent_t recorded right before the KD kernel */
    void* kernel_stop_event;   /* optional cudaEvent_t recorded right after it */
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

/* ----------------------------------------------------------- backward -- */

/* Bytes of device scratch tk_knn_backward needs when grad_ref is requested. */
size_t tk_knn_backward_workspace_size(int64_t nq, int k, int64_t n);

/* Gradient of squared KNN distances dist[i,j] = |q[i] - ref[idx[i,j]]|^2:
 *   grad_q[i]   = sum_j 2 g[i,j] (q[i] - ref[idx[i,j]])
 *   grad_ref[m] = sum over pairs with idx[i,j] == m of 2 g[i,j] (ref[m] - q[i])
 * q [nq,dims], ref [n,dims], idx int32 [nq,k] (original indices; entries
 * outside [0,n) are skipped), grad_dists [nq,k]; grad_q [nq,dims] and
 * grad_ref [n,dims] are overwritten; either may be NULL to skip it.  The ref
 * gradient is a stable-sort + fixed-order segmented reduction: bitwise
 * identical run to run.  nq * k < 2^31.
 * Replaces the torch re-gather + autograd of torch_kdtree/nn_distance.py:111-112
 * (index_put_ with accumulate, float atomics). */
int tk_knn_backward(const void* q, const void* ref, const int32_t* idx, const void* grad_dists, int64_t nq,
                    int64_t n, int k, int dims, int dtype, void* grad_q, void* grad_ref, void* workspace,
                    size_t workspace_bytes, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* TK_KNN_H */
