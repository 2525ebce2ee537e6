// Internal host-side declarations shared by the library's translation units.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/tk_knn.h"

namespace tk {

constexpr int kMaxLevels = 24;   // 2^24 leaves; the stack of a traversal holds <= kMaxLevels entries
constexpr int kMaxK = 128;       // reference GPU cap (src/kdtree_g.cu:283,421)
constexpr int kMaxBinLevels = 16;
constexpr int kMaxDims = 8;      // KD-tree dimensions (brute force: up to 128)

// Coordinates per device point record of a tree of `dims` dimensions: up to
// 3 share one 16-byte record with the original index; 4 or 5-8 dimensions use
// 4 or 8 zero-padded coordinates with the indices in a separate array.
inline int record_width(int dims) { return dims <= 3 ? 3 : (dims <= 4 ? 4 : (dims <= 6 ? 6 : 8)); }

// Sets the thread-local error text and returns the status.
int fail(int status, const std::string& msg);

// Caller workspaces are carved into 256-byte aligned sub-buffers (some are
// read by bulk copies, which need 16-byte alignment), so the caller's pointer
// must be 256-byte aligned, as cudaMalloc's are.
inline bool ws_misaligned(const void* p) { return p && (reinterpret_cast<uintptr_t>(p) & 255) != 0; }
void clear_error();

// Host copy of a tree in the reference's layout (src/kdtree.hpp:126-217) plus
// the device image used by the kernels.
template <typename T>
struct HostTree {
    int64_t n = 0;
    int dims = 0;
    int levels = 0;
    std::vector<T> structured;        // [n*dims] points in leaf order
    std::vector<int32_t> perm;        // [n] original index of structured point i
    std::vector<T> medians;           // [2^L - 1] heap order; axis = depth % dims
    std::vector<int32_t> leaf_off;    // [2^L + 1] prefix offsets of the leaves
    // Tight bounding boxes of every node's points, heap order over all
    // 2^(L+1) - 1 nodes (leaves last), box_stride() coordinates each (unused
    // ones 0); empty nodes have lo = +inf, hi = -inf.
    std::vector<T> box_lo, box_hi;
    int box_stride() const { return record_width(dims); }
};

// Builds the tree (tree_build.cpp).  Returns TK_OK or sets the error.
template <typename T>
int build_host_tree(const T* pts, int64_t n, int dims, int levels, int n_threads, HostTree<T>& out);

// Takes over a saved layout (tree_build.cpp): validates it (leaf offsets,
// permutation, no NaN, every split separating its children) and computes
// the node boxes.  Returns TK_OK or sets the error.
template <typename T>
int tree_from_layout(const T* structured, const int32_t* perm, const T* medians, const int32_t* leaf_off, int64_t n,
                     int dims, int levels, HostTree<T>& out);

}  // namespace tk

struct tk_tree;

namespace tk {
// Streams, events and device staging of tk_tree_query_host (tk_api.cu),
// created on a tree's first host-buffer query.
struct HostPipe;
void free_host_pipe(HostPipe* p);
// Builds the tree on the GPU from device points straight into t's device
// image (tree_build_gpu.cu), same layout as build_host_tree.  The arguments
// are validated by the caller; runs on and synchronises the CUDA stream
// `stream` before returning.
template <typename T>
int build_device_tree(const T* pts, int64_t n, int dims, int levels, void* stream, tk_tree* t);
}  // namespace tk

// Opaque handle behind the C ABI.
struct tk_tree {
    int dtype = TK_F32;
    int dims = 0;
    int levels = 0;
    int device = 0;
    int64_t n = 0;
    // host layout (one of the two is filled when the tree was built on the
    // host; a tree built on the GPU keeps only its device image and the
    // layout getters copy from there)
    bool host_layout = true;
    tk::HostTree<float> h32;
    tk::HostTree<double> h64;
    // device image
    void* d_pts = nullptr;       // point records: coordinates + original index (see tk_device.cuh)
    void* d_medians = nullptr;   // T[2^L - 1]
    int32_t* d_leaf_off = nullptr;  // int32[2^L + 1]
    void* d_boxes = nullptr;     // per node {lo.xyz, 0}, {hi.xyz, 0} (see tk_device.cuh); lo / hi rows when wide
    int32_t* d_perm = nullptr;   // trees of 4-8 dims: original index of each point (records hold coordinates only)
    int64_t device_bytes = 0;
    mutable tk::HostPipe* pipe = nullptr;  // host-buffer query resources (see tk_tree_query_host)
};
