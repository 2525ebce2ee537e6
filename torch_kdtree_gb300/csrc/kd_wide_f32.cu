// KD query kernels of 4-8 dimensional trees for float (see kd_wide.cuh).
#include <string>

#include "kd_wide.cuh"

namespace tk {

#define TK_WIDE_LIST(X) \
    X(4, 1, 1) X(4, 1, 2) X(4, 1, 4) X(4, 1, 8) X(4, 1, 16) X(4, 32, 1) X(4, 32, 2) X(4, 32, 4) \
    X(6, 1, 1) X(6, 1, 2) X(6, 1, 4) X(6, 1, 8) X(6, 1, 16) X(6, 32, 1) X(6, 32, 2) X(6, 32, 4) \
    X(8, 1, 1) X(8, 1, 2) X(8, 1, 4) X(8, 1, 8) X(8, 1, 16) X(8, 32, 1) X(8, 32, 2) X(8, 32, 4)

template <>
const void* kd_wide_kernel<float>(int W, int G, int R) {
#define TK_WPTR(w, g, r) \
    if (W == w && G == g && R == r) return reinterpret_cast<const void*>(&k_kd_wide<float, w, g, r>);
    TK_WIDE_LIST(TK_WPTR)
#undef TK_WPTR
    return nullptr;
}

template <>
int kd_wide_launch<float>(const KdWideArgs<float>& a, int W, int G, int R, int grid, int block, size_t smem,
                        cudaStream_t s) {
    bool launched = false;
#define TK_WLAUNCH(w, g, r)                                                  \
    if (!launched && W == w && G == g && R == r) {                           \
        k_kd_wide<float, w, g, r><<<grid, block, smem, s>>>(a);                 \
        launched = true;                                                     \
    }
    TK_WIDE_LIST(TK_WLAUNCH)
#undef TK_WLAUNCH
    if (!launched) return fail(TK_EUNSUPPORTED, "no KD query kernel compiled for this width / lanes / registers");
    const cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) return fail(TK_ECUDA, std::string("KD query launch: ") + cudaGetErrorString(err));
    return TK_OK;
}

template <>
void bin_count_wide_launch<float>(const float* q, int nq, int dims, const float* medians, int B, int L, const float* boxes,
                                int W, int* counts, int* bin_of, int* pos_of, cudaStream_t s) {
    k_bin_count_wide<float><<<(nq + 255) / 256, 256, 0, s>>>(q, nq, dims, medians, B, L, boxes, W, counts, bin_of, pos_of);
}

}  // namespace tk
