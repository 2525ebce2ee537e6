// Batched-query kernels of 4-8 dimensional trees for float (see batch_wide.cuh).
#include <string>

#include "batch_wide.cuh"

namespace tk {

#define TK_BW_LIST(X) X(4, 1) X(4, 32) X(6, 1) X(6, 32) X(8, 1) X(8, 32)

template <>
const void* batch_wide_kernel<float>(int W, int G) {
#define TK_BWPTR(w, g) \
    if (W == w && G == g)                                                                \
        return g == 1 ? reinterpret_cast<const void*>(&k_batch_query_wide1<float, w>)        \
                      : reinterpret_cast<const void*>(&k_batch_query_wide32<float, w>);
    TK_BW_LIST(TK_BWPTR)
#undef TK_BWPTR
    return nullptr;
}

template <>
int batch_wide_launch<float>(const WideBatchArgs<float>& a, int W, int G, int grid, cudaStream_t s) {
    bool launched = false;
#define TK_BWLAUNCH(w, g)                                        \
    if (!launched && W == w && G == g) {                         \
        if (g == 1) k_batch_query_wide1<float, w><<<grid, 256, 0, s>>>(a);                   \
        else k_batch_query_wide32<float, w><<<grid, 256, 0, s>>>(a);                        \
        launched = true;                                         \
    }
    TK_BW_LIST(TK_BWLAUNCH)
#undef TK_BWLAUNCH
    if (!launched) return fail(TK_EUNSUPPORTED, "no batched kernel for this record width / lanes");
    const cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) return fail(TK_ECUDA, std::string("batch launch: ") + cudaGetErrorString(err));
    return TK_OK;
}

template <>
void batch_wide_bin_launch<float>(const WideBatchArgs<float>& a, int* counts, int* bin_of, int* pos_of, cudaStream_t s) {
    k_batch_bin_count_wide<float><<<(a.total + 255) / 256, 256, 0, s>>>(a, counts, bin_of, pos_of);
}

}  // namespace tk
