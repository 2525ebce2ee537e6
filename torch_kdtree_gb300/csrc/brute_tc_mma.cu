// mma.sync candidate search (rows deeper than the tcgen05 kernels take, or
// k > 32), both operand modes (see brute_tc_kernels.cuh).
#include "brute_tc_kernels.cuh"

namespace tk {
namespace tcx {

int tc_select_dispatch(const TcArgs& a, int mode, int qblocks, cudaStream_t s) {
    return mode == TK_BRUTE_TF32 ? dispatch_kp<TK_BRUTE_TF32>(a, qblocks, s)
                                 : dispatch_kp<TK_BRUTE_BF16_SPLIT>(a, qblocks, s);
}

}  // namespace tcx
}  // namespace tk
