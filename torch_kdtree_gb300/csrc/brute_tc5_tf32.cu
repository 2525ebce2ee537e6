// tcgen05 candidate search, TF32 operands, rows of up to 24 (see brute_tc_kernels.cuh).
#include "brute_tc_kernels.cuh"

namespace tk {
namespace tcx {

int tc5_dispatch_tf32(const Tc5Args& a, int KP, int CH, int qblocks, cudaStream_t s) {
    switch (KP) {
        case 8: return tc5_dispatch_ch<TK_BRUTE_TF32, 8>(a, CH, qblocks, s);
        case 16: return tc5_dispatch_ch<TK_BRUTE_TF32, 16>(a, CH, qblocks, s);
        case 24: return tc5_dispatch_ch<TK_BRUTE_TF32, 24>(a, CH, qblocks, s);
        default: return tc5_dispatch_tf32_deep(a, KP, CH, qblocks, s);  // 32, 40
    }
}

}  // namespace tcx
}  // namespace tk
