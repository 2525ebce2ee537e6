// tcgen05 candidate search, TF32 operands, rows of 32 and 40 (see brute_tc_kernels.cuh).
#include "brute_tc_kernels.cuh"

namespace tk {
namespace tcx {

int tc5_dispatch_tf32_deep(const Tc5Args& a, int KP, int CH, int qblocks, cudaStream_t s) {
    switch (KP) {
        case 32: return tc5_dispatch_ch<TK_BRUTE_TF32, 32>(a, CH, qblocks, s);
        case 40: return tc5_dispatch_ch<TK_BRUTE_TF32, 40>(a, CH, qblocks, s);
        default: return fail(TK_EUNSUPPORTED, "tcgen05 path: unsupported depth");
    }
}

}  // namespace tcx
}  // namespace tk
