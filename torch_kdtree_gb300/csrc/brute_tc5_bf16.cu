// tcgen05 candidate search, BF16 hi/lo split operands (see brute_tc_kernels.cuh).
#include "brute_tc_kernels.cuh"

namespace tk {
namespace tcx {

int tc5_dispatch_bf16(const Tc5Args& a, int KP, int CH, int qblocks, cudaStream_t s) {
    switch (KP) {
        case 16: return tc5_dispatch_ch<TK_BRUTE_BF16_SPLIT, 16>(a, CH, qblocks, s);
        case 32: return tc5_dispatch_ch<TK_BRUTE_BF16_SPLIT, 32>(a, CH, qblocks, s);
        case 48: return tc5_dispatch_ch<TK_BRUTE_BF16_SPLIT, 48>(a, CH, qblocks, s);
        default: return fail(TK_EUNSUPPORTED, "tcgen05 path: unsupported depth");
    }
}

}  // namespace tcx
}  // namespace tk
