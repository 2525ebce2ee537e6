// Tensor-core brute force: not implemented yet in this build.
#include "brute_tc.cuh"
#include "tk_internal.h"

namespace tk {

size_t brute_tc_workspace_bytes(int64_t, int64_t, int, int, int) { return 256; }

int run_brute_tc(const float*, int64_t, const float*, int64_t, int, int, int, float*, int32_t*, void*, size_t,
                 cudaStream_t) {
    return fail(TK_EUNSUPPORTED, "tensor-core brute force is not available in this build");
}

}  // namespace tk
