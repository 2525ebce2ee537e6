// Exhaustive exact KNN in float64 for 5 to 128 dimensions (see brute.cuh); a
// unit of its own so that it compiles in parallel with brute.cu.  FP64 stays
// FP64 end to end; on GB300 it is a correctness path, not a fast one.
#include "brute.cuh"

namespace tk {

int launch_brute_f64_wide(const BruteArgs<double>& a, const BrutePlan& p, cudaStream_t s) {
    switch (p.DP) {
        case 8: return launch_dp<double, 8>(a, p, s);
        case 16: return launch_dp<double, 16>(a, p, s);
        case 32: return launch_dp<double, 32>(a, p, s);
        case 64: return launch_dp<double, 64>(a, p, s);
        case 128: return launch_dp<double, 128>(a, p, s);
        default: return fail(TK_EUNSUPPORTED, "no brute-force kernel for this dimension");
    }
}

}  // namespace tk
