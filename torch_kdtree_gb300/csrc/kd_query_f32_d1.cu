// KD query kernels for float, 1 dimension(s).
#include <string>

#include "kd_query.cuh"

namespace tk {
#define TK_T float
#define TK_D 1
#define TK_GR_LIST(X) X(1, 1) X(1, 2) X(1, 4) X(1, 8) X(1, 16) X(4, 1) X(4, 2) X(4, 4) X(4, 8) X(4, 16) X(32, 1) X(32, 2) X(32, 4)
#include "kd_query_inst.inc"
}  // namespace tk
