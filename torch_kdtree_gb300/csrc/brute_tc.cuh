// Tensor-core brute force (declarations; see brute_tc.cu).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace tk {

size_t brute_tc_workspace_bytes(int64_t n, int64_t nq, int d, int k, int mode);
int run_brute_tc(const float* ref, int64_t n, const float* q, int64_t nq, int d, int k, int mode, float* dists,
                 int32_t* idx, void* ws, size_t ws_bytes, cudaStream_t s);

}  // namespace tk
