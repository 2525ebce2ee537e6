// Device-wide primitives written for this engine: an exclusive prefix sum and
// a stable LSD radix sort of (uint32 key, uint32 value) pairs.  The sort is
// stable, so pairs entered in ascending value order come out ordered by
// (key, value): this is what makes the backward reduction deterministic.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace tk {

// Scratch bytes for exclusive_scan over n ints.
size_t scan_workspace_bytes(int64_t n);
// In-place exclusive prefix sum of data[0..n).  Returns a cudaError_t.
cudaError_t exclusive_scan(int* data, int64_t n, void* ws, cudaStream_t s);

// Scratch bytes for sort_pairs over n pairs (excluding the two output arrays).
size_t sort_workspace_bytes(int64_t n);
// Stable sort of n (key, value) pairs by the low `key_bits` bits of the key.
// keys_in / vals_in are read only; the sorted result is written to
// keys_out / vals_out.  If vals_in is null the values are 0..n-1.
cudaError_t sort_pairs(const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out, uint32_t* vals_out,
                       int64_t n, int key_bits, void* ws, size_t ws_bytes, cudaStream_t s);

// One stable pass over 8-bit keys (key < 256): the same pass as sort_pairs
// with key_bits = 8, without its ping-pong buffers.  Scratch bytes:
size_t sort_pass8_workspace_bytes(int64_t n);
cudaError_t sort_pass8(const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out, uint32_t* vals_out,
                       int64_t n, void* ws, size_t ws_bytes, cudaStream_t s);

}  // namespace tk
