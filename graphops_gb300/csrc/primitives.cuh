// Device-wide building blocks used by the CSR build: exclusive prefix sum and
// a stable LSD radix sort of (key, value) pairs.  Both are integer-only and so
// bit-reproducible; the sort is stable, which is what makes the in-edge CSR
// list each node's in-edges in source order (the reference's scatter order).
#pragma once
#include "gops_internal.cuh"

namespace gops {

// out[i] = sum_{j<i} in[i]; out may alias in.  n may be 0.  Temporary storage
// comes from the stream-ordered allocator.
Status exclusive_scan_i64(const int64_t *in, int64_t *out, int64_t n, cudaStream_t s);
Status exclusive_scan_u32(const uint32_t *in, uint32_t *out, int64_t n, cudaStream_t s);

// Stable sort of (keys, vals) by the low `key_bits` bits of keys.  keys/vals
// and keys_alt/vals_alt are ping-pong buffers of n entries; on return
// *result_in_alt tells which pair holds the sorted sequence.
Status radix_sort_pairs_u32(uint32_t *keys, uint32_t *vals, uint32_t *keys_alt,
                            uint32_t *vals_alt, int64_t n, int key_bits,
                            bool *result_in_alt, cudaStream_t s);

// The same with the input read from `keys_in` (left unchanged) and the values
// being the input positions 0..n-1: keys/vals and keys_alt/vals_alt are only
// written.
Status radix_sort_index_u32(const uint32_t *keys_in, uint32_t *keys, uint32_t *vals, uint32_t *keys_alt,
                            uint32_t *vals_alt, int64_t n, int key_bits, bool *result_in_alt,
                            cudaStream_t s);

}  // namespace gops
