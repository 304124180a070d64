// Device-wide primitives of the sbpgpu library: exclusive / inclusive scan of int32
// and a stable LSD radix sort of 64-bit keys with optional int32 values.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace sbp {

struct Scratch;  // host-side bookkeeping of preallocated device buffers

// Temporary bytes needed by scan_i32 for n elements.
size_t scan_temp_bytes(int64_t n);
// out[i] = sum(in[0..i)) (exclusive) or sum(in[0..i]) (inclusive).  in may equal out.
// Writes the grand total to *d_total if non-null (device pointer).
void scan_i32(const int32_t* in, int32_t* out, int64_t n, bool inclusive, int32_t* d_total, void* temp,
              cudaStream_t st);

// Temporary bytes needed by radix_sort for n keys.
size_t radix_temp_bytes(int64_t n);
// Stably sorts (keys, vals) by bits [0, end_bit) of the keys.  keys_alt/vals_alt are
// ping-pong buffers of the same size; the sorted data ends in the primary buffers.
// vals may be null.
void radix_sort_u64(uint64_t* keys, uint64_t* keys_alt, int32_t* vals, int32_t* vals_alt, int64_t n,
                    int end_bit, void* temp, cudaStream_t st);

// Launch count of the last primitive calls (for kernel-launch accounting).
int64_t prims_launch_count();

}  // namespace sbp
