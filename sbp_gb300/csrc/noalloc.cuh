// Allocation-free staging for sbpgpu_delta_mdl_batch_noalloc (see noalloc.cu).
#pragma once

#include <cstdint>
#include <string>

#include <cuda_runtime.h>

namespace sbp {

// Largest batch of the allocation-free delta-MDL entry point, and its staging size:
// int32 vertex ids, int32 proposals and int64 results for every entry (1 MiB).
constexpr int64_t kNoAllocMaxBatch = 65536;
constexpr size_t kNoAllocScratchBytes = (size_t)kNoAllocMaxBatch * (4 + 4 + 8);

struct NoAllocScratch {
    int32_t* vertex;
    int32_t* proposal;
    long long* result;  // converted in place to double before it is copied out
};

// The staging array of `device`: its address is looked up once per device (with that
// device current) and cached.  Returns false with a message when the lookup fails.
bool noalloc_scratch(int device, NoAllocScratch* out, std::string* err);

// result[i] (units of 2^-24) -> double, in place.
void launch_fixed_to_double(long long* v, int64_t n, cudaStream_t st);

}  // namespace sbp
