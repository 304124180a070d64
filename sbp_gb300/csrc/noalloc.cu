// Staging memory for the allocation-free delta-MDL batch (sbpgpu_delta_mdl_batch_noalloc).
//
// The batch's vertex ids, proposals and fixed-point results live in one file-scope device
// array of kNoAllocScratchBytes instead of buffers allocated per call.  The first call on a
// device looks up the array's address with cudaGetSymbolAddress while that device is
// current and keeps it for later calls; nothing here allocates device or host memory.
//
// Nothing in the array has to start at zero: a call writes every slot it later reads
// (the copied-in ids and proposals, then one result per batch entry).  Calls that overlap
// in time on the same device -- from two host threads, or two contexts whose streams run
// concurrently -- share the one array and race.
#include <mutex>
#include <string>

#include "kernels.cuh"
#include "noalloc.cuh"

namespace sbp {

namespace {

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
void* g_scratch_ptr[kMaxDevices] = {};

__global__ void k_fixed_to_double(long long* v, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const long long q = v[i];
        reinterpret_cast<double*>(v)[i] = (double)q * (1.0 / 16777216.0);
    }
}

}  // namespace

bool noalloc_scratch(int device, NoAllocScratch* out, std::string* err) {
    if (device < 0 || device >= kMaxDevices) {
        *err = "device ordinal outside the supported range";
        return false;
    }
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_ptr[device]) {
        int prev = -1;
        cudaError_t e = cudaGetDevice(&prev);
        if (e == cudaSuccess && prev != device) e = cudaSetDevice(device);
        void* p = nullptr;
        if (e == cudaSuccess) e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (prev >= 0 && prev != device) cudaSetDevice(prev);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            *err = std::string("cudaGetSymbolAddress of the staging array failed: ") + cudaGetErrorString(e);
            return false;
        }
        g_scratch_ptr[device] = p;
    }
    unsigned char* base = static_cast<unsigned char*>(g_scratch_ptr[device]);
    out->vertex = reinterpret_cast<int32_t*>(base);
    out->proposal = reinterpret_cast<int32_t*>(base + sizeof(int32_t) * kNoAllocMaxBatch);
    out->result = reinterpret_cast<long long*>(base + 2 * sizeof(int32_t) * kNoAllocMaxBatch);
    return true;
}

void launch_fixed_to_double(long long* v, int64_t n, cudaStream_t st) {
    if (n <= 0) return;
    const int64_t blocks = std::min<int64_t>((n + 255) / 256, device_sms() * 8);
    k_fixed_to_double<<<(unsigned)blocks, 256, 0, st>>>(v, n);
    count_launches(1);
}

}  // namespace sbp
