// pobtaf for callers that cannot allocate device memory.
//
// Some callers have no way to obtain device scratch: code that runs while
// a CUDA stream is being captured (cudaMalloc is not a stream operation and
// breaks or is refused inside capture), real-time loops that forbid
// allocator calls, and foreign-language hosts (Go, Java, Fortran) that hold
// plain device pointers but no handle on the application's allocator.
// sgb_pobtaf_noalloc serves them: its scratch is a file-scope static
// __device__ array, so the call allocates nothing.
//
// The array costs kStaticScratchBytes of device memory on every GPU that
// loads this library, for the lifetime of the process.  All calls share it
// and it keeps the previous call's contents; pobtaf overwrites every byte it
// reads before reading it (the 32 x 32 tile inverse), so nothing needs
// clearing.  Two calls that overlap on the GPU (different streams, or
// different host threads on one device) race on the array and must be
// serialised by the caller.
#include <mutex>

#include "sgb_internal.cuh"

namespace {

constexpr size_t kStaticScratchBytes = 128 * 1024;
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_pobtaf_scratch[kStaticScratchBytes];

std::mutex g_mu;
void* g_scratch_addr[kMaxDevices] = {};

// Device address of g_pobtaf_scratch on the current device.  The host-side
// symbol is only a stand-in; the address must come from
// cudaGetSymbolAddress, taken once per device with that device current.
int scratch_address(void** out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return SGB_ERR_CUDA;
    if (dev < 0 || dev >= kMaxDevices) return SGB_ERR_UNSUPPORTED;
    std::lock_guard<std::mutex> lk(g_mu);
    if (g_scratch_addr[dev] == nullptr) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_pobtaf_scratch);
        if (e != cudaSuccess || p == nullptr) return SGB_ERR_CUDA;
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
    return SGB_OK;
}

}  // namespace

extern "C" {

size_t sgb_pobtaf_noalloc_scratch_bytes(void) { return kStaticScratchBytes; }

int sgb_pobtaf_noalloc(const sgb_bta* m, int factorize_last_block, int32_t* info, void* stream) {
    size_t need = 0;
    int rc = sgb_pobtaf_workspace_size(m, SGB_PREC_NATIVE, &need);
    if (rc != SGB_OK) return rc;
    if (need > kStaticScratchBytes) return SGB_ERR_WORKSPACE;
    void* scratch = nullptr;
    rc = scratch_address(&scratch);
    if (rc != SGB_OK) return rc;
    return sgb_pobtaf(m, factorize_last_block, SGB_PREC_NATIVE, scratch, kStaticScratchBytes, info, stream);
}

}  // extern "C"
