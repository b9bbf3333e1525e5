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
// and it keeps the previous call's contents.  It holds pobtaf's workspace,
// whose three regions are each made safe to reuse by the call itself:
//
//   * the status word (first 4 bytes): cleared by a memset at the start of
//     every call;
//   * the barrier and column counters of the persistent column-block
//     kernel: cleared by a memset before every launch of that kernel;
//   * the column-block kernel's staging buffers and published columns: the
//     factorizer CTA resets every staging element to a sentinel on entry,
//     before any other CTA can see a column counter move, and every
//     published column is written before its counter is raised; the
//     launch-based tile sweep (small blocks) writes its 32 x 32 tile
//     scratch before reading it.
//
// So leftover contents from an earlier call are never read as data.  Two
// calls that overlap on the GPU (different streams, or different host
// threads on one device) race on the array and must be serialised by the
// caller.
//
// A bounded wait that gives up inside the column-block kernel sets the
// status word; that word lives in the private array, so after the sweep a
// one-thread kernel copies a non-zero status into the caller's `info` word
// as -SGB_ERR_TIMEOUT (info > 0 keeps its meaning: the failing pivot row).
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

// A timeout recorded in the private status word becomes -SGB_ERR_TIMEOUT in
// the caller's info word.
__global__ void k_status_to_info(const int32_t* status, int32_t* info) {
    const int32_t s = *status;
    if (s != 0) *info = -s;
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
    rc = sgb_pobtaf(m, factorize_last_block, SGB_PREC_NATIVE, scratch, kStaticScratchBytes, info, stream);
    if (rc != SGB_OK || info == nullptr) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    sgb::prof_before(s);
    k_status_to_info<<<1, 1, 0, s>>>((const int32_t*)scratch, info);
    const cudaError_t e = cudaGetLastError();
    sgb::prof_after(-1, s, 0.0);
    return e == cudaSuccess ? SGB_OK : sgb::record_cuda_error(e);
}

}  // extern "C"
