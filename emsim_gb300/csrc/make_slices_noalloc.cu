// emsim_gb300_make_slices_noalloc: projected-potential slices from histograms without a
// caller-provided workspace and without allocating.
//
// Some callers cannot allocate device memory at the moment they need slices: a plugin
// running inside a host program that owns all device memory through its own pool
// allocator, or a tight loop that must not allocate after start-up (cudaMalloc and
// cudaFree can synchronise the whole device).  For them this entry point does what
// emsim_gb300_make_slices does, but keeps the complex intermediate in one fixed,
// file-scope device buffer.  It calls no cudaMalloc, cudaFree or allocating library
// routine; the slice plan, created once up front, still owns its own tables.
//
// Rules of the shared buffer:
//  * its size is EMSIM_GB300_NOALLOC_SCRATCH_BYTES (32 MiB); a plan whose
//    emsim_gb300_make_slices_workspace_size is larger is rejected with
//    EMSIM_GB300_ERR_UNSUPPORTED before any work is queued;
//  * every GPU that loads this part of the library may keep the buffer until the
//    process exits;
//  * every call on a device uses the same buffer, which keeps whatever the previous call
//    left there; nothing in it has to start at zero (a call writes every byte it later
//    reads), but two calls that overlap on the GPU (unordered streams) race on it;
//  * the buffer's device address is looked up once per device, by the first call made
//    with that device current (cudaGetSymbolAddress); make that first call before any
//    stream capture.  A call whose plan belongs to another device is refused before that
//    look-up, so it reserves nothing on the wrong device;
//  * the looked-up address, like every plan, belongs to the device's context:
//    cudaDeviceReset invalidates it, and the entry point must not be called on a device
//    after that device was reset.
#include <mutex>

#include "common.cuh"
#include "slice_plan.h"

// The name is a host-side stand-in in host code: kernels only ever receive the device
// address that cudaGetSymbolAddress returns for it.
static __device__ __align__(256) unsigned char g_make_slices_scratch[EMSIM_GB300_NOALLOC_SCRATCH_BYTES];

namespace {

constexpr int MAX_DEVICES = 64;
std::mutex g_scratch_mu;
void* g_scratch_addr[MAX_DEVICES] = {};

}  // namespace

extern "C" int emsim_gb300_make_slices_noalloc(emsim_gb300_slice_plan* plan, const float* hist, float* out,
                                               void* stream) {
    using emsim_gb300::set_error;
    EMSIM_REQUIRE(plan != nullptr && hist != nullptr && out != nullptr, EMSIM_GB300_ERR_INVALID,
                  "make_slices_noalloc: null plan, histogram or output");
    EMSIM_TRY(emsim_gb300::check_slice_device(plan));
    const size_t need = emsim_gb300_make_slices_workspace_size(plan);
    if (need > (size_t)EMSIM_GB300_NOALLOC_SCRATCH_BYTES) {
        set_error("make_slices_noalloc: this plan needs " + std::to_string(need) +
                  " bytes of scratch, more than the static buffer's " +
                  std::to_string((size_t)EMSIM_GB300_NOALLOC_SCRATCH_BYTES) +
                  "; call emsim_gb300_make_slices with a workspace instead");
        return EMSIM_GB300_ERR_UNSUPPORTED;
    }
    int dev = -1;
    EMSIM_CHECK_CUDA(cudaGetDevice(&dev));
    EMSIM_REQUIRE(dev >= 0 && dev < MAX_DEVICES, EMSIM_GB300_ERR_UNSUPPORTED,
                  "make_slices_noalloc: device index above 63");
    void* scratch = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_scratch_mu);
        if (g_scratch_addr[dev] == nullptr) {
            void* addr = nullptr;
            const cudaError_t e = cudaGetSymbolAddress(&addr, g_make_slices_scratch);
            if (e != cudaSuccess || addr == nullptr) {
                set_error(std::string("make_slices_noalloc: cudaGetSymbolAddress of the static buffer failed: ") +
                          cudaGetErrorString(e));
                return EMSIM_GB300_ERR_CUDA;
            }
            g_scratch_addr[dev] = addr;
        }
        scratch = g_scratch_addr[dev];
    }
    return emsim_gb300_make_slices(plan, hist, out, scratch, (size_t)EMSIM_GB300_NOALLOC_SCRATCH_BYTES, stream);
}
