// Inline-PTX helpers for TMA staging on sm_103a: mbarriers with bounded waits, 1-D bulk
// copies and 2-D tensor copies global -> shared.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <cstdint>

namespace emsim_gb300 {
namespace tma {

// device error word written by kernels whose barrier waits time out (see check_error)
enum DeviceError : int { DEV_OK = 0, DEV_MBAR_TIMEOUT = 1 };

// default limit of a bounded mbarrier wait (ns of global time); kernels get the limit in
// their arguments (RowArgs / ColArgs::wait_ns, emsim_gb300_set_wait_limit_ns)
constexpr unsigned long long DEFAULT_WAIT_LIMIT_NS = 2000000000ull;
// the shortest limit the C ABI accepts for the pipelined kernels
constexpr unsigned long long MIN_WAIT_LIMIT_NS = 1000000ull;

// Record a device error code in the error word (mapped page-locked host memory, one word
// per device: the host reads it without synchronising the device).
__device__ __forceinline__ void record_error(int* err, int code) {
    if (err) {
        *reinterpret_cast<volatile int*>(err) = code;
        __threadfence_system();
    }
}

// Programmatic dependent launch.  A kernel launched with programmatic stream
// serialisation may start while the kernel before it in the stream still runs: it does
// its set-up (barriers, shared-memory tables computed at plan creation), then pdl_wait()
// blocks until every preceding kernel of the stream has completed and its writes are
// visible, before any global data of the chain is read or written.  pdl_launch_dependents()
// lets the next kernel of the stream launch early; it is called after pdl_wait(), so a
// kernel that starts early knows that all kernels before its predecessor have completed.
// Without the launch attribute both are no-ops.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;" :::); }

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// make mbarrier initialisation visible to the async (TMA) proxy
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

// order this CTA's generic-proxy shared-memory accesses before later async-proxy ones
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// try_wait that may suspend the thread for up to `hint_ns` (it resumes when the phase
// completes), so a waiting warp takes no issue slots from the warps that have work
__device__ __forceinline__ bool mbar_try_wait_suspend(uint64_t* bar, uint32_t parity, uint32_t hint_ns) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity), "r"(hint_ns)
        : "memory");
    return ok != 0;
}

// Wait for the phase with the given parity, suspending between polls; false after
// limit_ns of global time without completion.
__device__ __forceinline__ bool mbar_wait_suspend(uint64_t* bar, uint32_t parity,
                                                  unsigned long long limit_ns = DEFAULT_WAIT_LIMIT_NS) {
    const uint64_t t0 = global_ns();
    for (;;) {
        if (mbar_try_wait_suspend(bar, parity, 100000u)) return true;
        if (global_ns() - t0 > limit_ns) return false;
    }
}

// Wait for the phase with the given parity; false after limit_ns of global time without
// completion.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity,
                                          unsigned long long limit_ns = DEFAULT_WAIT_LIMIT_NS) {
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = global_ns();
    for (;;) {
#pragma unroll 1
        for (int i = 0; i < 64; ++i)
            if (mbar_try_wait(bar, parity)) return true;
        if (global_ns() - t0 > limit_ns) return false;
    }
}

// After a wait gave up: wait for a copy of this CTA that is still in flight with at least
// the default limit, so that it lands before the CTA's shared memory is released.
__device__ __forceinline__ void mbar_drain(uint64_t* bar, uint32_t parity, unsigned long long limit_ns) {
    mbar_wait(bar, parity, limit_ns > DEFAULT_WAIT_LIMIT_NS ? limit_ns : DEFAULT_WAIT_LIMIT_NS);
}

// contiguous global -> shared copy of `bytes` (multiple of 16, both addresses 16-byte
// aligned), completing on `bar`
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

// 2-D tiled tensor copy of one box at element coordinates (x, y), completing on `bar`
__device__ __forceinline__ void tensor_g2s_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
        "[%4];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

// 2-D tiled tensor copy of one box from shared memory to global element coordinates
// (x, y) (both >= 0, x * element size a multiple of 16 bytes), in the issuing thread's
// bulk async-group
__device__ __forceinline__ void tensor_s2g_2d(const CUtensorMap* map, int x, int y, const void* src) {
    asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%1, %2}], [%3];" ::"l"(
                     reinterpret_cast<uint64_t>(map)),
                 "r"(x), "r"(y), "r"(smem_u32(src))
                 : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// the issuing thread's bulk groups: wait until at most N of them still read shared memory
// (READ) or are incomplete; they are the thread's own copies, which always finish
template <int N>
__device__ __forceinline__ void bulk_wait_read() {
    asm volatile("cp.async.bulk.wait_group.read %0;" ::"n"(N) : "memory");
}
template <int N>
__device__ __forceinline__ void bulk_wait() {
    asm volatile("cp.async.bulk.wait_group %0;" ::"n"(N) : "memory");
}

}  // namespace tma
}  // namespace emsim_gb300
