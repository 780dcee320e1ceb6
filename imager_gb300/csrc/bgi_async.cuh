// Bulk asynchronous copies (TMA, cp.async.bulk) and mbarriers, as inline PTX for sm_100+.
//
// Every wait is bounded: a wait that has not completed after kWaitCycles SM clock cycles (about
// 50 ms) records BGI_FAULT_ASYNC_WAIT in the device fault word and returns false, and the
// kernel then skips its work.  The host reads the word (bgi_device_fault in the C ABI).
#pragma once

#include <stdint.h>

namespace bgi {

constexpr unsigned BGI_FAULT_ASYNC_WAIT = 1u;
constexpr long long kWaitCycles = 100000000LL;

// Device fault word.  Each translation unit that includes this header has its own copy (the
// library is compiled without relocatable device code); the kernels that use these helpers and
// the host reader (read_device_fault) are all in bgi_fft.cu.
static __device__ unsigned int g_device_fault = 0;

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

// makes an initialised mbarrier visible to the async proxy
__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// orders this thread's shared-memory writes before later async-proxy reads of them
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return done != 0;
}

// Waits for phase `parity` of the barrier to complete, for at most kWaitCycles.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, unsigned parity) {
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity)) {
        if (clock64() - t0 > kWaitCycles) {
            atomicOr(&g_device_fault, BGI_FAULT_ASYNC_WAIT);
            return false;
        }
    }
    return true;
}

// global -> shared bulk copy completing on `bar` (bytes: multiple of 16, both addresses
// 16-byte aligned)
__device__ __forceinline__ void bulk_load(void *dst_smem, const void *src, unsigned bytes, uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst_smem)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}

// shared -> global bulk copy in the thread's current bulk group
__device__ __forceinline__ void bulk_store(void *dst, const void *src_smem, unsigned bytes) {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(smem_addr(src_smem)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }

// waits until every committed bulk group of this thread has completed (writes performed)
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

}  // namespace bgi
