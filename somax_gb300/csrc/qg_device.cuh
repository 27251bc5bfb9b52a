// Device-side PTX helpers shared by the libqgcore kernels: mbarriers with bounded waits,
// TMA tensor copies, programmatic dependent launch.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace qg {

constexpr long long kTimeoutCycles = 4000000000LL;  // ~2 s at 2 GHz: bound of every device wait

__device__ __forceinline__ uint32_t su32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* b, uint32_t n) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(b)), "r"(n) : "memory");
}
__device__ __forceinline__ void mbar_init_fence() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* b, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(su32(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint64_t* b, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(su32(b)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait: false after kTimeoutCycles or when another role already gave up (*abort).
__device__ __forceinline__ bool mbar_wait(uint64_t* b, uint32_t parity, volatile int* abort) {
    const long long t0 = clock64();
    while (!mbar_try(b, parity)) {
        if (abort && *abort) return false;
        if (clock64() - t0 > kTimeoutCycles) {
            if (abort) *abort = 1;
            return false;
        }
    }
    return true;
}
// Bounded wait that ignores the abort flag (draining copies in flight after an abort).
__device__ __forceinline__ bool mbar_drain(uint64_t* b, uint32_t parity) {
    const long long t0 = clock64();
    while (!mbar_try(b, parity))
        if (clock64() - t0 > kTimeoutCycles) return false;
    return true;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            su32(dst)),
        "l"((uint64_t)map), "r"(x), "r"(y), "r"(su32(bar))
        : "memory");
}
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y, int z) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
            su32(dst)),
        "l"((uint64_t)map), "r"(x), "r"(y), "r"(z), "r"(su32(bar))
        : "memory");
}
__device__ __forceinline__ void tma_prefetch_desc(const CUtensorMap* map) {
    asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)map) : "memory");
}

// Programmatic dependent launch.  Every kernel calls pdl_wait() (all prerequisite grids
// complete, their memory visible) before touching data a predecessor writes, and only then
// pdl_launch_dependents(), so at most one launch waits ahead of the running one instead of
// the whole chain cascading onto the SMs.
__device__ __forceinline__ void pdl_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

}  // namespace qg
