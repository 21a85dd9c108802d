// sfh_ptx.cuh -- inline-PTX helpers shared by the TMA / mbarrier kernels (sm_103a):
// mbarrier init / arrive / bounded wait, 2-D tensor loads (cp.async.bulk.tensor) and
// the driver entry point that encodes tensor maps.
#pragma once
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>
#include <stdint.h>

// Budget of one mbarrier wait: ~2 s of SM clock.
constexpr long long kSfhWaitBudget = 4000000000LL;

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void mbar_arrive_n(uint64_t *bar, uint32_t n) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(n)
                 : "memory");
}

__device__ __forceinline__ bool mbar_test(uint64_t *bar, uint32_t parity) {
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

// Bounded wait for the phase with the given parity.  Gives up (returns false) when
// another role has raised the abort flag or after kSfhWaitBudget clocks, recording
// `code` in *err.
static __device__ __noinline__ bool mbar_wait(uint64_t *bar, uint32_t parity,
                                              volatile int *abort_flag, int *err, int code) {
    const long long t0 = clock64();
    for (;;) {
        if (mbar_test(bar, parity)) return true;
        if (*abort_flag) return false;
        if (clock64() - t0 > kSfhWaitBudget) {
            *abort_flag = 1;
            atomicExch(err, code);
            return false;
        }
    }
}

// try_wait with a suspend-time hint: a thread whose phase is not complete may sleep up
// to `ns` nanoseconds inside the instruction instead of spinning.
__device__ __forceinline__ bool mbar_test_sleep(uint64_t *bar, uint32_t parity, uint32_t ns) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity), "r"(ns)
        : "memory");
    return ok != 0;
}

// mbar_wait with sleeping polls (for roles that often wait long: producers on a full
// ring, consumers ahead of the memory stream) and a caller-given budget in SM cycles.
static __device__ __noinline__ bool mbar_wait_sleep(uint64_t *bar, uint32_t parity,
                                                    volatile int *abort_flag, int *err, int code,
                                                    long long budget = kSfhWaitBudget) {
    const long long t0 = clock64();
    for (;;) {
        if (mbar_test_sleep(bar, parity, 1000u)) return true;
        if (*abort_flag) return false;
        if (clock64() - t0 > budget) {
            *abort_flag = 1;
            atomicExch(err, code);
            return false;
        }
    }
}

__device__ __forceinline__ void fence_barrier_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Named barrier over `count` threads (a multiple of 32), id 1..15.
__device__ __forceinline__ void named_bar_sync(int id, int count) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
}

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int x, int y,
                                            uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
        "l"((uint64_t)map), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

// Contiguous global -> shared copy by the TMA unit (both addresses 16-byte aligned, bytes a
// multiple of 16), completing on the mbarrier.
__device__ __forceinline__ void bulk_load(void *dst, const void *src, uint32_t bytes,
                                          uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
            "r"(smem_u32(dst)),
        "l"((uint64_t)src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (nullptr if absent).
PFN_cuTensorMapEncodeTiled_v12000 sfh_tensor_map_encoder();
