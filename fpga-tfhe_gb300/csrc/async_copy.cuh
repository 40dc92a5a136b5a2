// async_copy.cuh -- shared-memory barriers and bulk copies (sm_90+ PTX) with
// bounded waits.
//
// Every wait in the engine's kernels gives up after kWaitLimitNs of
// %globaltimer time and reports failure to the caller, which records an
// error status for the host (TFHE_GPU_TIMEOUT) instead of spinning forever.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace tfhe_gb300 {

constexpr uint64_t kWaitLimitNs = 2000000000ull;  // 2 s

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
                 : "memory");
}

// Make barrier initialisation visible to the async (bulk-copy) proxy.
__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile(
        "{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile(
        "{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(
            smem_u32(bar)),
        "r"(bytes)
        : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Wait for the phase of `bar` with the given parity to complete; false after
// kWaitLimitNs.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = global_ns();
    while (!mbar_try_wait(bar, parity)) {
        if (global_ns() - t0 > kWaitLimitNs) return false;
    }
    return true;
}

// The same with a CTA-wide abort flag: once any wait of the CTA has given up
// (and set *abort), the others return false at once instead of waiting out
// their own limit, so a failed kernel ends within about one limit.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity,
                                                  const volatile int* abort) {
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = global_ns();
    while (!mbar_try_wait(bar, parity)) {
        if (*abort || global_ns() - t0 > kWaitLimitNs) return false;
    }
    return true;
}
// ---- distributed shared memory (thread-block clusters) --------------------
// Shared::cluster address of the same location in CTA `rank` of the cluster.
__device__ __forceinline__ uint32_t cluster_map(uint32_t local_smem, uint32_t rank) {
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(local_smem), "r"(rank));
    return r;
}

// Store 8 bytes into another CTA's shared memory; the bytes count as
// transaction bytes on that CTA's mbarrier `rbar` when they land.
__device__ __forceinline__ void st_async_f2(uint32_t raddr, float x, float y, uint32_t rbar) {
    asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.v2.f32 [%0], {%1, %2}, [%3];" ::"r"(raddr),
                 "f"(x), "f"(y), "r"(rbar)
                 : "memory");
}

// The same for 16 bytes (two doubles, as four 32-bit words).
__device__ __forceinline__ void st_async_d2(uint32_t raddr, double x, double y, uint32_t rbar) {
    asm volatile(
        "st.async.shared::cluster.mbarrier::complete_tx::bytes.v4.b32 [%0], {%1, %2, %3, %4}, [%5];" ::"r"(raddr),
        "r"(__double2loint(x)), "r"(__double2hiint(x)), "r"(__double2loint(y)), "r"(__double2hiint(y)), "r"(rbar)
        : "memory");
}

// Wait (bounded, with the CTA's abort flag) for a phase of a barrier that
// other CTAs of the cluster complete; acquire at cluster scope, so their
// stores are visible afterwards.
__device__ __forceinline__ bool mbar_try_wait_cluster(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ bool mbar_wait_cluster_bounded(uint64_t* bar, uint32_t parity,
                                                          const volatile int* abort) {
    if (mbar_try_wait_cluster(bar, parity)) return true;
    const uint64_t t0 = global_ns();
    while (!mbar_try_wait_cluster(bar, parity)) {
        if (*abort || global_ns() - t0 > kWaitLimitNs) return false;
    }
    return true;
}

// Bulk copy global -> this CTA's shared memory; completion is counted in
// bytes on `bar`.  dst, src 16-byte aligned; bytes a multiple of 16.
// Start fetching `bytes` (a multiple of 16, 16-byte aligned) of global
// memory into L2 without waiting for it.
__device__ __forceinline__ void bulk_prefetch_l2(const void* src, uint32_t bytes) {
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"(bytes) : "memory");
}

__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes,
                                              uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
            "r"(smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

}  // namespace tfhe_gb300
