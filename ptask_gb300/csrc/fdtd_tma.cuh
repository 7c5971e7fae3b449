// fdtd_tma.cuh -- device helpers shared by the TMA-staged step kernels: mbarriers with bounded
// waits, 3-D tensor copies into shared memory, and the Yee update expression in the reference's
// operation order (graphfdtd.cpp:185-312: new = D*old + C*((a1 - a0)*s1 - (b1 - b0)*s2), no FMA).
#pragma once

#include <cuda.h>
#include <cudaTypedefs.h>

#include <cstdint>

namespace ptk {
namespace tma {

constexpr int kWaitLimit = 1 << 22;                     // polls: a hard cap (about 16 s on GB300)
constexpr unsigned long long kWaitNs = 1000000000ull;   // a wait gives up after 1 s of global time
constexpr size_t kTabBytes = 256 * sizeof(float4);      // material table (Ca, Cb, Da, Db) per entry

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Bounded wait for the phase with the given parity to complete: gives up after kWaitNs of global
// time (read only once a poll has come back empty) or kWaitLimit polls, whichever comes first.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity)
{
    const uint32_t a = smem_u32(bar);
    unsigned long long t0 = 0;
    for (int it = 0; it < kWaitLimit; ++it) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
        if (it == 0) t0 = global_ns();
        else if ((it & 15) == 0 && global_ns() - t0 > kWaitNs) return false;
    }
    return false;
}

__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int x, int y, int z, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(smem_u32(dst)),
        "l"(map), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void tma_acquire(const CUtensorMap *map)
{
    asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(map) : "memory");
}

__device__ __forceinline__ float4 ld4s(const float *p) { return *reinterpret_cast<const float4 *>(p); }

__device__ __forceinline__ float yee_b(float d, float h, float c, float a1, float a0, float s1, float b1, float b0,
                                       float s2)
{
    const float curl = __fsub_rn(__fmul_rn(__fsub_rn(a1, a0), s1), __fmul_rn(__fsub_rn(b1, b0), s2));
    return __fadd_rn(__fmul_rn(d, h), __fmul_rn(c, curl));
}

}  // namespace tma

// cuTensorMapEncodeTiled through the runtime's driver entry point (null when unavailable).
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder();

}  // namespace ptk
