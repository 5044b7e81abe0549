// nsdg_tma.cuh — mbarrier and TMA (cp.async.bulk.tensor) helpers in inline
// PTX for the operator-staging stress kernels, with bounded waits.
//
// Waits are bounded in time (limitNs of the GPU's global timer, and at most
// kTmaSpin polls): a caller whose copy has not landed by then records an
// error and returns after a second bounded wait for the copy it issued, so a
// lost copy can never hang the GPU.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace nsdg {
namespace {

constexpr long kTmaSpin = 1L << 26;
constexpr unsigned long long kWaitNs = 1000000000ull; // 1 s

__device__ __forceinline__ unsigned smemAddr(const void* p)
{
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbarInit(uint64_t* bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smemAddr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbarExpectTx(uint64_t* bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smemAddr(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbarTryWait(uint64_t* bar, unsigned parity)
{
    unsigned done;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(done)
                 : "r"(smemAddr(bar)), "r"(parity)
                 : "memory");
    return done != 0;
}
__device__ __forceinline__ unsigned long long globalTimerNs()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ bool mbarWaitBounded(uint64_t* bar, unsigned parity,
    unsigned long long limitNs = kWaitNs)
{
    const unsigned long long t0 = globalTimerNs();
    for (long i = 0; i < kTmaSpin; ++i) {
        if (mbarTryWait(bar, parity))
            return true;
        if ((i & 63) == 63 && globalTimerNs() - t0 > limitNs)
            break;
    }
    return false;
}
__device__ __forceinline__ void tmaLoad2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar)
{
    asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
                 " [%0], [%1, {%2, %3}], [%4];" ::"r"(smemAddr(dst)),
                 "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smemAddr(bar))
                 : "memory");
}
} // namespace
} // namespace nsdg
