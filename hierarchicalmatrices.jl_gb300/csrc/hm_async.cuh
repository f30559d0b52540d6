// Device helpers shared by the kernels: asynchronous copies (cp.async,
// cp.async.bulk), mbarriers with bounded waits, and the compensated fold.
// Written for sm_103a.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace hm {
namespace {
constexpr unsigned long long kWaitLimitNs = 2000000000ull;
constexpr unsigned long long kDrainLimitNs = 200000000ull;

// Programmatic dependent launch: a kernel launched with the programmatic
// stream serialisation attribute may start while its predecessor in the stream
// is finishing; pdl_wait() returns once the predecessor has completed and its
// writes are visible (immediately for a kernel launched without the
// attribute).  pdl_trigger() lets the successor be scheduled early.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

__device__ __forceinline__ uint32_t smem_addr(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ uint64_t global_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ bool mbar_test(uint64_t *bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Waits for the completion of the phase of `bar` with the given parity;
// false once limit_ns has passed.
__device__ bool mbar_wait(uint64_t *bar, uint32_t parity, unsigned long long limit_ns)
{
    if (mbar_test(bar, parity)) return true;
    const uint64_t t0 = global_ns();
    for (uint32_t it = 1;; ++it) {
        if (mbar_test(bar, parity)) return true;
        if ((it & 1023) == 0 && global_ns() - t0 > limit_ns) return false;   // the clock, now and then
    }
}
// The first wait of a CTA in the kernels with bounded waits: on `bar`, or,
// when `stall` is set (the handle's test hook for the timeout path), on
// `never`, a barrier that nothing arrives on, so that the wait runs out after
// limit_ns and the kernel takes its give-up path.  Later waits use `bar`.
__device__ __forceinline__ bool mbar_wait_first(uint64_t *bar, uint32_t parity, unsigned long long limit_ns,
                                                bool &stall, uint64_t *never)
{
    if (stall) {
        stall = false;
        return mbar_wait(never, 0, limit_ns);
    }
    return mbar_wait(bar, parity, limit_ns);
}
// bytes (a multiple of 16) from 16-byte aligned global src to 16-byte
// aligned shared dst, completing on bar.
__device__ __forceinline__ void bulk_load(void *dst, const void *src, uint32_t bytes, uint64_t *bar)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}
template <int B>
__device__ __forceinline__ void async_copy(void *dst, const void *src)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"(smem_addr(dst)), "l"(src), "n"(B) : "memory");
}
// 16 bytes, global -> shared, bypassing L1 (both addresses 16-byte aligned)
__device__ __forceinline__ void async_copy16(void *dst, const void *src)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void async_wait_all()
{
    asm volatile("cp.async.wait_all;" ::: "memory");
}
__device__ __forceinline__ void async_commit()
{
    asm volatile("cp.async.commit_group;" ::: "memory");
}
// waits until at most `pending` (0..2) of this thread's latest cp.async groups are in flight
__device__ __forceinline__ void async_wait_pending(int pending)
{
    if (pending <= 0) asm volatile("cp.async.wait_group 0;" ::: "memory");
    else if (pending == 1) asm volatile("cp.async.wait_group 1;" ::: "memory");
    else asm volatile("cp.async.wait_group 2;" ::: "memory");
}
// hi + lo += p: compensated (TwoSum) for FP32; FP64 adds plainly (its
// products are exact enough, and FP64 adds are scarce on this part).
__device__ __forceinline__ void fold(float &hi, float &lo, float p)
{
    const float sm = hi + p;
    const float bp = sm - hi;
    lo += (hi - (sm - bp)) + (p - bp);
    hi = sm;
}
__device__ __forceinline__ void fold(double &hi, double &, double p) { hi += p; }
}  // namespace
}  // namespace hm
