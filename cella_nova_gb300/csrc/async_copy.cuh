// async_copy.cuh — bulk (TMA) copies, mbarriers and cp.async for sm_103a.
//
// Every wait is bounded: after kWaitLimitNs of %globaltimer a wait gives up,
// records kErrTimeout in the kernel's error word and reports failure, so a
// copy that never lands ends the kernel with an error status the host reads
// instead of a hung GPU.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace cg {

constexpr unsigned long long kWaitLimitNs = 2000000000ull;   // 2 s
constexpr int kErrTimeout = 1;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
                 : "memory");
}

// Make the initialised barrier (generic proxy) visible to the async proxy.
__device__ __forceinline__ void fence_barrier_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Order this thread's earlier generic-proxy shared-memory accesses before
// later async-proxy (bulk copy) writes to the same bytes.
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}

// 1-D bulk copy global -> shared (TMA engine), completing on `bar`.
// dst, src 16-byte aligned; bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes,
                                         uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

// 2-D tiled tensor copy global -> shared (TMA engine): the box of `map` at
// element coordinates (x, y), x innermost, lands dense in shared memory and
// completes on `bar`.  `map` is the address of a CUtensorMap in kernel
// parameter space (__grid_constant__) or global memory; x times the element
// size must be a multiple of 16 bytes, dst 128-byte aligned.
__device__ __forceinline__ void tensor2d_g2s(void* dst, const void* map, int x, int y,
                                             uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

// Before the TMA engine reads a tensor map held in global memory: order its
// (host-written) bytes before the tensor-map proxy's reads.
__device__ __forceinline__ void tensormap_acquire(const void* map) {
    asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(
                     reinterpret_cast<uint64_t>(map))
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

// Bounded wait for phase `parity` of `bar`; false (and *err set) on timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int* err,
                                          unsigned long long limit_ns = kWaitLimitNs) {
    if (mbar_try_wait(bar, parity)) return true;
    const unsigned long long t0 = global_ns();
    while (!mbar_try_wait(bar, parity)) {
        if (global_ns() - t0 > limit_ns) {
            if (err) atomicExch(err, kErrTimeout);
            return false;
        }
    }
    return true;
}

// Ampere-style per-thread async copy of 8 bytes (used where the destination
// layout is a transpose that a bulk copy cannot produce).
__device__ __forceinline__ void cp_async8(void* dst, const void* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_u32(dst)), "l"(src)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
    asm volatile("cp.async.commit_group;" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// Programmatic dependent launch.  A kernel launched with the programmatic
// stream serialization attribute may start while the kernel before it in the
// stream is still running; pdl_wait blocks until that kernel has completed
// and its memory operations are visible (a no-op for a kernel launched
// without the attribute), and pdl_launch_dependents lets the next such
// kernel start launching its CTAs, which then wait in their own pdl_wait.
// The step kernels call both before touching global memory, so the overlap
// covers only launch latency and the last wave's tail.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_launch_dependents() {
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Reciprocal estimate to ~1 ulp (MUFU); div_head_tail refines it.
__device__ __forceinline__ float rcp_approx(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// q = x / (zh + zt) for a head zh and a tail zt with |zt| <= |zh|, close to
// correctly rounded, from two published methods:
//  * Fast2Sum (T. J. Dekker, "A floating-point technique for extending the
//    available precision", Numer. Math. 18 (1971) 224-242): with
//    z = fl(zh + zt), zl = zt - (z - zh) is exact and z + zl == zh + zt;
//  * one quotient correction with the fused multiply-add remainder
//    (P. Markstein, "Computation of elementary functions on the IBM RISC
//    System/6000 processor", IBM J. Res. Dev. 34 (1990) 111-119): for
//    q0 = fl(x r) with r close to 1/z, x - q0 z is exact in one fma, and
//    q0 + (rem - q0 zl) r corrects q0 for its own rounding and for the
//    tail zl of the divisor.
// r is the hardware reciprocal estimate (rcp.approx.ftz.f32).
__device__ __forceinline__ float div_head_tail(float x, float zh, float zt) {
    const float z = zh + zt;
    const float zl = zt - (z - zh);
    const float r = rcp_approx(z);
    const float q0 = x * r;
    const float rem = fmaf(-q0, z, x);
    return fmaf(rem - q0 * zl, r, q0);
}

// 2^x to a few ulp (MUFU); subnormal results flush to zero.
__device__ __forceinline__ float ex2_approx(float x) {
    float r;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

}  // namespace cg
