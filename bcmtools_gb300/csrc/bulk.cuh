// bulk.cuh -- bulk asynchronous copies global -> shared (the TMA engine's
// non-tensor form, cp.async.bulk) completed on an mbarrier, with bounded
// waits.
//
// Every wait gives up after kWaitLimit polls (mbar_wait) or kWaitNs
// nanoseconds of global time (mbar_wait_quiet): the waiting kernel then
// records an error code in a device word the host reads (bcmg_sync and the
// solvers report it), waits (again bounded) for its own copies and returns,
// so a lost completion can never hang the GPU.
#pragma once
#include <cstdint>

namespace bcmg {

constexpr unsigned kWaitLimit = 1u << 22;
constexpr int kErrWaitTimeout = 0x100;

__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}

__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

// Adds `bytes` to the transaction count of the current phase without arriving.
__device__ __forceinline__ void mbar_add_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.expect_tx.relaxed.cta.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Orders this thread's earlier generic-proxy shared-memory accesses before
// later async-proxy (bulk copy) accesses.
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// dst (shared) <- src (global), `bytes` a multiple of 16, both 16-B aligned.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes,
                                         uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

// dst (global) <- src (shared), `bytes` a multiple of 16, both 16-B aligned;
// committed per thread with bulk_commit.
__device__ __forceinline__ void bulk_s2g(void* dst, const void* src, unsigned bytes) {
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst),
               "r"(smem_u32(src)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_commit() {
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}
// Waits until this thread's committed bulk stores have read their shared
// memory (the source may then be overwritten or released).
__device__ __forceinline__ void bulk_wait_read() {
  asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}

// Programmatic dependent launch: griddep_wait blocks until the grids this
// launch depends on have completed and their writes are visible (a no-op
// without such a dependency); griddep_launch_dependents lets the next
// dependent launch start once every CTA of this grid has issued it.
__device__ __forceinline__ void griddep_wait() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
}
__device__ __forceinline__ void griddep_launch_dependents() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}" : "=r"(ok) : "r"(smem_u32(bar)), "r"(parity) : "memory");
  return ok != 0;
}

// try_wait that may suspend the thread (up to `ns` nanoseconds) until the
// phase completes, instead of returning at once.
__device__ __forceinline__ bool mbar_try_wait_suspend(uint64_t* bar, unsigned parity,
                                                      unsigned ns) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n"
      " selp.u32 %0, 1, 0, p;\n}" : "=r"(ok) : "r"(smem_u32(bar)), "r"(parity), "r"(ns)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Bounded wait that leaves the issue slots to the other warps: the thread
// sleeps in the barrier (up to 20 us a try) rather than polling; gives up
// (false, *err set) after kWaitNs nanoseconds of global time.
constexpr uint64_t kWaitNs = 2000000000ull;
__device__ __forceinline__ bool mbar_wait_quiet(uint64_t* bar, unsigned parity, int* err) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_ns();
  for (;;) {
    if (mbar_try_wait_suspend(bar, parity, 20000u)) return true;
    if (global_ns() - t0 > kWaitNs) {
      if (err) atomicExch(err, kErrWaitTimeout);
      return false;
    }
  }
}

// Bounded wait for phase `parity` of `bar`; false (and *err set) on timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity, int* err) {
  for (unsigned k = 0; k < kWaitLimit; k++)
    if (mbar_try_wait(bar, parity)) return true;
  if (err) atomicExch(err, kErrWaitTimeout);
  return false;
}

}  // namespace bcmg
