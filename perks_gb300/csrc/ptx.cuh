// Thin inline-PTX helpers for sm_103a: mbarriers, bulk (TMA) copies, proxy
// fences, L2 cache policies, and a bounded grid barrier.
//
// Every wait in this file is bounded by a clock64() budget. When a budget
// runs out the caller gets `false`, records an error word in global memory and
// leaves its kernel; nothing here traps or spins forever.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace perks {

// Error bits written to the device-side status word.
enum : unsigned {
  kErrBarrierTimeout = 1u << 0,   // grid barrier budget exhausted
  kErrCopyTimeout = 1u << 1,      // an mbarrier (bulk copy) wait ran out
  kErrPeerAbort = 1u << 2,        // another CTA reported an error first
  kErrBreakdown = 1u << 3,        // CG: p.Ap <= 0 or non-finite
  kErrNonFinite = 1u << 4,        // CG: non-finite residual
};

// Default budget of every device-side wait: about 2^32 clocks (~2 s at
// 2 GHz), far above any legitimate wait. Kernels take the budget as a launch
// parameter (WaitCtl below), so a test can shorten it.
constexpr long long kWaitBudget = 1ll << 32;

// Wait budget and the test hook that makes one CTA skip its first grid-barrier
// arrival (so that every other CTA's bounded wait runs out). Filled on the
// host from the process-wide settings (perks_debug_set_wait_fault); in normal
// use budget = kWaitBudget and skip_cta = -1.
struct WaitCtl {
  long long budget = kWaitBudget;
  int skip_cta = -1;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// ---------------------------------------------------------------- mbarrier
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_inval(uint64_t* bar) {
  asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}
// Make mbarrier initialisation visible to the async proxy (bulk copies).
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.acquire.cta.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait for phase `parity` of `bar`. Returns false on timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity, long long budget) {
  if (mbar_try_wait(bar, parity)) return true;
  long long t0 = clock64();
  while (!mbar_try_wait(bar, parity)) {
    if (clock64() - t0 > budget) return false;
  }
  return true;
}

// ---------------------------------------------------------------- L2 policy
__device__ __forceinline__ uint64_t policy_evict_first() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ uint64_t policy_evict_last() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ uint64_t policy_evict_normal() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_normal.b64 %0, 1.0;" : "=l"(p));
  return p;
}

// ------------------------------------------------------------- bulk copies
// Global -> shared bulk copy completing on `bar` (tx-count). Both addresses
// 16-byte aligned and `bytes` a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void* dst_smem, const void* src_gmem, unsigned bytes,
                                         uint64_t* bar, uint64_t policy) {
  asm volatile(
      "cp.async.bulk.shared::cta.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], "
      "%4;" ::"r"(smem_u32(dst_smem)),
      "l"(src_gmem), "r"(bytes), "r"(smem_u32(bar)), "l"(policy)
      : "memory");
}

// ------------------------------------------------------------------ fences
// Order this thread's generic-proxy global writes before later async-proxy
// (bulk copy) reads of the same addresses, possibly by other CTAs.
__device__ __forceinline__ void fence_proxy_async_global() {
  asm volatile("fence.proxy.async.global;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Drop one 128-byte L2 line without writing it back. Only for data that is
// dead: nobody reads it again before it is overwritten.
__device__ __forceinline__ void l2_discard_line(const void* gptr) {
  asm volatile("discard.global.L2 [%0], 128;" ::"l"(gptr) : "memory");
}

// ------------------------------------------------------------ stores/loads
template <class V>
__device__ __forceinline__ void st_global_policy(V* p, const V& v, uint64_t pol);

template <>
__device__ __forceinline__ void st_global_policy<float4>(float4* p, const float4& v, uint64_t pol) {
  asm volatile("st.global.L2::cache_hint.v4.f32 [%0], {%1, %2, %3, %4}, %5;" ::"l"(p), "f"(v.x), "f"(v.y),
               "f"(v.z), "f"(v.w), "l"(pol)
               : "memory");
}
template <>
__device__ __forceinline__ void st_global_policy<double2>(double2* p, const double2& v, uint64_t pol) {
  asm volatile("st.global.L2::cache_hint.v2.f64 [%0], {%1, %2}, %3;" ::"l"(p), "d"(v.x), "d"(v.y), "l"(pol)
               : "memory");
}

__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_gpu(unsigned* p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// ----------------------------------------------------------------- clusters
// Thread-block cluster helpers: rank of this CTA in its cluster, the
// cluster's index in the grid, distributed shared memory (DSMEM) access to a
// peer CTA's shared memory (mapa + ld/st.shared::cluster), and the cluster
// barrier (every thread of every CTA of the cluster arrives, then waits; the
// release/acquire pair orders the memory accesses made before the arrival).
__device__ __forceinline__ unsigned cluster_ctarank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ unsigned cluster_nctarank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ unsigned cluster_index_x() {
  unsigned r;
  asm volatile("mov.u32 %0, %%clusterid.x;" : "=r"(r));
  return r;
}
__device__ __forceinline__ unsigned cluster_count_x() {
  unsigned r;
  asm volatile("mov.u32 %0, %%nclusterid.x;" : "=r"(r));
  return r;
}
// Shared-memory address of `p` (this CTA's variable) in CTA `rank` of the cluster.
__device__ __forceinline__ uint32_t dsmem_addr(const void* p, unsigned rank) {
  uint32_t out;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(out) : "r"(smem_u32(p)), "r"(rank));
  return out;
}
__device__ __forceinline__ void dsmem_st_f64(uint32_t addr, double v) {
  asm volatile("st.shared::cluster.f64 [%0], %1;" ::"r"(addr), "d"(v) : "memory");
}
__device__ __forceinline__ double dsmem_ld_f64(uint32_t addr) {
  double v;
  asm volatile("ld.shared::cluster.f64 %0, [%1];" : "=d"(v) : "r"(addr) : "memory");
  return v;
}
__device__ __forceinline__ void dsmem_st_u32(uint32_t addr, unsigned v) {
  asm volatile("st.shared::cluster.u32 [%0], %1;" ::"r"(addr), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned dsmem_ld_u32(uint32_t addr) {
  unsigned v;
  asm volatile("ld.shared::cluster.u32 %0, [%1];" : "=r"(v) : "r"(addr) : "memory");
  return v;
}
// (Not the .aligned form: the threads of a warp may arrive after divergent
// branches, e.g. one thread that waited at the grid barrier.)
__device__ __forceinline__ void cluster_sync_all() {
  asm volatile("barrier.cluster.arrive.release;\n\tbarrier.cluster.wait.acquire;" ::: "memory");
}

// ------------------------------------------------------------- grid barrier
// Barrier over all CTAs of a cooperative launch on a monotonically increasing
// arrival counter (bar[0], zeroed before the launch): the k-th barrier
// completes when the counter reaches k * nblocks, so no reset and no second
// word are needed (about 1.2 us for 152 CTAs on GB300, half the cost of a
// sense-reversing barrier with a shared counter/generation line). `status` is
// the kernel's error word: a waiting CTA that finds it non-zero leaves early,
// so one failing CTA does not make every other CTA wait out its budget.
// Returns false when the caller must abandon the kernel.
struct GridBarrier {
  unsigned* bar;
  unsigned* status;
  unsigned nblocks;
  WaitCtl ctl;
  unsigned epoch = 0;  // barriers passed by this CTA (identical in every thread)

  __device__ __forceinline__ bool sync() {
    __shared__ unsigned s_ok;
    epoch++;
    __syncthreads();
    if (threadIdx.x == 0) {
      // The fence publishes the whole CTA's writes (ordered before it by the
      // __syncthreads); acq_rel makes the last arriver, which does not spin,
      // acquire the other CTAs' writes too (L1 may hold stale lines otherwise).
      __threadfence();
      s_ok = arrive_wait(int(blockIdx.x)) ? 1u : 0u;
    }
    __syncthreads();
    return s_ok != 0;
  }

  // One thread's arrival and bounded wait for the `epoch`-th completion
  // (epoch already counted by the caller); `me` is the arriving unit's index
  // for the test hook. The caller has fenced its unit's writes.
  __device__ __forceinline__ bool arrive_wait(int me) {
    {
      unsigned ok = 1;
      const unsigned target = epoch * nblocks;
      unsigned old;
      bool skip = epoch == 1 && me == ctl.skip_cta;
      if (skip) {
        // test hook: this CTA does not arrive, so at most nblocks - 1 arrivals
        // come and every CTA's wait (its own included) runs out its budget
        old = 0u;
      } else {
        asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], 1;" : "=r"(old) : "l"(bar) : "memory");
      }
      if (skip || int(old + 1u - target) < 0) {
        long long t0 = clock64();
        unsigned spins = 0;
        while (int(ld_acquire_gpu(bar) - target) < 0) {
          if ((++spins & 63u) == 0u) {
            if (*((volatile unsigned*)status) != 0u) { ok = 0; break; }
            if (clock64() - t0 > ctl.budget) {
              atomicOr(status, kErrBarrierTimeout);
              ok = 0;
              break;
            }
          }
        }
      }
      if (ok && *((volatile unsigned*)status) != 0u) ok = 0;
      return ok != 0;
    }
  }
};

}  // namespace perks
