// Inline-PTX building blocks for sm_100a/sm_103a: mbarriers, TMA tensor
// loads and the 5th-generation tensor core (tcgen05: TMEM allocation, MMA,
// commit, TMEM loads).  Written from the PTX ISA; no library code.
//
// Every wait is bounded: a spin that exceeds kSpinLimit polls gives up,
// records `where` in the kernel's status word and returns false, so a
// broken pipeline ends with an error status instead of a hung GPU.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace emc {
namespace ptx {

constexpr uint32_t kSpinLimit = 1u << 24;  // try_wait polls (each suspends briefly)

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// ---- mbarrier ---------------------------------------------------------------
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
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

// try_wait with acquire at cluster scope: for a barrier that threads of the
// pair peer arrive on (their prior TMEM reads happen before what follows).
__device__ __forceinline__ bool mbar_try_wait_cluster(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Arrives (release at cluster scope) on the mbarrier at shared::cluster
// address `bar_cluster`, this CTA's or its pair peer's.
__device__ __forceinline__ void mbar_arrive_cluster(uint32_t bar_cluster) {
  asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(bar_cluster)
               : "memory");
}

// Bounded wait for the phase with the given parity to complete.  On timeout
// sets bit `where` of *status and returns false.  `limit` polls at most (a
// plan's debug option lowers it for the pipeline waits; the drain waits that
// make an aborted CTA safe to exit always use kSpinLimit).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int* status, int where,
                                          uint32_t limit = kSpinLimit) {
  for (uint32_t i = 0; i < limit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  if (status) atomicOr(status, 1 << where);
  return false;
}

// mbar_wait at cluster scope (mbar_try_wait_cluster).
__device__ __forceinline__ bool mbar_wait_cluster(uint64_t* bar, uint32_t parity, int* status,
                                                  int where, uint32_t limit = kSpinLimit) {
  for (uint32_t i = 0; i < limit; ++i)
    if (mbar_try_wait_cluster(bar, parity)) return true;
  if (status) atomicOr(status, 1 << where);
  return false;
}

// Bounded wait that sleeps `ns` nanoseconds between polls, for warps that
// wait long (epilogue warps waiting for a tile's accumulators): polling
// warps take issue slots from the single threads that issue the TMA loads
// and the MMAs.  Gives up after kSpinLimit polls (seconds).
__device__ __forceinline__ bool mbar_wait_sleep(uint64_t* bar, uint32_t parity, int* status,
                                                int where, uint32_t ns,
                                                uint32_t limit = kSpinLimit) {
  for (uint32_t i = 0; i < limit; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    __nanosleep(ns);
  }
  if (status) atomicOr(status, 1 << where);
  return false;
}

// Exit path of a pipeline that gave up (a bounded wait timed out): waits, at
// the full limit, until the TMA loads of the last `issued` k-blocks have
// landed, so that no copy into this CTA's shared memory is in flight when the
// CTA exits.  The loads of k-block it complete phase (it / stages) & 1 of
// full[it % stages]; each of the last `stages` k-blocks is the newest phase
// armed on its stage, so a completed phase is recognised by its parity.  When
// a phase never completes (a CTA pair whose peer stopped issuing leaves bytes
// outstanding), the wait gives up after kDrainLimit polls
// and records bit `where`; settle_after_timeout then covers what is left.
constexpr uint32_t kDrainLimit = 1u << 16;
__device__ __forceinline__ void drain_loads(uint64_t* full, int stages, uint32_t issued,
                                            int* status, int where) {
  const uint32_t first = issued > (uint32_t)stages ? issued - (uint32_t)stages : 0u;
  for (uint32_t it = first; it < issued; ++it)
    mbar_wait(&full[it % stages], (it / stages) & 1, status, where, kDrainLimit);
}

// Last step of every tensor kernel before TMEM is freed.  A CTA pair's loads
// complete on rank 0's barriers, so rank 1 cannot wait for its own copies,
// and after a timeout rank 1 may have issued loads for a stage that rank 0
// never armed; a drain wait may also have given up.  When any bounded wait of
// the launch gave up (a nonzero status word, read after the CTA's or pair's
// final barrier), the CTA pauses 200 us -- two orders of magnitude beyond the
// latency of a TMA copy -- before it frees TMEM and exits.  The normal path
// reads one word.
__device__ __forceinline__ void settle_after_timeout(const int* status) {
  if (!status || *(volatile const int*)status == 0) return;
  const long long t0 = clock64();
  while (clock64() - t0 < 400000) __nanosleep(1000);
}

// ---- TMA ------------------------------------------------------------------
__device__ __forceinline__ void tma_prefetch_desc(const CUtensorMap* map) {
  asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)map) : "memory");
}

// 2D tiled bulk tensor load into shared memory, completing on `bar`.
// x = innermost (contiguous) coordinate in elements, y = row.
__device__ __forceinline__ void tma_load_2d(void* smem_dst, const CUtensorMap* map, int x, int y,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(smem_dst)),
      "l"((uint64_t)map), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

// ---- tcgen05 ---------------------------------------------------------------
// Allocates ncols TMEM columns (power of two >= 32); the base address is
// written to *dst_smem.  Executed by one full warp.
__device__ __forceinline__ void tmem_alloc(uint32_t* dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   smem_u32(dst_smem)),
               "r"(ncols)
               : "memory");
}

__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// D[tmem] (+)= A[smem] * B[smem]^T, kind::f16 (both operands FP16 or both
// BF16, FP32 accumulate).  accumulate = 0 overwrites D.
__device__ __forceinline__ void mma_f16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc,
                                        uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// Arrives once on `bar` when every tcgen05.mma issued so far by this thread
// has completed (and its shared-memory operands may be overwritten).
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}


// 32 lanes x 16 columns of 32-bit TMEM values: lane i of the warp gets row
// (taddr.lane + i), columns taddr.col .. +15.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32"
      " {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_wait_ld() {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// Shared-memory matrix descriptor of a K-major tile in the canonical
// swizzled layout (rows of `row_bytes` = the swizzle span, 8-row atoms
// `sbo` bytes apart).  swizzle: 2 = 128B, 4 = 64B, 6 = 32B.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t sbo, uint32_t swizzle) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);        // start address
  d |= (uint64_t)1 << 16;                        // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;    // stride byte offset: 8-row atom pitch
  d |= (uint64_t)1 << 46;                        // descriptor version (tcgen05)
  d |= (uint64_t)(swizzle & 7) << 61;            // layout / swizzle mode
  return d;
}

// Instruction descriptor, kind::f16: FP16 A and B (K-major), FP32 D,
// M x N tile.
__host__ __device__ constexpr uint32_t idesc_f16(int M, int N) {
  return (1u << 4)                        // D format: F32
         | (0u << 7) | (0u << 10)         // A, B format: F16
         | ((uint32_t)(N >> 3) << 17)     // N / 8
         | ((uint32_t)(M >> 4) << 24);    // M / 16
}

// ---- CTA pairs (cta_group::2) ---------------------------------------------
// A cluster of two CTAs runs one 256-row MMA: rank 0 issues it, each CTA
// holds its 128 rows of A and half of B, and the accumulator rows live in
// each CTA's own TMEM.

__device__ __forceinline__ uint32_t cluster_ctarank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}

// Shared::cluster address of the object at shared address `saddr` in the
// cluster's CTA `rank`.
__device__ __forceinline__ uint32_t mapa_shared(uint32_t saddr, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(saddr), "r"(rank));
  return r;
}

// Every thread of both CTAs arrives and waits (release / acquire).
__device__ __forceinline__ void cluster_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\t"
               "barrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// One warp of each CTA of the pair executes these together.
__device__ __forceinline__ void tmem_alloc_pair(uint32_t* dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   smem_u32(dst_smem)),
               "r"(ncols)
               : "memory");
}

__device__ __forceinline__ void tmem_relinquish_pair() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc_pair(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}

// 2D tiled load into this CTA's shared memory completing on the mbarrier at
// shared::cluster address `bar_cluster` (this CTA's or its pair peer's).
__device__ __forceinline__ void tma_load_2d_pair(void* smem_dst, const CUtensorMap* map, int x,
                                                 int y, uint32_t bar_cluster) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cta.global.tile.mbarrier::complete_tx::bytes.cta_group::2"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(smem_dst)),
      "l"((uint64_t)map), "r"(x), "r"(y), "r"(bar_cluster)
      : "memory");
}

// D (+)= A * B^T over the pair: M = 256 (128 rows of A per CTA), B's N rows
// split in halves between the CTAs (same shared offsets), D rows in each
// CTA's TMEM.  Issued by one thread of rank 0.
__device__ __forceinline__ void mma_f16_pair(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc,
                                             uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::2.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// Arrives once on the mbarrier at the same shared offset in every CTA of
// cta_mask when the pair MMAs issued so far by this thread have completed.
__device__ __forceinline__ void mma_commit_pair(uint64_t* bar, uint16_t cta_mask) {
  asm volatile(
      "tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64"
      " [%0], %1;" ::"r"(smem_u32(bar)),
      "h"(cta_mask)
      : "memory");
}

__device__ __forceinline__ bool elect_one_lane() { return (threadIdx.x & 31) == 0; }

}  // namespace ptx
}  // namespace emc
