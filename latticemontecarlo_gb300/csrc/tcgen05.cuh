// Inline-PTX building blocks of the 5th-generation tensor-core kernels
// (mlp_tc.cu inference, mlp_gemm_tc.cu training GEMMs) for sm_100 and later:
// mbarriers with bounded waits, cp.async / bulk copies into shared memory,
// tcgen05.mma (kind::f16, one CTA), tcgen05.commit and tcgen05.ld.
//
// Operand layout in shared memory (K-major, no swizzle): 8-row x 16-byte core
// matrices; a tile of 32 K columns keeps element (r, k) at
//   (r / 8) * 512 + (k / 8) * 128 + (r % 8) * 16 + (k % 8) * 2   bytes,
// i.e. leading (K) byte offset 128 and 8-row stride 512.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace lmc {
namespace tc {

constexpr int kK = 32;                 // K columns of one operand tile
constexpr uint32_t kLbo = 128;         // byte offset between K-adjacent core matrices
constexpr uint32_t kSbo = kK * 16;     // byte offset between 8-row groups of a 32-wide tile
constexpr long long kWaitLimit = 1LL << 26;

__device__ __forceinline__ uint32_t Smem(const void *p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

// Byte offset of element (r, k) inside one 32-wide operand tile.
__device__ __forceinline__ uint32_t CoreOffset(int r, int k) {
  return static_cast<uint32_t>((r >> 3) * kSbo + (k >> 3) * kLbo + (r & 7) * 16 + (k & 7) * 2);
}

// Shared-memory matrix descriptor: start address, leading and stride byte offsets,
// descriptor version of sm_100 and later, base offset 0, no swizzle.
__device__ __forceinline__ uint64_t OperandDesc(uint32_t addr) {
  uint64_t d = static_cast<uint64_t>((addr & 0x3FFFF) >> 4);
  d |= static_cast<uint64_t>(kLbo >> 4) << 16;
  d |= static_cast<uint64_t>(kSbo >> 4) << 32;
  d |= static_cast<uint64_t>(1) << 46;
  return d;
}

// kind::f16 instruction descriptor: FP32 accumulator, BF16 A and B, both K-major, M x N.
__host__ __device__ constexpr uint32_t IdescBf16(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | (static_cast<uint32_t>(n >> 3) << 17) |
         (static_cast<uint32_t>(m >> 4) << 24);
}

__device__ __forceinline__ void Mma(uint32_t tmem, uint64_t a, uint64_t b, uint32_t idesc, bool accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate ? 1 : 0));
}
// The same with A read from tensor memory (`a_tmem`: 128 lanes = rows, each 32-bit column
// holding two consecutive 16-bit K elements, the lower K in the low half).
__device__ __forceinline__ void MmaTmemA(uint32_t tmem, uint32_t a_tmem, uint64_t b, uint32_t idesc, bool accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n\t}\n" ::"r"(tmem),
      "r"(a_tmem), "l"(b), "r"(idesc), "r"(accumulate ? 1 : 0));
}
// Arrives on `bar` once every MMA this thread issued before has completed.
__device__ __forceinline__ void Commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(Smem(bar)));
}
__device__ __forceinline__ void Arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(Smem(bar)) : "memory");
}
__device__ __forceinline__ void BarInit(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(Smem(bar)), "r"(count));
}
__device__ __forceinline__ void FenceBarrierInit() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ bool TryWait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(Smem(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Waits for the completion of the barrier phase with the given parity. False when it
// expires or another thread gave up (the abort flag), which it then sets.
__device__ __forceinline__ bool Wait(uint64_t *bar, uint32_t parity, volatile int *abort) {
  for (long long it = 0; it < kWaitLimit; ++it) {
    if (TryWait(bar, parity)) return true;
    if ((it & 63) == 0 && *abort) return false;
  }
  *abort = 1;
  return false;
}
// try_wait with a suspend-time hint (ns): the thread sleeps until the phase completes or
// the hint expires, so waiting warps take few issue slots.
__device__ __forceinline__ bool TryWaitSleep(uint64_t *bar, uint32_t parity, uint32_t hint_ns) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(Smem(bar)), "r"(parity), "r"(hint_ns)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ uint64_t GlobalTimerNs() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
constexpr uint64_t kWaitLimitNs = 2000000000ull;  // 2 s
// Wait as above with sleeping probes, bounded by kWaitLimitNs of wall time.
__device__ __forceinline__ bool WaitSleep(uint64_t *bar, uint32_t parity, volatile int *abort) {
  if (TryWaitSleep(bar, parity, 200)) return true;
  const uint64_t t0 = GlobalTimerNs();
  for (;;) {
    if (TryWaitSleep(bar, parity, 2000)) return true;
    if (*abort) return false;
    if (GlobalTimerNs() - t0 > kWaitLimitNs) {
      *abort = 1;
      return false;
    }
  }
}

// Bounded wait that ignores the abort flag (draining work already issued).
__device__ __forceinline__ bool WaitDrain(uint64_t *bar, uint32_t parity) {
  for (long long it = 0; it < kWaitLimit; ++it)
    if (TryWait(bar, parity)) return true;
  return false;
}
__device__ __forceinline__ void ArriveExpectTx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(Smem(bar)), "r"(bytes) : "memory");
}
// Bulk copy global -> shared (16-byte aligned, size a multiple of 16), completing on `bar`.
__device__ __forceinline__ void BulkCopy(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(Smem(dst)),
      "l"(src), "r"(bytes), "r"(Smem(bar))
      : "memory");
}
__device__ __forceinline__ void CpAsync16(void *smem, const void *gmem) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(Smem(smem)), "l"(gmem));
}
__device__ __forceinline__ void CpAsyncCommit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int kPending>
__device__ __forceinline__ void CpAsyncWait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(kPending) : "memory");
}
// Makes this thread's generic-proxy shared-memory writes visible to the tensor cores.
__device__ __forceinline__ void FenceAsyncSmem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void FenceBeforeSync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void FenceAfterSync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// TMEM allocation of `cols` columns (a power of two >= 32) by one whole warp; the
// address lands in *slot (shared memory).
__device__ __forceinline__ void TmemAlloc(uint32_t *slot, uint32_t cols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(Smem(slot)), "r"(cols));
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
}
__device__ __forceinline__ void TmemFree(uint32_t addr, uint32_t cols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(addr), "r"(cols));
}

// 32 consecutive fp32 columns of this thread's TMEM lane. The wait carries the
// 32 registers as operands (no memory clobber), so the compiler keeps their uses
// after it while still free to issue independent loads earlier.
__device__ __forceinline__ void TmemLoad32(uint32_t addr, float *v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(addr));
  asm volatile("tcgen05.wait::ld.sync.aligned;"
               : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]), "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]), "+r"(r[15]), "+r"(r[16]), "+r"(r[17]), "+r"(r[18]), "+r"(r[19]), "+r"(r[20]), "+r"(r[21]), "+r"(r[22]), "+r"(r[23]), "+r"(r[24]), "+r"(r[25]), "+r"(r[26]), "+r"(r[27]), "+r"(r[28]), "+r"(r[29]), "+r"(r[30]), "+r"(r[31]));
#pragma unroll
  for (int j = 0; j < 32; ++j) v[j] = __uint_as_float(r[j]);
}

// Stores 16 consecutive 32-bit columns of this thread's TMEM lane and waits for the store.
__device__ __forceinline__ void TmemStore16(uint32_t addr, const uint32_t *r) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};" ::"r"(addr),
      "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]), "r"(r[8]), "r"(r[9]),
      "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15])
      : "memory");
  asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}

}  // namespace tc
}  // namespace lmc
