// Fused ensemble inference of the BF16 barrier surrogate on the 5th-generation
// tensor cores (tcgen05): one persistent CTA per SM walks tiles of 128 samples.
// Per tile and member m:
//   D1 (TMEM, 128 x 256 fp32) = X (smem) . W1[m]^T          tcgen05.mma kind::f16, K in chunks of 64
//   H1 (smem, bf16)            = GELU(D1 + b1[m])            tcgen05.ld epilogue, written in operand layout
//   D2 (TMEM)                  = H1 . W2[m]^T
//   y_m                        = GELU(D2 + b2[m]) . w3[m] + b3[m]   (in registers, one row per thread pair)
// then the ensemble mean and spread. Weight chunks (256 rows x 64 K, 32 KB) stream
// through a double buffer with cp.async while the tensor cores work on the other.
//
// Operand layout in shared memory (K-major, no swizzle): 8-row x 16-byte core
// matrices; element (r, k) of a tile with K columns sits at
//   (r / 8) * (K / 8) * 128 + (k / 8) * 128 + (r % 8) * 16 + (k % 8) * 2,
// i.e. leading-dimension (K) byte offset 128 and stride (8-row group) byte offset
// K * 16. Every wait on the tensor cores is bounded; on expiry the kernel records
// kMlpTimeout, waits (bounded) for its last commit, frees its TMEM and returns.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "mlp.cuh"

namespace lmc {
namespace {

constexpr int kTcRows = 128;       // samples per tile (MMA M)
constexpr int kTcHidden = 256;     // MMA N and the hidden width
constexpr int kTcChunk = 64;       // K per weight chunk
constexpr int kTcThreads = 256;    // 8 warps: TMEM lane group = warp % 4, column half = warp / 4
constexpr uint32_t kTmemCols = 512;
constexpr int kMlpTimeout = 1;
constexpr long long kWaitLimit = 1LL << 26;

__device__ __forceinline__ uint32_t Smem(const void *p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

__device__ __forceinline__ uint64_t OperandDesc(uint32_t addr, uint32_t sbo) {
  uint64_t d = static_cast<uint64_t>((addr & 0x3FFFF) >> 4);
  d |= static_cast<uint64_t>(128 >> 4) << 16;             // leading (K) byte offset between core matrices
  d |= static_cast<uint64_t>((sbo >> 4) & 0x3FFF) << 32;  // stride byte offset between 8-row groups
  d |= static_cast<uint64_t>(1) << 46;                    // descriptor version of sm_100 and later
  return d;                                               // base offset 0, no swizzle
}

// kind::f16 instruction descriptor: D fp32, A and B bf16, both K-major, N = 256, M = 128.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((kTcHidden >> 3) << 17) | ((kTcRows >> 4) << 24);

__device__ __forceinline__ void Mma(uint32_t tmem, uint64_t a, uint64_t b, bool accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
      "l"(a), "l"(b), "r"(kIdesc), "r"(accumulate ? 1 : 0));
}
__device__ __forceinline__ void Commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(Smem(bar)));
}
// Waits for the completion of the barrier phase with the given parity; false on expiry.
__device__ __forceinline__ bool WaitPhase(uint64_t *bar, uint32_t parity) {
  for (long long it = 0; it < kWaitLimit; ++it) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(Smem(bar)), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}
__device__ __forceinline__ void CpAsync16(void *smem, const void *gmem) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(Smem(smem)), "l"(gmem));
}
__device__ __forceinline__ void CpAsyncWaitAll() { asm volatile("cp.async.wait_all;" ::: "memory"); }
__device__ __forceinline__ void FenceAsyncSmem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void TmemLoad32(uint32_t addr, float *v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,"
      "%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(addr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int j = 0; j < 32; ++j) v[j] = __uint_as_float(r[j]);
}

// Loads rows [row0, row0 + rows) x K columns [k0, k0 + 64) of a row-major bf16
// matrix (leading dimension ld) into a 64-wide operand tile (zeros past `valid` rows).
__device__ __forceinline__ void LoadChunk(__nv_bfloat16 *dst, const __nv_bfloat16 *src, int ld, int rows, int valid,
                                          int k0) {
  char *d = reinterpret_cast<char *>(dst);
  for (int c = threadIdx.x; c < rows * 8; c += kTcThreads) {
    const int r = c >> 3, kc = c & 7;
    char *to = d + (r >> 3) * (kTcChunk / 8) * 128 + kc * 128 + (r & 7) * 16;
    if (r < valid) CpAsync16(to, src + static_cast<long long>(r) * ld + k0 + kc * 8);
    else *reinterpret_cast<uint4 *>(to) = make_uint4(0, 0, 0, 0);
  }
}

}  // namespace

__global__ void __launch_bounds__(kTcThreads, 1)
    mlp_tc_infer_kernel(MlpDev d, const __nv_bfloat16 *__restrict__ x, long long n, float mean_label, float std_label,
                        float *mean, float *spread, int *status) {
  extern __shared__ __align__(1024) unsigned char smem[];
  const int K1 = d.in, members = d.members;
  const int k1_chunks = K1 / kTcChunk, k2_chunks = kTcHidden / kTcChunk;
  // X tile as k1_chunks tiles of 128 x 64, H1 as 4 tiles of 128 x 64, two 256 x 64 weight buffers
  __nv_bfloat16 *sx = reinterpret_cast<__nv_bfloat16 *>(smem);
  __nv_bfloat16 *sh = sx + kTcRows * K1;
  __nv_bfloat16 *sw = sh + kTcRows * kTcHidden;
  float *partial = reinterpret_cast<float *>(sw + 2 * kTcHidden * kTcChunk);  // [128] second column half
  uint64_t *bar = reinterpret_cast<uint64_t *>(partial + kTcRows);
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bar + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int row = (warp & 3) * 32 + lane, half = warp >> 2;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(Smem(tmem_slot)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(Smem(bar)));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  const uint32_t d1 = tmem, d2 = tmem + kTcHidden;
  const uint32_t lane_base = static_cast<uint32_t>((warp & 3) * 32) << 16;

  uint32_t commits = 0;  // commits issued so far; commit j completes barrier phase j
  bool failed = false;
  const int chunks_per_member = k1_chunks + k2_chunks;
  const int chunks = members * chunks_per_member;
  const uint32_t sbo_w = kTcChunk * 16;  // 8-row group stride of a 64-wide operand tile
  const long long tiles = (n + kTcRows - 1) / kTcRows;

  auto chunk_src = [&](int q, const __nv_bfloat16 *&src, int &ld, int &k0) {
    const int m = q / chunks_per_member, c = q % chunks_per_member;
    if (c < k1_chunks) {
      src = d.w1h + static_cast<long long>(m) * kTcHidden * K1;
      ld = K1;
      k0 = c * kTcChunk;
    } else {
      src = d.w2h + static_cast<long long>(m) * kTcHidden * kTcHidden;
      ld = kTcHidden;
      k0 = (c - k1_chunks) * kTcChunk;
    }
  };

  for (long long tile = blockIdx.x; tile < tiles && !failed; tile += gridDim.x) {
    const long long r0 = tile * kTcRows;
    const int valid = static_cast<int>(n - r0 < kTcRows ? n - r0 : kTcRows);
    // X tile (one 128 x 64 operand tile per K chunk) and the first weight chunk
    for (int c = 0; c < k1_chunks; ++c)
      LoadChunk(sx + c * kTcRows * kTcChunk, x + r0 * K1, K1, kTcRows, valid, c * kTcChunk);
    {
      const __nv_bfloat16 *src;
      int ld, k0;
      chunk_src(0, src, ld, k0);
      LoadChunk(sw, src, ld, kTcHidden, kTcHidden, k0);
    }
    CpAsyncWaitAll();
    FenceAsyncSmem();
    __syncthreads();
    float ysum = 0.f, ymin = 3.4e38f, ymax = -3.4e38f;
    for (int q = 0; q < chunks && !failed; ++q) {
      const int m = q / chunks_per_member, c = q % chunks_per_member;
      // the buffer of chunk q + 1 was read by chunk q - 1: wait for it, then prefetch
      // (the failure flag is made uniform over the CTA before anyone branches on it)
      if (q >= 1) failed = __syncthreads_or(!WaitPhase(bar, (commits - 1) & 1));
      if (q + 1 < chunks && !failed) {
        const __nv_bfloat16 *src;
        int ld, k0;
        chunk_src(q + 1, src, ld, k0);
        LoadChunk(sw + ((q + 1) & 1) * kTcHidden * kTcChunk, src, ld, kTcHidden, kTcHidden, k0);
      }
      if (failed) break;
      if (tid == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t b = Smem(sw + (q & 1) * kTcHidden * kTcChunk);
        const bool layer1 = c < k1_chunks;
        const int kc = layer1 ? c : c - k1_chunks;
        const uint32_t a = layer1 ? Smem(sx + kc * kTcRows * kTcChunk) : Smem(sh + kc * kTcRows * kTcChunk);
#pragma unroll
        for (int s = 0; s < kTcChunk / 16; ++s)
          Mma(layer1 ? d1 : d2, OperandDesc(a + s * 256, sbo_w), OperandDesc(b + s * 256, sbo_w),
              kc > 0 || s > 0);
        Commit(bar);
      }
      ++commits;
      const bool end1 = c == k1_chunks - 1, end2 = c == chunks_per_member - 1;
      if (end1 || end2) {
        failed = __syncthreads_or(!WaitPhase(bar, (commits - 1) & 1));
        if (failed) break;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        if (end1) {
          // H1 = GELU(D1 + b1): this thread's row, columns [128 half, 128 half + 128)
          const float *b1 = d.b1 + m * kTcHidden;
#pragma unroll 1
          for (int j0 = 0; j0 < 128; j0 += 32) {
            float v[32];
            const int col0 = half * 128 + j0;
            TmemLoad32(d1 + lane_base + col0, v);
#pragma unroll
            for (int g = 0; g < 4; ++g) {
              uint32_t packed[4];
#pragma unroll
              for (int e = 0; e < 4; ++e) {
                const int col = col0 + g * 8 + 2 * e;
                const __nv_bfloat162 p = __floats2bfloat162_rn(MlpGelu(v[g * 8 + 2 * e] + __ldg(&b1[col])),
                                                               MlpGelu(v[g * 8 + 2 * e + 1] + __ldg(&b1[col + 1])));
                packed[e] = *reinterpret_cast<const uint32_t *>(&p);
              }
              const int col = col0 + g * 8;  // 8 consecutive columns: one 16-byte row of a core matrix
              char *to = reinterpret_cast<char *>(sh + (col / kTcChunk) * kTcRows * kTcChunk) + (row >> 3) * sbo_w +
                         ((col % kTcChunk) >> 3) * 128 + (row & 7) * 16;
              *reinterpret_cast<uint4 *>(to) = make_uint4(packed[0], packed[1], packed[2], packed[3]);
            }
          }
          asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
          FenceAsyncSmem();
        } else {
          // y_m = GELU(D2 + b2) . w3 + b3 over this thread's 128 columns
          const float *b2 = d.b2 + m * kTcHidden, *w3 = d.w3 + m * kTcHidden;
          float acc = 0.f;
#pragma unroll 1
          for (int j0 = 0; j0 < 128; j0 += 32) {
            float v[32];
            const int col0 = half * 128 + j0;
            TmemLoad32(d2 + lane_base + col0, v);
#pragma unroll
            for (int e = 0; e < 32; ++e) acc += MlpGelu(v[e] + __ldg(&b2[col0 + e])) * __ldg(&w3[col0 + e]);
          }
          asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
          if (half == 1) partial[row] = acc;
          __syncthreads();
          if (half == 0) {
            const float y = acc + partial[row] + __ldg(&d.b3[m]);
            ysum += y;
            ymin = fminf(ymin, y);
            ymax = fmaxf(ymax, y);
          }
        }
      }
      CpAsyncWaitAll();
      FenceAsyncSmem();
      __syncthreads();
    }
    if (!failed && half == 0 && row < valid) {
      mean[r0 + row] = mean_label + std_label * ysum / members;
      if (spread) spread[r0 + row] = std_label * (ymax - ymin);
    }
  }
  if (failed) {
    if (tid == 0) atomicOr(status, kMlpTimeout);
    WaitPhase(bar, (commits - 1) & 1);  // the last commit, bounded
  }
  CpAsyncWaitAll();
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
}

size_t MlpTcSharedBytes(int in) {
  return static_cast<size_t>(kTcRows) * in * 2 + static_cast<size_t>(kTcRows) * kTcHidden * 2 +
         2ull * kTcHidden * kTcChunk * 2 + kTcRows * 4 + 16 + 1024;
}

bool MlpTcSupported(const MlpDev &d) {
  return d.hidden == kTcHidden && d.in % kTcChunk == 0 && d.in <= 256 && d.members >= 1 && d.members <= 16;
}

cudaError_t MlpTcPredict(const MlpDev &d, const __nv_bfloat16 *x, long long n, float mean_label, float std_label,
                         float *mean, float *spread, int *status, cudaStream_t s) {
  if (!MlpTcSupported(d)) return cudaErrorInvalidValue;
  if (n <= 0) return cudaSuccess;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long tiles = (n + kTcRows - 1) / kTcRows;
  const int grid = static_cast<int>(tiles < sms ? tiles : sms);
  const size_t sm = MlpTcSharedBytes(d.in);
  cudaError_t err = cudaFuncSetAttribute(mlp_tc_infer_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(sm));
  if (err != cudaSuccess) return err;
  mlp_tc_infer_kernel<<<grid, kTcThreads, sm, s>>>(d, x, n, mean_label, std_label, mean, spread, status);
  return cudaGetLastError();
}

}  // namespace lmc
