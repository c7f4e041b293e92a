// Training GEMMs of the barrier surrogate on the 5th-generation tensor cores:
// C[m][n] = sum_k A[m][k] B[n][k] with BF16 operands (both K-major, as the
// mma.sync kernel of mlp.cu takes them) and FP32 accumulators in TMEM, batched
// over grid.z, with the same fused epilogues (store, bias + GELU, GELU gradient).
//
// One CTA of 4 warps per 128 x BN tile (BN = 256, 128 or 64, the largest that
// divides N). The K loop streams 128 x 32 A tiles and BN x 32 B tiles into a
// 3-stage shared-memory ring with cp.async (every thread copies 16-byte pieces
// into the core-matrix layout of tcgen05.cuh, then fences them to the async
// proxy); one thread issues two tcgen05.mma (K = 16 each) per stage and commits
// them to the stage's mbarrier, which the copy of the tile three stages later
// waits on. After the last stage a final commit releases the epilogue: warp w
// reads TMEM lanes 32w..32w+31 (its rows) 32 columns at a time with
// tcgen05.ld and writes the outputs. Every wait is bounded; on expiry the CTA
// records *status, drains its MMAs (bounded), frees its TMEM and writes nothing.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "mlp.cuh"
#include "tcgen05.cuh"

namespace lmc {
namespace {

constexpr int kGm = 128;     // tile rows (MMA M)
constexpr int kGk = tc::kK;  // K per stage
constexpr int kGStages = 4;
constexpr int kGThreads = 128;

struct GemmTcBars {
  uint64_t mma_done[kGStages];
  uint64_t done;
  int abort;
  uint32_t tmem;
};

// Dynamic shared memory of a CTA: the ring and the barriers, raised where needed so that no
// more CTAs fit on an SM than its 512 TMEM columns hold (512 / BN), and a TMEM
// allocation never has to wait for another CTA.
size_t GemmTcSmemBytes(int bn) {
  const size_t need = static_cast<size_t>(kGStages) * (kGm + bn) * kGk * 2 + sizeof(GemmTcBars);
  const size_t ctas = 512 / static_cast<size_t>(bn);          // CTAs whose TMEM fits one SM
  const size_t floor = 228 * 1024 / (ctas + 1) + 1024;        // more than a share of ctas + 1
  return need > floor ? need : floor;
}

template <int kEpi>
__global__ void __launch_bounds__(kGThreads) gemm_tc_kernel(GemmArgs g, int bn, int *status) {
  extern __shared__ __align__(1024) unsigned char smem[];
  const int a_bytes = kGm * kGk * 2, stage_bytes = (kGm + bn) * kGk * 2;
  GemmTcBars *bars = reinterpret_cast<GemmTcBars *>(smem + kGStages * stage_bytes);
  volatile int *abort = &bars->abort;
  // grid.z = batch x splits: member z, K range of split `split`
  const int splits = g.splits > 1 ? g.splits : 1;
  const int z = blockIdx.z / splits, split = blockIdx.z % splits;
  const __nv_bfloat16 *A = g.a + z * g.stride_a;
  const __nv_bfloat16 *B = g.b + z * g.stride_b;
  const int m0 = blockIdx.y * kGm, n0 = blockIdx.x * bn;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t cols = static_cast<uint32_t>(bn);

  if (tid == 0) {
    for (int s = 0; s < kGStages; ++s) tc::BarInit(&bars->mma_done[s], 1);
    tc::BarInit(&bars->done, 1);
    bars->abort = 0;
    tc::FenceBarrierInit();
  }
  if (warp == 0) tc::TmemAlloc(&bars->tmem, cols);
  tc::FenceBeforeSync();
  __syncthreads();
  tc::FenceAfterSync();
  const uint32_t tmem = bars->tmem;
  const uint32_t idesc = tc::IdescBf16(kGm, bn);
  const int ktiles = g.k / kGk / splits;
  const int kbase = split * ktiles * kGk;

  // copies K tile j into its stage: 4 x 16-byte pieces per row of A and of B
  auto load = [&](int j) {
    unsigned char *base = smem + (j % kGStages) * stage_bytes;
    const int k0 = kbase + j * kGk;
    for (int c = tid; c < kGm * 4; c += kGThreads) {
      const int r = c >> 2, kc = (c & 3) * 8;
      tc::CpAsync16(base + tc::CoreOffset(r, kc), A + static_cast<long long>(m0 + r) * g.lda + k0 + kc);
    }
    for (int c = tid; c < bn * 4; c += kGThreads) {
      const int r = c >> 2, kc = (c & 3) * 8;
      tc::CpAsync16(base + a_bytes + tc::CoreOffset(r, kc), B + static_cast<long long>(n0 + r) * g.ldb + k0 + kc);
    }
  };

  // prologue: the first kGStages - 1 tiles (one commit group each, empty past the end)
  for (int j = 0; j < kGStages - 1; ++j) {
    if (j < ktiles) load(j);
    tc::CpAsyncCommit();
  }
  for (int kt = 0; kt < ktiles; ++kt) {
    const int j = kt + kGStages - 1;
    if (j < ktiles) {
      // the stage of tile j last held tile j - kGStages: its MMAs must have finished reading it
      const int i = j - kGStages;
      const bool free_stage = i < 0 || tc::Wait(&bars->mma_done[i % kGStages], (i / kGStages) & 1, abort);
      if (free_stage) load(j);
    }
    tc::CpAsyncCommit();
    tc::CpAsyncWait<kGStages - 1>();  // tile kt has landed
    tc::FenceAsyncSmem();
    __syncthreads();
    if (tid == 0 && !*abort) {
      tc::FenceAfterSync();
      const uint32_t a = tc::Smem(smem + (kt % kGStages) * stage_bytes), b = a + a_bytes;
      tc::Mma(tmem, tc::OperandDesc(a), tc::OperandDesc(b), idesc, kt > 0);
      tc::Mma(tmem, tc::OperandDesc(a + 256), tc::OperandDesc(b + 256), idesc, true);
      tc::Commit(&bars->mma_done[kt % kGStages]);
    }
  }
  tc::CpAsyncWait<0>();
  if (tid == 0) tc::Commit(&bars->done);  // completes when every MMA issued above has finished
  if (!tc::WaitDrain(&bars->done, 0)) *abort = 1;
  tc::FenceAfterSync();
  __syncthreads();

  if (!*abort) {
    const int row = m0 + warp * 32 + lane;
    const uint32_t lane_base = static_cast<uint32_t>(warp * 32) << 16;
    for (int col0 = 0; col0 < bn; col0 += 32) {
      float v[32];
      tc::TmemLoad32(tmem + lane_base + static_cast<uint32_t>(col0), v);
      const int n = n0 + col0;
      if (kEpi == kEpiStoreF32) {
        if (splits > 1) {  // raw partial tile, summed and scaled by splitk_reduce_kernel
          float4 *out = reinterpret_cast<float4 *>(
              g.ws + ((static_cast<long long>(split) * gridDim.z / splits + z) * g.m + row) * g.n + n);
#pragma unroll
          for (int e = 0; e < 8; ++e) out[e] = make_float4(v[4 * e], v[4 * e + 1], v[4 * e + 2], v[4 * e + 3]);
        } else {
          float4 *out = reinterpret_cast<float4 *>(g.c + z * g.stride_c + static_cast<long long>(row) * g.ldc + n);
#pragma unroll
          for (int e = 0; e < 8; ++e)
            out[e] = make_float4(g.alpha * v[4 * e], g.alpha * v[4 * e + 1], g.alpha * v[4 * e + 2],
                                 g.alpha * v[4 * e + 3]);
        }
      } else {
        float *zrow = g.c + z * g.stride_c + static_cast<long long>(row) * g.ldc + n;
        __nv_bfloat16 *hrow = g.h + z * g.stride_h + static_cast<long long>(row) * g.ldh + n;
        alignas(16) __nv_bfloat16 out[32];
        if (kEpi == kEpiBiasGelu) {
          const float *bias = g.bias + z * g.stride_bias + n;
#pragma unroll
          for (int e = 0; e < 32; e += 4) {
            const float4 bb = *reinterpret_cast<const float4 *>(bias + e);
            const float4 zz = make_float4(v[e] + bb.x, v[e + 1] + bb.y, v[e + 2] + bb.z, v[e + 3] + bb.w);
            *reinterpret_cast<float4 *>(zrow + e) = zz;
            out[e] = __float2bfloat16(MlpGelu(zz.x));
            out[e + 1] = __float2bfloat16(MlpGelu(zz.y));
            out[e + 2] = __float2bfloat16(MlpGelu(zz.z));
            out[e + 3] = __float2bfloat16(MlpGelu(zz.w));
          }
        } else {
#pragma unroll
          for (int e = 0; e < 32; e += 4) {
            const float4 zz = *reinterpret_cast<const float4 *>(zrow + e);
            out[e] = __float2bfloat16(v[e] * MlpGeluGrad(zz.x));
            out[e + 1] = __float2bfloat16(v[e + 1] * MlpGeluGrad(zz.y));
            out[e + 2] = __float2bfloat16(v[e + 2] * MlpGeluGrad(zz.z));
            out[e + 3] = __float2bfloat16(v[e + 3] * MlpGeluGrad(zz.w));
          }
        }
#pragma unroll
        for (int e = 0; e < 32; e += 8)
          *reinterpret_cast<uint4 *>(hrow + e) = *reinterpret_cast<const uint4 *>(out + e);
        if (g.ht) {
          // transposed copy: for each column, the warp's 32 consecutive rows (64 contiguous bytes)
          __nv_bfloat16 *ht = g.ht + z * g.stride_ht + static_cast<long long>(n) * g.ldt + row;
#pragma unroll
          for (int e = 0; e < 32; ++e) ht[static_cast<long long>(e) * g.ldt] = out[e];
        }
      }
    }
  }
  tc::FenceBeforeSync();
  __syncthreads();
  if (tid == 0 && *abort) atomicOr(status, 1);
  if (warp == 0) tc::TmemFree(tmem, cols);
}

// C[z][row][col] = alpha * sum over the splits, in split order, of the partial tiles.
__global__ void splitk_reduce_kernel(const float *ws, int splits, int batch, int m, int n, float alpha, float *c,
                                     int ldc, long long stride_c) {
  const long long total = static_cast<long long>(batch) * m * n;
  const long long plane = total;
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < total;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    float s = 0.f;
    for (int q = 0; q < splits; ++q) s += ws[q * plane + i];
    const long long z = i / (static_cast<long long>(m) * n), r = (i / n) % m, col = i % n;
    c[z * stride_c + r * ldc + col] = alpha * s;
  }
}

int TileN(int n) { return n % 256 == 0 ? 256 : (n % 128 == 0 ? 128 : 64); }

}  // namespace

bool GemmTcFits(const GemmArgs &g) {
  auto al8 = [](long long v) { return v % 8 == 0; };
  auto al16 = [](const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; };
  if (g.m <= 0 || g.n <= 0 || g.k <= 0 || g.m % kGm || g.n % 64 || g.k % kGk) return false;
  if (!al8(g.lda) || !al8(g.ldb) || !al8(g.stride_a) || !al8(g.stride_b) || !al16(g.a) || !al16(g.b)) return false;
  if (!al8(g.ldc) || !al8(g.stride_c) || !al16(g.c)) return false;  // float4 rows of C / Z
  if (g.h && (!al8(g.ldh) || !al8(g.stride_h) || !al16(g.h))) return false;
  if (g.bias && (!al8(g.stride_bias) || !al16(g.bias))) return false;
  return true;
}

cudaError_t GemmTc(const GemmArgs &g, int epi, int batch, int *status, cudaStream_t s) {
  if (!GemmTcFits(g) || batch <= 0) return cudaErrorInvalidValue;
  const int splits = g.splits > 1 ? g.splits : 1;
  if (splits > 1 && (epi != kEpiStoreF32 || !g.ws || (g.k / kGk) % splits)) return cudaErrorInvalidValue;
  const int bn = TileN(g.n);
  const size_t sm = GemmTcSmemBytes(bn);
  const dim3 grid(g.n / bn, g.m / kGm, batch * splits);
  cudaError_t err;
  switch (epi) {
    case kEpiStoreF32:
      err = cudaFuncSetAttribute(gemm_tc_kernel<kEpiStoreF32>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(sm));
      if (err != cudaSuccess) return err;
      gemm_tc_kernel<kEpiStoreF32><<<grid, kGThreads, sm, s>>>(g, bn, status);
      if (splits > 1) {
        err = cudaGetLastError();
        if (err != cudaSuccess) return err;
        const long long total = static_cast<long long>(batch) * g.m * g.n;
        const int blocks = static_cast<int>(std::min<long long>((total + 255) / 256, 4096));
        splitk_reduce_kernel<<<blocks, 256, 0, s>>>(g.ws, splits, batch, g.m, g.n, g.alpha, g.c, g.ldc, g.stride_c);
      }
      break;
    case kEpiBiasGelu:
      err = cudaFuncSetAttribute(gemm_tc_kernel<kEpiBiasGelu>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(sm));
      if (err != cudaSuccess) return err;
      gemm_tc_kernel<kEpiBiasGelu><<<grid, kGThreads, sm, s>>>(g, bn, status);
      break;
    case kEpiGeluGrad:
      err = cudaFuncSetAttribute(gemm_tc_kernel<kEpiGeluGrad>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(sm));
      if (err != cudaSuccess) return err;
      gemm_tc_kernel<kEpiGeluGrad><<<grid, kGThreads, sm, s>>>(g, bn, status);
      break;
    default:
      return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace lmc
