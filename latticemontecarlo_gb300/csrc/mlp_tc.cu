// Fused ensemble inference of the barrier surrogate on the 5th-generation
// tensor cores (tcgen05): one persistent CTA per SM walks tiles of 128 samples.
// Per tile and member m:
//   D1 (TMEM, 128 x 256 fp32) = X (smem, bf16) . W1[m]^T (bf16)   tcgen05.mma kind::f16
//   H1 (smem, IEEE half)       = GELU(D1 + b1[m])   epilogue warps (tcgen05.ld, packed half GELU)
//   D2 (TMEM)                  = H1 . W2[m]^T (half)               tcgen05.mma kind::f16
//   y_m                        = GELU(D2 + b2[m]) . w3[m] + b3[m]
// then the ensemble mean and spread.
//
// Warp roles, coordinated by mbarriers (no block-wide barrier inside the loop):
//   warp 0     producer: cp.async of the X tiles (fence.proxy.async, then arrive),
//              and one bulk copy (cp.async.bulk, completing on the stage's
//              mbarrier) per weight block of 256 rows x 32 K (16 KB, pre-tiled in
//              global memory) into a ring of kStages buffers;
//   warp 1     one thread issues the MMAs and the tcgen05.commit arrivals;
//   warps 2-17 epilogue: TMEM lane group = warp % 4, column quarter = (warp - 2) / 4.
// The layer-1 MMAs of member m + 1 overlap the layer-2 epilogue of member m.
//
// Operand layout in shared memory (K-major, no swizzle): 8-row x 16-byte core
// matrices; an operand tile of 32 K columns keeps element (r, k) at
//   (r / 8) * 512 + (k / 8) * 128 + (r % 8) * 16 + (k % 8) * 2,
// i.e. leading (K) byte offset 128 and 8-row stride 512; X and H1 are stored as
// consecutive such tiles. Every wait is bounded and also polls a shared abort
// flag: on expiry the kernel records kMlpTimeout, drains its MMAs (bounded wait
// on a final commit) and its copies, frees its TMEM and returns.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "mlp.cuh"
#include "tcgen05.cuh"

namespace lmc {
namespace {

using tc::Arrive;
using tc::ArriveExpectTx;
using tc::BarInit;
using tc::BulkCopy;
using tc::Commit;
using tc::CpAsync16;
using tc::CpAsyncCommit;
using tc::CpAsyncWait;
using tc::FenceAsyncSmem;
using tc::Mma;
using tc::OperandDesc;
using tc::Smem;
using tc::TmemLoad32;
using tc::Wait;
using tc::WaitDrain;

constexpr int kTcRows = 128;     // samples per tile (MMA M)
constexpr int kTcHidden = 256;   // MMA N and the hidden width
constexpr int kTcK = 32;         // K per operand tile / weight chunk
constexpr int kTcTile = kTcRows * kTcK;           // elements of a 128 x 32 operand tile
constexpr int kTcChunkElems = kTcHidden * kTcK;   // elements of a 256 x 32 weight chunk (16 KB)
constexpr int kTcStages = 6;
constexpr int kEpiWarps = 16;    // 4 per TMEM lane group, 64 columns each
constexpr int kTcThreads = 64 + 32 * kEpiWarps;  // producer, MMA issuer, epilogue
constexpr uint32_t kTmemCols = 512;
constexpr int kMlpTimeout = 1;
constexpr uint32_t kSbo = kTcK * 16;  // 8-row group stride of a 32-wide operand tile

// kind::f16 instruction descriptors: D fp32, both operands K-major, N = 256, M = 128;
// layer 1 reads bf16 A and B (features, W1), layer 2 IEEE half A and B (H1, W2).
constexpr uint32_t kIdescBf16 =
    (1u << 4) | (1u << 7) | (1u << 10) | ((kTcHidden >> 3) << 17) | ((kTcRows >> 4) << 24);
constexpr uint32_t kIdescF16 = (1u << 4) | ((kTcHidden >> 3) << 17) | ((kTcRows >> 4) << 24);

// GELU of two values in packed half precision (layer-1 epilogue: H1 is stored in
// half for the layer-2 MMA): u = z (c0 + c1 z^2), GELU = h + h tanh(u), h = z / 2.
__device__ __forceinline__ __half2 GeluHalf2(__half2 z) {
  const __half2 u = __hmul2(z, __hfma2(__hmul2(z, z), __float2half2_rn(0.0356774081363001f),
                                       __float2half2_rn(0.7978845608028654f)));
  uint32_t ub = *reinterpret_cast<const uint32_t *>(&u), tb;
  asm("tanh.approx.f16x2 %0, %1;" : "=r"(tb) : "r"(ub));
  const __half2 t = *reinterpret_cast<const __half2 *>(&tb);
  const __half2 h = __hmul2(z, __float2half2_rn(0.5f));
  return __hfma2(h, t, h);
}

// Byte offset of element (r, k) in a sequence of 32-wide operand tiles of `rows` rows.
__device__ __forceinline__ uint32_t TileOffset(int rows, int r, int k) {
  return static_cast<uint32_t>((k / kTcK) * rows * kTcK * 2 + (r >> 3) * kSbo + ((k % kTcK) >> 3) * 128 + (r & 7) * 16);
}

struct TcBars {
  uint64_t full[kTcStages], empty[kTcStages];
  uint64_t x_full, x_empty, d1_full, d1_empty, h1_full, h1_empty, d2_full, d2_empty, part_full, part_empty, done;
  int abort;
  uint32_t tmem;
  float partial[3][kTcRows];  // column quarters 1-3 of each row's output dot product
};

}  // namespace

__global__ void __launch_bounds__(kTcThreads, 1)
    mlp_tc_infer_kernel(MlpDev d, const __nv_bfloat16 *__restrict__ x, long long n, float mean_label, float std_label,
                        float *mean, float *spread, int *status) {
  extern __shared__ __align__(1024) unsigned char smem[];
  const int K1 = d.in, members = d.members;
  const int k1_tiles = K1 / kTcK, k2_tiles = kTcHidden / kTcK;
  __nv_bfloat16 *sx = reinterpret_cast<__nv_bfloat16 *>(smem);         // k1_tiles x (128 x 32)
  __nv_bfloat16 *sh = sx + kTcRows * K1;                                // 8 x (128 x 32), IEEE half H1
  __nv_bfloat16 *sw = sh + kTcRows * kTcHidden;                         // kStages x (256 x 32), W1 bf16 / W2 half
  TcBars *bars = reinterpret_cast<TcBars *>(sw + kTcStages * kTcChunkElems);
  volatile int *abort = &bars->abort;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  if (tid == 0) {
    for (int i = 0; i < kTcStages; ++i) {
      BarInit(&bars->full[i], 1);
      BarInit(&bars->empty[i], 1);
    }
    BarInit(&bars->x_full, 32);
    BarInit(&bars->x_empty, 1);
    BarInit(&bars->d1_full, 1);
    BarInit(&bars->d1_empty, kEpiWarps);
    BarInit(&bars->h1_full, kEpiWarps);
    BarInit(&bars->h1_empty, 1);
    BarInit(&bars->d2_full, 1);
    BarInit(&bars->d2_empty, kEpiWarps);
    BarInit(&bars->part_full, 3 * 4);
    BarInit(&bars->part_empty, 4);
    BarInit(&bars->done, 1);
    bars->abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(Smem(&bars->tmem)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = bars->tmem;
  const uint32_t d1 = tmem, d2 = tmem + kTcHidden;
  const long long tiles = (n + kTcRows - 1) / kTcRows;
  const int chunks_per_member = k1_tiles + k2_tiles;

  if (warp == 0) {
    // ---- producer: X tiles with cp.async (all lanes; fence, then arrive on x_full),
    // weight blocks with one bulk copy each (lane 0; completes on the stage's full barrier) ----
    long long g = 0;  // weight blocks issued
    int t_local = 0;
    bool stop = false;
    for (long long tile = blockIdx.x; tile < tiles && !stop; tile += gridDim.x, ++t_local) {
      const long long r0 = tile * kTcRows;
      const int valid = static_cast<int>(n - r0 < kTcRows ? n - r0 : kTcRows);
      if (t_local >= 1 && !Wait(&bars->x_empty, (t_local - 1) & 1, abort)) break;
      for (int c = lane; c < kTcRows * (K1 / 8); c += 32) {
        const int r = c / (K1 / 8), k = (c % (K1 / 8)) * 8;
        char *to = reinterpret_cast<char *>(sx) + TileOffset(kTcRows, r, k);
        if (r < valid) CpAsync16(to, x + (r0 + r) * K1 + k);
        else *reinterpret_cast<uint4 *>(to) = make_uint4(0, 0, 0, 0);
      }
      CpAsyncCommit();
      CpAsyncWait<0>();
      FenceAsyncSmem();
      Arrive(&bars->x_full);
      if (lane == 0) {
        for (int m = 0; m < members && !stop; ++m)
          for (int c = 0; c < chunks_per_member; ++c, ++g) {
            const int s = static_cast<int>(g % kTcStages);
            const long long round = g / kTcStages;
            if (round >= 1 && !Wait(&bars->empty[s], (round - 1) & 1, abort)) {
              stop = true;
              break;
            }
            const void *src =
                c < k1_tiles
                    ? static_cast<const void *>(d.w1_tiles + (static_cast<long long>(m) * k1_tiles + c) * kTcChunkElems)
                    : static_cast<const void *>(d.w2_tiles +
                                                (static_cast<long long>(m) * k2_tiles + (c - k1_tiles)) * kTcChunkElems);
            ArriveExpectTx(&bars->full[s], kTcChunkElems * 2);
            BulkCopy(sw + s * kTcChunkElems, src, kTcChunkElems * 2, &bars->full[s]);
          }
      }
      stop = __shfl_sync(0xffffffffu, stop ? 1 : 0, 0) != 0;
    }
    CpAsyncWait<0>();
  } else if (warp == 1) {
    // ---- MMA issuer ----
    if (lane == 0) {
      long long g = 0;
      int u = 0, t_local = 0;
      bool ok = true;
      for (long long tile = blockIdx.x; tile < tiles && ok; tile += gridDim.x, ++t_local) {
        ok = Wait(&bars->x_full, t_local & 1, abort);
        for (int m = 0; m < members && ok; ++m, ++u) {
          if (u >= 1 && !(ok = Wait(&bars->d1_empty, (u - 1) & 1, abort))) break;
          for (int c = 0; c < k1_tiles && ok; ++c, ++g) {
            const int s = static_cast<int>(g % kTcStages);
            if (!(ok = Wait(&bars->full[s], (g / kTcStages) & 1, abort))) break;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t a = Smem(sx + c * kTcTile), b = Smem(sw + s * kTcChunkElems);
            Mma(d1, OperandDesc(a), OperandDesc(b), kIdescBf16, c > 0);
            Mma(d1, OperandDesc(a + 256), OperandDesc(b + 256), kIdescBf16, true);
            Commit(&bars->empty[s]);
          }
          if (!ok) break;
          Commit(&bars->d1_full);
          if (m == members - 1) Commit(&bars->x_empty);
          if (!(ok = Wait(&bars->h1_full, u & 1, abort))) break;
          if (u >= 1 && !(ok = Wait(&bars->d2_empty, (u - 1) & 1, abort))) break;
          for (int c = 0; c < k2_tiles && ok; ++c, ++g) {
            const int s = static_cast<int>(g % kTcStages);
            if (!(ok = Wait(&bars->full[s], (g / kTcStages) & 1, abort))) break;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t a = Smem(sh + c * kTcTile), b = Smem(sw + s * kTcChunkElems);
            Mma(d2, OperandDesc(a), OperandDesc(b), kIdescF16, c > 0);
            Mma(d2, OperandDesc(a + 256), OperandDesc(b + 256), kIdescF16, true);
            Commit(&bars->empty[s]);
          }
          if (!ok) break;
          Commit(&bars->d2_full);
          Commit(&bars->h1_empty);
        }
      }
      // drain: the done barrier completes when every MMA issued so far has finished
      Commit(&bars->done);
      if (!WaitDrain(&bars->done, 0)) *abort = 1;
    }
    __syncwarp();
  } else {
    // ---- epilogue warps ----
    const int ew = warp - 2, quarter = ew >> 2;  // columns [64 quarter, 64 quarter + 64)
    const int row = (warp & 3) * 32 + lane;
    const uint32_t lane_base = static_cast<uint32_t>((warp & 3) * 32) << 16;
    int u = 0;
    bool ok = true;
    for (long long tile = blockIdx.x; tile < tiles && ok; tile += gridDim.x) {
      const long long r0 = tile * kTcRows;
      const int valid = static_cast<int>(n - r0 < kTcRows ? n - r0 : kTcRows);
      float ysum = 0.f, ymin = 3.4e38f, ymax = -3.4e38f;
      for (int m = 0; m < members && ok; ++m, ++u) {
        // H1 = GELU(D1 + b1): this thread's row, its column quarter
        if (!(ok = Wait(&bars->d1_full, u & 1, abort))) break;
        if (u >= 1 && !(ok = Wait(&bars->h1_empty, (u - 1) & 1, abort))) break;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const float *b1 = d.b1 + m * kTcHidden;
#pragma unroll 1
        for (int j0 = 0; j0 < 64; j0 += 32) {
          float v[32];
          const int col0 = quarter * 64 + j0;
          TmemLoad32(d1 + lane_base + col0, v);
#pragma unroll
          for (int g8 = 0; g8 < 4; ++g8) {
            // the 8 biases of this 16-byte row (one broadcast load per 4 columns)
            const float4 ba = __ldg(reinterpret_cast<const float4 *>(b1 + col0 + g8 * 8));
            const float4 bb = __ldg(reinterpret_cast<const float4 *>(b1 + col0 + g8 * 8 + 4));
            const float bias[8] = {ba.x, ba.y, ba.z, ba.w, bb.x, bb.y, bb.z, bb.w};
            uint32_t packed[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
              const __half2 p = GeluHalf2(
                  __floats2half2_rn(v[g8 * 8 + 2 * e] + bias[2 * e], v[g8 * 8 + 2 * e + 1] + bias[2 * e + 1]));
              packed[e] = *reinterpret_cast<const uint32_t *>(&p);
            }
            *reinterpret_cast<uint4 *>(reinterpret_cast<char *>(sh) + TileOffset(kTcRows, row, col0 + g8 * 8)) =
                make_uint4(packed[0], packed[1], packed[2], packed[3]);
          }
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        FenceAsyncSmem();
        __syncwarp();
        if (lane == 0) {
          Arrive(&bars->d1_empty);
          Arrive(&bars->h1_full);
        }
        // y_m = GELU(D2 + b2) . w3 + b3
        if (!(ok = Wait(&bars->d2_full, u & 1, abort))) break;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const float *b2 = d.b2 + m * kTcHidden, *w3 = d.w3 + m * kTcHidden;
        float acc = 0.f;
#pragma unroll 1
        for (int j0 = 0; j0 < 64; j0 += 32) {
          float v[32];
          const int col0 = quarter * 64 + j0;
          TmemLoad32(d2 + lane_base + col0, v);
#pragma unroll
          for (int e = 0; e < 32; e += 4) {
            const float4 bb = __ldg(reinterpret_cast<const float4 *>(b2 + col0 + e));
            const float4 ww = __ldg(reinterpret_cast<const float4 *>(w3 + col0 + e));
            acc += MlpGelu(v[e] + bb.x) * ww.x + MlpGelu(v[e + 1] + bb.y) * ww.y + MlpGelu(v[e + 2] + bb.z) * ww.z +
                   MlpGelu(v[e + 3] + bb.w) * ww.w;
          }
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncwarp();
        if (lane == 0) Arrive(&bars->d2_empty);
        // the four column quarters of a row meet in shared memory: quarters 1-3
        // publish (part_full), quarter 0 consumes and releases the slots (part_empty)
        if (quarter != 0) {
          if (u >= 1 && !(ok = Wait(&bars->part_empty, (u - 1) & 1, abort))) break;
          bars->partial[quarter - 1][row] = acc;
          __syncwarp();
          if (lane == 0) Arrive(&bars->part_full);
        } else {
          if (!(ok = Wait(&bars->part_full, u & 1, abort))) break;
          const float y = acc + (bars->partial[0][row] + bars->partial[1][row] + bars->partial[2][row]) +
                          __ldg(&d.b3[m]);
          __syncwarp();
          if (lane == 0) Arrive(&bars->part_empty);
          ysum += y;
          ymin = fminf(ymin, y);
          ymax = fmaxf(ymax, y);
        }
      }
      if (ok && quarter == 0 && row < valid) {
        mean[r0 + row] = mean_label + std_label * ysum / members;
        if (spread) spread[r0 + row] = std_label * (ymax - ymin);
      }
    }
  }
  __syncthreads();
  if (tid == 0 && bars->abort) atomicOr(status, kMlpTimeout);
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 1) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
}

size_t MlpTcSharedBytes(int in) {
  return static_cast<size_t>(kTcRows) * in * 2 + static_cast<size_t>(kTcRows) * kTcHidden * 2 +
         static_cast<size_t>(kTcStages) * kTcChunkElems * 2 + sizeof(TcBars);
}

bool MlpTcSupported(const MlpDev &d) {
  return d.hidden == kTcHidden && d.in % 64 == 0 && d.in <= 256 && d.members >= 1 && d.members <= 16 &&
         MlpTcSharedBytes(d.in) <= 227 * 1024;
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
