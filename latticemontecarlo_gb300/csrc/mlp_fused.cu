// Fused surrogate barriers of lattice jumps for a compact ensemble whose weights
// stay in shared memory: 2 members of in -> 128 -> 128 -> 1 (GELU) over the
// solute-channel features (kC channels per site, the base species all zero:
// 59 sites x kC inputs, padded to in = 128 for three-species alphabets, kC = 2,
// and to 192 for four, kC = 3). One persistent CTA per SM loads both members'
// weights once (128 / 160 KB, two bulk copies) and walks tiles of 128 jumps.
// Per tile and member m:
//   X  (smem, bf16)        the features, gathered from the lattice by the producer warps
//   D  (TMEM, fp32)        = (X . W1[m]^T + b1[m]) / 2     tcgen05.mma kind::f16, A and B in smem
//   H1 (TMEM, IEEE half)   = GELU(2 D)                     epilogue warps (tcgen05.ld, tcgen05.st)
//   D  (TMEM, same columns)= H1 . W2[m]^T / 2 (half)       tcgen05.mma kind::f16, A in TMEM
//   y_m                    = GELU(2 (D + b2[m] / 2)) . w3[m] + b3[m]   packed half, FP32 sums of 8
// then the ensemble mean and spread. The layer-1 bias is the last input column: the
// producer sets feature in - 1 (padding in the solute encoding) to 1 and the weight
// tiles hold b1 there. W1, b1, W2 and b2 are stored halved (exact in binary floating
// point), so the MMAs produce h = z / 2 and GELU(z) = h + h tanh(h (2 c0 + 8 c1 h^2))
// takes one multiply less. A row whose pair is not a 1NN jump inside the lattice, or
// whose environment holds a species without a one-hot slot (a second vacancy), gets
// spread = +inf, so the caller's fallback sends it to the plain predictor.
//
// Warp roles (mbarriers only, no block-wide barrier inside the loop):
//   warps 0-7   producer: row r of the tile is gathered by threads r of warps 0-3
//               (its direction and sites 0-31: the first half of the row) and of
//               warps 4-7 (sites 32-58, the migrant being site 58), with
//               independent loads issued before the wait for the X buffer; each
//               writes its half of the row into the operand layout; warp 0 lane 0
//               also issues the weight copies;
//   warp 8      lane 0 issues the MMAs and the tcgen05.commit arrivals;
//   warps 9-24  epilogue: TMEM lane group = warp % 4, 32-column quarter =
//               (warp - 9) / 4.
// TMEM (512 columns allocated): member m owns columns [192 m, 192 m + 192): D in the
// first 128 (layer 1, then layer 2 once H1 is written), H1 in the last 64 (128 half
// values per row). The members give the pipeline its overlap: the layer-1 MMAs of the
// next tile's member m start once the epilogue has read member m's layer-2 result,
// while it works on the other member.
//
// Operand layout in shared memory: K-major 8-row x 16-byte core matrices, 32-wide K
// tiles of 128 rows (tcgen05.cuh); the gather, MMA and epilogue pieces are in mlp_fused.cuh. Every wait is bounded (sleeping probes, 2 s of wall
// time) and polls a shared abort flag: on expiry the kernel records kMlpFusedTimeout,
// drains its MMAs and copies, frees its TMEM and returns.
#include <cuda_runtime.h>

#include <cstdint>

#include "mlp_fused.cuh"

namespace lmc {
namespace {

using namespace fused;
using tc::Arrive;
using tc::ArriveExpectTx;
using tc::BarInit;
using tc::BulkCopy;
using tc::Commit;
using tc::FenceAfterSync;
using tc::FenceAsyncSmem;
using tc::FenceBarrierInit;
using tc::FenceBeforeSync;
using tc::Smem;
using tc::TmemAlloc;
using tc::TmemFree;
using tc::TmemLoad32;
using tc::WaitDrain;
using tc::WaitSleep;

constexpr int kProdWarps = 8;  // two per row: sites [0, 32) and [32, 64)
constexpr int kMmaWarp = kProdWarps;
constexpr int kFirstEpi = kProdWarps + 1;
constexpr int kEpiWarps = 16;
constexpr int kThreads = 32 * (kFirstEpi + kEpiWarps);
constexpr int kFlagRing = 4;

struct FusedBars {
  uint64_t w_full, x_full, x_empty;
  uint64_t acc_full[kMembers];   // phases 2t (layer 1 of tile t) and 2t + 1 (layer 2)
  uint64_t acc_empty[kMembers];  // the epilogue has read layer 2 of the member's tile
  uint64_t h1_full[kMembers];
  uint64_t flag_full[kFlagRing];
  uint64_t part_full, part_empty, done;
  int abort;
  uint32_t tmem;
  uint32_t site_word[8];                 // kC = 2: per species code, the row word of a site
  int8_t chan[8];                        // per species code: its channel, -1 none
  float partial[3][kRows];               // column quarters 1-3 of each row's output dot product
  uint32_t flag[kFlagRing][kProdWarps];  // per tile (ring) and producer warp: bit l set when row
                                         // (warp % 4) 32 + l goes to the plain predictor
};

template <int kC>
constexpr size_t SmemBytes() {
  return static_cast<size_t>(Shape<kC>::kW1Bytes) + kW2Bytes + Shape<kC>::kXBytes + sizeof(FusedBars);
}
static_assert(SmemBytes<3>() <= 232448, "the fused kernel's shared memory exceeds 227 KB");

// Bounded wait by lane 0 (sleeping probes), its outcome broadcast to the warp.
__device__ __forceinline__ bool WarpWait(uint64_t *bar, uint32_t parity, volatile int *abort, int lane) {
  int ok = 1;
  if (lane == 0) ok = WaitSleep(bar, parity, abort) ? 1 : 0;
  return __shfl_sync(0xffffffffu, ok, 0) != 0;
}

// Producer of half `half` (warps 0-3: 0, warps 4-7: 1) of every row of the CTA's tiles, with
// its loads issued before the wait for the feature buffer. One code path for both halves keeps
// the kernel's instruction footprint small. Returns the status bits of rejected pairs.
template <int kC>
__device__ __forceinline__ unsigned ProduceRows(const FusedJumps &j, long long m_rows, FusedBars *bars,
                                                unsigned char *sx, long long tiles, int warp, int lane,
                                                volatile int *abort) {
  const int half = warp >> 2;
  const int r = (warp & 3) * 32 + lane;
  unsigned bad_all = 0;
  int t_local = 0;
  for (long long tile = blockIdx.x; tile < tiles; tile += gridDim.x, ++t_local) {
    const long long row = tile * kRows + r;
    int code[32];
    bool fallback = true;
    if (row < m_rows) {
      unsigned bad = 0;
      fallback = LoadRowPart<2>(j, __ldg(&j.pairs[2 * row]), __ldg(&j.pairs[2 * row + 1]), half, code, &bad);
      if (half == 0) bad_all |= bad;
    }
    if (fallback) {
#pragma unroll
      for (int k = 0; k < 32; ++k) code[k] = -1;
    }
    // the X buffer is free once the previous tile's layer-1 MMAs have completed
    if (t_local >= 1 && !WarpWait(&bars->x_empty, (t_local - 1) & 1, abort, lane)) break;
    WriteRowPart<kC, 2>(code, bars->site_word, bars->chan, half, r, sx);
    const unsigned fb = __ballot_sync(0xffffffffu, fallback);
    if (lane == 0) bars->flag[t_local % kFlagRing][warp] = fb;
    FenceAsyncSmem();
    __syncwarp();
    if (lane == 0) {
      Arrive(&bars->x_full);
      Arrive(&bars->flag_full[t_local % kFlagRing]);
    }
  }
  return bad_all;
}

}  // namespace

constexpr int kMlpFusedTimeout = 1;

template <int kC>
__global__ void __launch_bounds__(kThreads, 1)
    mlp_fused_jump_kernel(const __grid_constant__ MlpDev d, const __grid_constant__ FusedJumps j, float mean_label,
                          float std_label, int *status) {
  using S = Shape<kC>;
  extern __shared__ __align__(1024) unsigned char smem[];
  unsigned char *sw1 = smem, *sw2 = sw1 + S::kW1Bytes, *sx = sw2 + kW2Bytes;
  FusedBars *bars = reinterpret_cast<FusedBars *>(sx + S::kXBytes);
  volatile int *abort = &bars->abort;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  if (tid == 0) {
    BarInit(&bars->w_full, 1);
    BarInit(&bars->x_full, kProdWarps);
    BarInit(&bars->x_empty, 1);
    for (int m = 0; m < kMembers; ++m) {
      BarInit(&bars->acc_full[m], 1);
      BarInit(&bars->acc_empty[m], kEpiWarps);
      BarInit(&bars->h1_full[m], kEpiWarps);
    }
    for (int i = 0; i < kFlagRing; ++i) BarInit(&bars->flag_full[i], kProdWarps);
    BarInit(&bars->part_full, 3 * 4);
    BarInit(&bars->part_empty, 4);
    BarInit(&bars->done, 1);
    bars->abort = 0;
    FenceBarrierInit();
  }
  if (tid < 8) {
    bars->site_word[tid] = j.site_word[tid];
    bars->chan[tid] = j.chan[tid];
  }
  if (warp == kMmaWarp) TmemAlloc(&bars->tmem, kCols);
  FenceBeforeSync();
  __syncthreads();
  FenceAfterSync();
  const uint32_t tmem = bars->tmem;
  const long long m_rows = j.m_dev ? min(j.m, static_cast<long long>(*j.m_dev)) : j.m;
  const long long tiles = (m_rows + kRows - 1) / kRows;

  if (warp < kProdWarps) {
    // ---- producer: weights once, then half a row per thread and tile ----
    if (warp == 0 && lane == 0) {
      ArriveExpectTx(&bars->w_full, S::kW1Bytes + kW2Bytes);
      BulkCopy(sw1, d.w1_tiles, S::kW1Bytes, &bars->w_full);
      BulkCopy(sw2, d.w2_tiles, kW2Bytes, &bars->w_full);
    }
    const unsigned bad_all = ProduceRows<kC>(j, m_rows, bars, sx, tiles, warp, lane, abort);
    if (bad_all) atomicOr(j.pair_status, static_cast<int>(bad_all));
    // the weight copies must land before the CTA exits
    if (warp == 0 && lane == 0 && !WaitDrain(&bars->w_full, 0)) *abort = 1;
  } else if (warp == kMmaWarp) {
    // ---- MMA issuer ----
    if (lane == 0) {
      const uint32_t a1 = Smem(sx), b1 = Smem(sw1), b2 = Smem(sw2);
      bool ok = WaitSleep(&bars->w_full, 0, abort);
      int t_local = 0;
      for (long long tile = blockIdx.x; tile < tiles && ok; tile += gridDim.x, ++t_local) {
        if (!(ok = WaitSleep(&bars->x_full, t_local & 1, abort))) break;
        FenceAfterSync();
        // layer 1 of both members, as each member's columns are released
        for (int m = 0; m < kMembers && ok; ++m) {
          if (t_local >= 1 && !(ok = WaitSleep(&bars->acc_empty[m], (t_local - 1) & 1, abort))) break;
          FenceAfterSync();
          IssueLayer1<kC>(tmem, a1, b1, m);
          Commit(&bars->acc_full[m]);
        }
        if (!ok) break;
        Commit(&bars->x_empty);
        // layer 2, A = H1 in TMEM, once the epilogue has written it
        for (int m = 0; m < kMembers && ok; ++m) {
          if (!(ok = WaitSleep(&bars->h1_full[m], t_local & 1, abort))) break;
          FenceAfterSync();
          IssueLayer2(tmem, b2, m);
          Commit(&bars->acc_full[m]);
        }
      }
      // drain: `done` completes once every MMA issued so far has finished
      Commit(&bars->done);
      if (!WaitDrain(&bars->done, 0)) *abort = 1;
    }
    __syncwarp();
  } else {
    // ---- epilogue warps ----
    const int ew = warp - kFirstEpi, q = ew >> 2, lg = warp & 3;
    const int r = lg * 32 + lane;
    const uint32_t lane_base = static_cast<uint32_t>(lg * 32) << 16;
    bool ok = true;
    int t_local = 0;
    for (long long tile = blockIdx.x; tile < tiles && ok; tile += gridDim.x, ++t_local) {
      const long long row = tile * kRows + r;
      bool fallback = false;
      if (q == 0) {
        if (!(ok = WarpWait(&bars->flag_full[t_local % kFlagRing], (t_local / kFlagRing) & 1, abort, lane))) break;
        const uint32_t *fw = bars->flag[t_local % kFlagRing];
        fallback = (((fw[lg] | fw[4 + lg]) >> lane) & 1u) != 0;
      }
      // H1 = GELU(2 D) (D holds layer 1 with b1, halved): this thread's row, its 32 columns,
      // as 16 packed-half columns of the member's H1
      for (int m = 0; m < kMembers && ok; ++m) {
        if (!(ok = WarpWait(&bars->acc_full[m], 0, abort, lane))) break;
        FenceAfterSync();
        Layer1Epilogue(tmem + lane_base + m * kMemberCols, q * 32);
        FenceBeforeSync();
        __syncwarp();
        if (lane == 0) Arrive(&bars->h1_full[m]);
      }
      // y_m = GELU(2 (D + b2 / 2)) . w3 + b3
      float ysum = 0.f, ymin = 3.4e38f, ymax = -3.4e38f;
      for (int m = 0; m < kMembers && ok; ++m) {
        if (!(ok = WarpWait(&bars->acc_full[m], 1, abort, lane))) break;
        FenceAfterSync();
        float v[32];
        TmemLoad32(tmem + lane_base + m * kMemberCols + q * 32, v);
        const float acc = GeluDotHalf(v, d.b2h + m * kHid + q * 32, d.w3h + m * kHid + q * 32);
        FenceBeforeSync();
        __syncwarp();
        if (lane == 0) Arrive(&bars->acc_empty[m]);
        // the four column quarters of a row meet in shared memory
        const int u = 2 * t_local + m;
        if (q != 0) {
          if (u >= 1 && !(ok = WarpWait(&bars->part_empty, (u - 1) & 1, abort, lane))) break;
          bars->partial[q - 1][r] = acc;
          __syncwarp();
          if (lane == 0) Arrive(&bars->part_full);
        } else {
          if (!(ok = WarpWait(&bars->part_full, u & 1, abort, lane))) break;
          const float y = acc + (bars->partial[0][r] + bars->partial[1][r] + bars->partial[2][r]) + __ldg(&d.b3[m]);
          __syncwarp();
          if (lane == 0) Arrive(&bars->part_empty);
          ysum += y;
          ymin = fminf(ymin, y);
          ymax = fmaxf(ymax, y);
        }
      }
      if (ok && q == 0 && row < m_rows) {
        j.mean[row] = mean_label + std_label * ysum * (1.0f / kMembers);
        j.spread[row] = fallback ? __int_as_float(0x7f800000) : std_label * (ymax - ymin);
      }
    }
  }
  __syncthreads();
  if (tid == 0 && bars->abort) atomicOr(status, kMlpFusedTimeout);
  FenceBeforeSync();
  __syncthreads();
  if (warp == kMmaWarp) TmemFree(tmem, kCols);
}

bool MlpFusedSupported(const MlpDev &d) {
  return (d.in == Shape<2>::kIn || d.in == Shape<3>::kIn) && d.hidden == kHid && d.members == kMembers &&
         d.w1_tiles != nullptr && d.w2_tiles != nullptr && d.b2h != nullptr && d.w3h != nullptr;
}

int MlpFusedChannels(const MlpDev &d) {
  if (!MlpFusedSupported(d)) return 0;
  return d.in == Shape<2>::kIn ? 2 : 3;
}

template <int kC>
static cudaError_t LaunchFused(const MlpDev &d, const FusedJumps &j, float mean_label, float std_label, int *status,
                               cudaStream_t s) {
  int dev = 0, sms = 0;
  cudaError_t err = cudaGetDevice(&dev);
  if (err != cudaSuccess) return err;
  err = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (err != cudaSuccess) return err;
  const long long tiles = (j.m + kRows - 1) / kRows;
  const int grid = static_cast<int>(tiles < sms ? tiles : sms);
  constexpr size_t smem = SmemBytes<kC>();
  err = cudaFuncSetAttribute(mlp_fused_jump_kernel<kC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             static_cast<int>(smem));
  if (err != cudaSuccess) return err;
  mlp_fused_jump_kernel<kC><<<grid, kThreads, smem, s>>>(d, j, mean_label, std_label, status);
  return cudaGetLastError();
}

cudaError_t MlpFusedPredict(const MlpDev &d, const FusedJumps &j, float mean_label, float std_label, int *status,
                            cudaStream_t s) {
  const int kc = MlpFusedChannels(d);
  if (kc == 0 || j.channels != kc) return cudaErrorInvalidValue;
  if (j.m <= 0) return cudaSuccess;
  return kc == 2 ? LaunchFused<2>(d, j, mean_label, std_label, status, s)
                 : LaunchFused<3>(d, j, mean_label, std_label, status, s);
}

}  // namespace lmc
