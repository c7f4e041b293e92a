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
// tiles of 128 rows (tcgen05.cuh). Every wait is bounded (sleeping probes, 2 s of wall
// time) and polls a shared abort flag: on expiry the kernel records kMlpFusedTimeout,
// drains its MMAs and copies, frees its TMEM and returns.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "kernels.cuh"
#include "lattice_index.cuh"
#include "mlp.cuh"
#include "tcgen05.cuh"

namespace lmc {
namespace {

using tc::Arrive;
using tc::ArriveExpectTx;
using tc::BarInit;
using tc::BulkCopy;
using tc::Commit;
using tc::FenceAfterSync;
using tc::FenceAsyncSmem;
using tc::FenceBarrierInit;
using tc::FenceBeforeSync;
using tc::IdescBf16;
using tc::Mma;
using tc::MmaTmemA;
using tc::OperandDesc;
using tc::Smem;
using tc::TmemAlloc;
using tc::TmemFree;
using tc::TmemLoad32;
using tc::TmemStore16;
using tc::WaitDrain;
using tc::WaitSleep;

constexpr int kRows = 128;      // jumps per tile (MMA M)
constexpr int kHid = 128;       // hidden width (MMA N of both layers)
constexpr int kMembers = 2;
constexpr int kSites = kEnvSites + 1;       // 58 environment sites and the migrant
constexpr int kTileBytes = kRows * 32 * 2;  // one 128 x 32 operand tile (8 KB)
constexpr int kProdWarps = 8;               // two per row: sites [0, 32) and [32, 64)
constexpr int kHalfSites = 32;
constexpr int kMmaWarp = kProdWarps;
constexpr int kFirstEpi = kProdWarps + 1;
constexpr int kEpiWarps = 16;
constexpr int kThreads = 32 * (kFirstEpi + kEpiWarps);
constexpr uint32_t kCols = 512;
constexpr uint32_t kMemberCols = 192;       // D (128) and H1 (64) of one member
constexpr int kFlagRing = 4;
constexpr uint32_t kIdescL1 = IdescBf16(kRows, kHid);                                    // bf16 x bf16
constexpr uint32_t kIdescL2 = (1u << 4) | ((kHid >> 3) << 17) | ((kRows >> 4) << 24);  // f16 x f16
constexpr int kW2Bytes = kMembers * kHid * kHid * 2;

template <int kC>
struct Shape {
  static constexpr int kIn = (kSites * kC + 63) / 64 * 64;  // 128 (kC = 2) or 192 (kC = 3)
  static constexpr int kKt = kIn / 32;                      // layer-1 K tiles
  static constexpr int kW1Bytes = kMembers * kHid * kIn * 2;
  static constexpr int kXBytes = kRows * kIn * 2;
};

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
static_assert(kSites <= 2 * kHalfSites, "a row is gathered in two halves of 32 sites");
static_assert(2 * kMemberCols <= kCols, "both members' TMEM columns");

// GELU(z) of two values in packed half precision from h = z / 2:
// u = z (c0 + c1 z^2) = h (2 c0 + 8 c1 h^2), GELU = h + h tanh(u).
__device__ __forceinline__ __half2 GeluHalf2FromHalfZ(__half2 h) {
  const __half2 u = __hmul2(h, __hfma2(__hmul2(h, h), __float2half2_rn(8.0f * 0.0356774081363001f),
                                       __float2half2_rn(2.0f * 0.7978845608028654f)));
  uint32_t ub = *reinterpret_cast<const uint32_t *>(&u), tb;
  asm("tanh.approx.f16x2 %0, %1;" : "=r"(tb) : "r"(ub));
  const __half2 t = *reinterpret_cast<const __half2 *>(&tb);
  return __hfma2(h, t, h);
}

// Byte offset of row r, 16-byte chunk c (columns 8c .. 8c + 7) in a sequence of 32-wide operand tiles.
__device__ __forceinline__ uint32_t ChunkOffset(int r, int c) {
  return static_cast<uint32_t>((c >> 2) * kTileBytes + (r >> 3) * 512 + (c & 3) * 128 + (r & 7) * 16);
}

// Bounded wait by lane 0 (sleeping probes), its outcome broadcast to the warp.
__device__ __forceinline__ bool WarpWait(uint64_t *bar, uint32_t parity, volatile int *abort, int lane) {
  int ok = 1;
  if (lane == 0) ok = WaitSleep(bar, parity, abort) ? 1 : 0;
  return __shfl_sync(0xffffffffu, ok, 0) != 0;
}

// Packed half GELU(2 (v + b)) . w over 32 columns (v and b halved), summed in FP32 per 8 columns.
__device__ __forceinline__ float GeluDotHalf(const float *v, const __half *b, const __half *w) {
  float acc = 0.f;
#pragma unroll
  for (int g8 = 0; g8 < 4; ++g8) {
    const uint4 bb = __ldg(reinterpret_cast<const uint4 *>(b + g8 * 8));
    const uint4 ww = __ldg(reinterpret_cast<const uint4 *>(w + g8 * 8));
    const uint32_t bw[4] = {bb.x, bb.y, bb.z, bb.w}, wv[4] = {ww.x, ww.y, ww.z, ww.w};
    __half2 s2 = __float2half2_rn(0.f);
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const __half2 z = __hadd2(__floats2half2_rn(v[g8 * 8 + 2 * e], v[g8 * 8 + 2 * e + 1]),
                                *reinterpret_cast<const __half2 *>(&bw[e]));
      s2 = __hfma2(GeluHalf2FromHalfZ(z), *reinterpret_cast<const __half2 *>(&wv[e]), s2);
    }
    const float2 f = __half22float2(s2);
    acc += f.x + f.y;
  }
  return acc;
}

// Producer of half `half` (warps 0-3: 0, warps 4-7: 1) of every row of the CTA's tiles:
// sites [32 half, 32 half + 32) of the row (MMM-ordered environment, then the migrant; past
// site 58 nothing), i.e. features [kIn / 2 half, kIn / 2 (half + 1)) (feature kC s + c is
// channel c of site s). One code path for both halves keeps the kernel's instruction
// footprint small. Returns the status bits of rejected pairs.
template <int kC>
__device__ __forceinline__ unsigned ProduceRows(const FusedJumps &j, long long m_rows, FusedBars *bars,
                                                unsigned char *sx, long long tiles, int warp, int lane,
                                                volatile int *abort) {
  constexpr int kIn = Shape<kC>::kIn;
  constexpr int kHalfFeat = kIn / 2;
  static_assert(kHalfFeat == kC * kHalfSites, "a half row is 32 sites");
  const int half = warp >> 2;
  const int r = (warp & 3) * 32 + lane;
  const int n = j.n;
  const long long nsites = 4LL * n * n * n;
  unsigned bad_all = 0;
  int t_local = 0;
  for (long long tile = blockIdx.x; tile < tiles; tile += gridDim.x, ++t_local) {
    const long long row = tile * kRows + r;
    int code[kHalfSites];
    bool fallback = true;
    if (row < m_rows) {
      const long long a = __ldg(&j.pairs[2 * row]), b = __ldg(&j.pairs[2 * row + 1]);
      unsigned bad = (a < 0 || b < 0 || a >= nsites || b >= nsites) ? kStatusBadSite : 0u;
      int di = -1;
      H3 hi{0, 0, 0};
      if (!bad) {
        hi = SiteCoord(a, n);
        const H3 hj = SiteCoord(b, n);
        const int dx = WrapDelta(hj.x - hi.x, n), dy = WrapDelta(hj.y - hi.y, n), dz = WrapDelta(hj.z - hi.z, n);
        if (dx >= -1 && dx <= 1 && dy >= -1 && dy <= 1 && dz >= -1 && dz <= 1)
          di = __ldg(&j.dir_of[(dx + 1) * 9 + (dy + 1) * 3 + (dz + 1)]);
        if (di < 0) bad = kStatusNotNeighbor;
      }
      if (half == 0) bad_all |= bad;
      if (!bad) {
        // the offsets of this direction, 4 bytes (dx, dy, dz, 0) per site
        const int *off = reinterpret_cast<const int *>(j.mmm_off) + di * kEnvSites;
#pragma unroll
        for (int k = 0; k < kHalfSites; ++k) {
          const int site = half * kHalfSites + k;
          int c = -1;
          if (site < kEnvSites) {
            const int o = __ldg(off + site);
            c = __ldg(&j.species[NeighborId(hi, static_cast<int8_t>(o), static_cast<int8_t>(o >> 8),
                                            static_cast<int8_t>(o >> 16), n)]);
          } else if (site == kEnvSites) {
            c = __ldg(&j.species[b]);
          }
          code[k] = c;
        }
        unsigned seen = 0;
#pragma unroll
        for (int k = 0; k < kHalfSites; ++k)
          if (half * kHalfSites + k < kSites) seen |= 1u << (code[k] & 7);
        fallback = (seen & j.fallback_codes) != 0;
      }
    }
    if (fallback) {
#pragma unroll
      for (int k = 0; k < kHalfSites; ++k) code[k] = -1;
    }
    // the X buffer is free once the previous tile's layer-1 MMAs have completed
    if (t_local >= 1 && !WarpWait(&bars->x_empty, (t_local - 1) & 1, abort, lane)) break;
#pragma unroll
    for (int c = 0; c < kHalfFeat / 8; ++c) {
      uint32_t w[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int f = 8 * c + 2 * e;  // features f (low half), f + 1 (high half) of this half row
        uint32_t word;
        if constexpr (kC == 2) {
          const int k = f / 2;  // site of features f, f + 1
          word = code[k] >= 0 ? bars->site_word[code[k] & 7] : 0u;
        } else {
          const int k0 = f / kC, k1 = (f + 1) / kC;
          const int ch0 = bars->chan[code[k0] & 7], ch1 = bars->chan[code[k1] & 7];
          word = ((code[k0] >= 0 && ch0 == f % kC) ? 0x3F80u : 0u) |
                 ((code[k1] >= 0 && ch1 == (f + 1) % kC) ? 0x3F800000u : 0u);
        }
        if (f + 1 == kHalfFeat - 1 && half == 1) word |= 0x3F800000u;  // the last feature is 1: the bias column
        w[e] = word;
      }
      *reinterpret_cast<uint4 *>(sx + ChunkOffset(r, half * (kHalfFeat / 8) + c)) =
          make_uint4(w[0], w[1], w[2], w[3]);
    }
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
          const uint32_t dcol = tmem + m * kMemberCols;
          for (int c = 0; c < S::kKt; ++c) {
            const uint32_t a = a1 + c * kTileBytes, b = b1 + (m * S::kKt + c) * kTileBytes;
            Mma(dcol, OperandDesc(a), OperandDesc(b), kIdescL1, c > 0);
            Mma(dcol, OperandDesc(a + 256), OperandDesc(b + 256), kIdescL1, true);
          }
          Commit(&bars->acc_full[m]);
        }
        if (!ok) break;
        Commit(&bars->x_empty);
        // layer 2, A = H1 in TMEM (16 K per MMA = 8 columns), once the epilogue has written it
        for (int m = 0; m < kMembers && ok; ++m) {
          if (!(ok = WaitSleep(&bars->h1_full[m], t_local & 1, abort))) break;
          FenceAfterSync();
          const uint32_t dcol = tmem + m * kMemberCols, hcol = dcol + kHid;
          for (int c = 0; c < kHid / 16; ++c) {
            const uint32_t b = b2 + (m * (kHid / 32) + (c >> 1)) * kTileBytes + (c & 1) * 256;
            MmaTmemA(dcol, hcol + c * 8, OperandDesc(b), kIdescL2, c > 0);
          }
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
        const uint32_t dcol = tmem + lane_base + m * kMemberCols;
        float v[32];
        TmemLoad32(dcol + q * 32, v);
        uint32_t packed[16];
#pragma unroll
        for (int e = 0; e < 16; ++e) {
          const __half2 p = GeluHalf2FromHalfZ(__floats2half2_rn(v[2 * e], v[2 * e + 1]));
          packed[e] = *reinterpret_cast<const uint32_t *>(&p);
        }
        TmemStore16(dcol + kHid + q * 16, packed);
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
