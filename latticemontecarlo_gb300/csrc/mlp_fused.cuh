// Device building blocks of the compact surrogate ensemble on the tensor cores (2 members of
// in -> 128 -> 128 -> 1 GELU over the solute-channel features, in = 128 or 192), shared by the
// fused jump kernel (mlp_fused.cu) and the persistent surrogate-assisted KMC kernel
// (kernels.cu): the operand tile layout, the gather of one half row of features from the
// lattice, the MMAs of both layers and the packed-half epilogue arithmetic.
//
// Weights (MlpCastWeights for this shape): W1 and W2 tiles in the K-major core-matrix layout
// (tcgen05.cuh), member m's W1 K tile c at byte (m * kKt + c) * kTileBytes, W2 likewise with
// 4 K tiles; W1, b1, W2 and b2 are stored halved (exact), so the MMAs produce h = z / 2; the
// last input column of the W1 tiles holds b1 / 2 and the feature row sets that input to 1.
// TMEM: member m owns columns [192 m, 192 m + 192): the accumulator D in the first 128 (layer 1,
// then layer 2), H1 in packed half in the last 64, read by the layer-2 MMA as its A operand.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "kernels.cuh"
#include "lattice_index.cuh"
#include "mlp.cuh"
#include "tcgen05.cuh"

namespace lmc {
namespace fused {

constexpr int kRows = 128;                  // rows per tile (MMA M)
constexpr int kHid = 128;                   // hidden width (MMA N of both layers)
constexpr int kMembers = 2;
constexpr int kSites = kEnvSites + 1;       // 58 environment sites and the migrant
constexpr int kTileBytes = kRows * 32 * 2;  // one 128 x 32 operand tile (8 KB)
constexpr uint32_t kCols = 512;             // TMEM columns allocated
constexpr uint32_t kMemberCols = 192;       // D (128) and H1 (64) of one member
constexpr uint32_t kIdescL1 = tc::IdescBf16(kRows, kHid);                                // bf16 x bf16
constexpr uint32_t kIdescL2 = (1u << 4) | ((kHid >> 3) << 17) | ((kRows >> 4) << 24);  // f16 x f16
constexpr int kW2Bytes = kMembers * kHid * kHid * 2;
static_assert(kSites <= 64, "a row is gathered in parts of 64 sites");
static_assert(2 * kMemberCols <= kCols, "both members' TMEM columns");

template <int kC>
struct Shape {
  static constexpr int kIn = (kSites * kC + 63) / 64 * 64;  // 128 (kC = 2) or 192 (kC = 3)
  static constexpr int kKt = kIn / 32;                      // layer-1 K tiles
  static constexpr int kW1Bytes = kMembers * kHid * kIn * 2;
  static constexpr int kXBytes = kRows * kIn * 2;
};

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

// A lattice site: the read-only data path when the lattice does not change during the kernel,
// a plain (coherent) load in a kernel that moves atoms.
template <bool kReadOnly>
__device__ __forceinline__ int8_t LatticeLoad(const int8_t *p) {
  if constexpr (kReadOnly) return __ldg(p);
  return *p;
}

// Species codes of part `part` of kParts of jump a -> b: sites [S part, S part + S) of the row,
// S = 64 / kParts (MMM-ordered environment, then the migrant at site 58; past it -1). Returns
// whether the row must take the plain predictor (rejected pair, or a species without a one-hot
// slot in its environment); *bad receives the rejected-pair status bits.
template <int kParts, bool kReadOnly = true>
__device__ __forceinline__ bool LoadRowPart(const FusedJumps &j, long long a, long long b, int part,
                                            int (&code)[64 / kParts], unsigned *bad) {
  constexpr int kS = 64 / kParts;
  const int n = j.n;
  const long long nsites = 4LL * n * n * n;
  unsigned st = (a < 0 || b < 0 || a >= nsites || b >= nsites) ? kStatusBadSite : 0u;
  int di = -1;
  H3 hi{0, 0, 0};
  if (!st) {
    hi = SiteCoord(a, n);
    const H3 hj = SiteCoord(b, n);
    const int dx = WrapDelta(hj.x - hi.x, n), dy = WrapDelta(hj.y - hi.y, n), dz = WrapDelta(hj.z - hi.z, n);
    if (dx >= -1 && dx <= 1 && dy >= -1 && dy <= 1 && dz >= -1 && dz <= 1)
      di = __ldg(&j.dir_of[(dx + 1) * 9 + (dy + 1) * 3 + (dz + 1)]);
    if (di < 0) st = kStatusNotNeighbor;
  }
  *bad = st;
  if (st) return true;
  // the offsets of this direction, 4 bytes (dx, dy, dz, 0) per site
  const int *off = reinterpret_cast<const int *>(j.mmm_off) + di * kEnvSites;
#pragma unroll
  for (int k = 0; k < kS; ++k) {
    const int site = part * kS + k;
    int c = -1;
    if (site < kEnvSites) {
      const int o = __ldg(off + site);
      c = LatticeLoad<kReadOnly>(&j.species[NeighborId(hi, static_cast<int8_t>(o), static_cast<int8_t>(o >> 8),
                                                       static_cast<int8_t>(o >> 16), n)]);
    } else if (site == kEnvSites) {
      c = LatticeLoad<kReadOnly>(&j.species[b]);
    }
    code[k] = c;
  }
  unsigned seen = 0;
#pragma unroll
  for (int k = 0; k < kS; ++k)
    if (part * kS + k < kSites) seen |= 1u << (code[k] & 7);
  return (seen & j.fallback_codes) != 0;
}

// Writes part `part` of kParts of feature row r into the operand tiles at sx (code -1: an
// all-zero site; the last feature of the row, in the last part, is 1: the bias column). kC = 2
// takes the per-species row words site_word, kC = 3 the per-species channels chan.
template <int kC, int kParts>
__device__ __forceinline__ void WriteRowPart(const int (&code)[64 / kParts], const uint32_t *site_word,
                                             const int8_t *chan, int part, int r, unsigned char *sx) {
  constexpr int kPartFeat = kC * (64 / kParts);
  static_assert(kPartFeat % 8 == 0 && kPartFeat * kParts == Shape<kC>::kIn, "a part is whole 16-byte chunks");
#pragma unroll
  for (int c = 0; c < kPartFeat / 8; ++c) {
    uint32_t w[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int f = 8 * c + 2 * e;  // features f (low half), f + 1 (high half) of this part
      uint32_t word;
      if constexpr (kC == 2) {
        const int k = f / 2;  // site of features f, f + 1
        word = code[k] >= 0 ? site_word[code[k] & 7] : 0u;
      } else {
        const int k0 = f / kC, k1 = (f + 1) / kC;
        const int ch0 = chan[code[k0] & 7], ch1 = chan[code[k1] & 7];
        word = ((code[k0] >= 0 && ch0 == f % kC) ? 0x3F80u : 0u) |
               ((code[k1] >= 0 && ch1 == (f + 1) % kC) ? 0x3F800000u : 0u);
      }
      if (f + 1 == kPartFeat - 1 && part == kParts - 1) word |= 0x3F800000u;  // bf16 1.0: the bias column
      w[e] = word;
    }
    *reinterpret_cast<uint4 *>(sx + ChunkOffset(r, part * (kPartFeat / 8) + c)) = make_uint4(w[0], w[1], w[2], w[3]);
  }
}

// Layer 1 of member m into its TMEM accumulator (one thread): X (sx) . W1[m]^T (sw1).
template <int kC>
__device__ __forceinline__ void IssueLayer1(uint32_t tmem, uint32_t sx, uint32_t sw1, int m) {
  const uint32_t dcol = tmem + m * kMemberCols;
  for (int c = 0; c < Shape<kC>::kKt; ++c) {
    const uint32_t a = sx + c * kTileBytes, b = sw1 + (m * Shape<kC>::kKt + c) * kTileBytes;
    tc::Mma(dcol, tc::OperandDesc(a), tc::OperandDesc(b), kIdescL1, c > 0);
    tc::Mma(dcol, tc::OperandDesc(a + 256), tc::OperandDesc(b + 256), kIdescL1, true);
  }
}

// Layer 2 of member m (one thread): H1 (TMEM, 16 K per MMA = 8 columns) . W2[m]^T (sw2).
__device__ __forceinline__ void IssueLayer2(uint32_t tmem, uint32_t sw2, int m) {
  const uint32_t dcol = tmem + m * kMemberCols, hcol = dcol + kHid;
  for (int c = 0; c < kHid / 16; ++c) {
    const uint32_t b = sw2 + (m * (kHid / 32) + (c >> 1)) * kTileBytes + (c & 1) * 256;
    tc::MmaTmemA(dcol, hcol + c * 8, tc::OperandDesc(b), kIdescL2, c > 0);
  }
}

// Layer-1 epilogue of 32 columns of one row: H1 = GELU(2 D) as 16 packed-half TMEM columns.
__device__ __forceinline__ void Layer1Epilogue(uint32_t dcol, int col0) {
  float v[32];
  tc::TmemLoad32(dcol + col0, v);
  uint32_t packed[16];
#pragma unroll
  for (int e = 0; e < 16; ++e) {
    const __half2 p = GeluHalf2FromHalfZ(__floats2half2_rn(v[2 * e], v[2 * e + 1]));
    packed[e] = *reinterpret_cast<const uint32_t *>(&p);
  }
  tc::TmemStore16(dcol + kHid + col0 / 2, packed);
}

}  // namespace fused
}  // namespace lmc
