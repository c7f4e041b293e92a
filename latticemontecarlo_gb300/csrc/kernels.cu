// sm_103a kernels of the lattice-MC hot path.
//
//  K1 barrier_batch_kernel   batched Quartic / E0 migration barriers
//                            (VacancyMigrationPredictorQuartic.cpp:112-276, VacancyMigrationPredictorE0.cpp:77-159)
//  K1e encode_batch_kernel   the integer encodings behind K1 (for bit-exact checks)
//  K2 de_pairs_kernel        PairSite swap energy change (EnergyChangePredictorPairSite.cpp:69-192)
//  K3 census_kernel          EnergyPredictor full-lattice census (EnergyPredictor.cpp:40-96)
//  K4 kmc_kernel             persistent batched-replica KMC (KineticMcAbstract.cpp:140-190,
//                            KineticMcFirstOmp.cpp:52-82)
//  K5 cmc_ref_kernel         CanonicalMcOmp batch semantics on the reference's RNG stream
//     cmc_tp_kernel          throughput CMC: cooperative rounds of non-overlapping swaps
//
// All cluster sums are int64 fixed point (weights folded on the host, see
// model.hpp), so they are exact and independent of summation order; FP64 is
// used only for the per-candidate epilogue, the rate sum and the clock.
// Lattice loads inside kernels that also write the lattice use plain
// (coherent) loads, never the read-only path.
#include <cooperative_groups.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <mutex>
#include <type_traits>

#include "kernels.cuh"
#include "fastmath.cuh"
#include "lattice_index.cuh"
#include "mlp_fused.cuh"
#include <cuda_bf16.h>

namespace cg = cooperative_groups;

namespace lmc {
namespace {

constexpr double kBoltzmannEv = 8.617333262145e-5;  // lmc/cfg/include/Constants.hpp:31
constexpr double kPrefactor = 1e13;                 // lmc/cfg/include/Constants.hpp:32
constexpr int kArr = 240;                           // per-warp sorted arrays: 60 + 3 * 58 (+pad)

// Direction index of a half-unit offset via the host-built 27-entry table
// ((dx+1)*9 + (dy+1)*3 + (dz+1) -> index of the 1NN offset, -1 otherwise).
__device__ __forceinline__ int DirIndex(const int8_t *dir_of, int dx, int dy, int dz) {
  if (dx < -1 || dx > 1 || dy < -1 || dy > 1 || dz < -1 || dz > 1) return -1;
  return __ldg(&dir_of[(dx + 1) * 9 + (dy + 1) * 3 + (dz + 1)]);
}

__device__ __forceinline__ long long WarpSum(long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ unsigned long long WarpSumU(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Shared-memory copies of the small model tables.
struct SmallTables {
  int8_t rank[8];
  int8_t slot[8];
  int8_t pairtype[192];
  uint8_t has_quartic[kMaxSlots];
  uint8_t has_e0[kMaxSlots];
  uint8_t pad[4];
};

__device__ __forceinline__ void StageSmall(const DevTables &t, SmallTables *s) {
  for (int i = threadIdx.x; i < 192; i += blockDim.x) s->pairtype[i] = t.pairtype[i];
  if (threadIdx.x < 8) {
    s->rank[threadIdx.x] = t.onehot_rank[threadIdx.x];
    s->slot[threadIdx.x] = t.migrant_slot[threadIdx.x];
  }
  if (threadIdx.x < kMaxSlots) {
    s->has_quartic[threadIdx.x] = t.has_quartic[threadIdx.x];
    s->has_e0[threadIdx.x] = t.has_e0[threadIdx.x];
  }
}

template <typename T>
__device__ __forceinline__ void StageArray(const T *src, T *dst, int n) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = src[i];
}

struct JumpAcc {
  long long de, d, ks;
  unsigned bad;
};

// The energy-change part of EvalJump: state clusters with exactly one pair site, and (first
// site not a vacancy) the clusters holding both pair sites and the two singlets.
__device__ __forceinline__ void AccumulateDe(const DevTables &t, const int8_t *st, const uint32_t *s_de, int lane,
                                             int stride, JumpAcc *acc) {
  JumpAcc &a = *acc;
  const int e = t.num_species;
  const int x = t.x_code;
  const int si = st[t.pos_first];
  const int sj = st[t.pos_second];
  const long long *__restrict__ wde = t.w_de;
  for (int c = lane; c < t.n_de_cl; c += stride) {
    const uint32_t w = s_de[c];
    const int label = w & 7, side = (w >> 3) & 1, o1 = (w >> 4) & 63, o2 = (w >> 10) & 63;
    const int c1 = st[o1];
    const bool has2 = o2 != 63;
    const int c2 = has2 ? st[o2] : 0;
    const int cs = side ? sj : si;
    const int ce = side ? x : sj;
    const int tail = c1 * e + c2;
    const long long ws = __ldg(&wde[(label * e + cs) * e * e + tail]);
    const long long we = __ldg(&wde[(label * e + ce) * e * e + tail]);
    a.de += we - ws;
    const int nx_other = (c1 == x) + (has2 && c2 == x);
    if (nx_other + (cs == x) >= 2 || nx_other + (ce == x) >= 2) a.bad |= kStatusBadCluster;
  }
  if (si != x) {
    // Clusters holding both pair sites and the two singlets keep their
    // multiset (and cancel) only when the first site is the vacancy; for any
    // other first species GetDe counts them (VacancyMigrationPredictorQuartic.cpp:127-154).
    for (int c = lane; c < t.n_de_both; c += stride) {
      const uint32_t w = t.de_both[c];
      const int label = w & 7, kind = (w >> 3) & 3, o = (w >> 5) & 63;
      const int co = o == 63 ? 0 : st[o];
      long long ws, we;
      if (kind == 0) {         // singlet of the first site: s_i -> migrant
        ws = __ldg(&wde[(label * e + si) * e * e]);
        we = __ldg(&wde[(label * e + sj) * e * e]);
      } else if (kind == 1) {  // singlet of the second site: migrant -> X
        ws = __ldg(&wde[(label * e + sj) * e * e]);
        we = __ldg(&wde[(label * e + x) * e * e]);
      } else {                 // {first, second, other}: (s_i, s_j) -> (s_j, X)
        ws = __ldg(&wde[((label * e + si) * e + sj) * e + co]);
        we = __ldg(&wde[((label * e + sj) * e + x) * e + co]);
        const int nx = (si == x) + (sj == x) + (o != 63 && co == x);
        if (nx >= 2 || (sj == x) + (o != 63 && co == x) >= 1) a.bad |= kStatusBadCluster;
      }
      a.de += we - ws;
    }
  }
}

// Per-lane partial sums of one jump's three linear forms from the sorted
// species arrays: st = state list codes (60), rm/rf/rb = MMM / MM2-forward /
// MM2-backward one-hot ranks (58 each, rank 7 = no slot).
//   de: sum over state clusters with exactly one pair site of
//       W(end tuple) - W(start tuple)   (clusters with both pair sites cancel)
//   d : sum over MMM clusters of the D (Quartic) or e0 (E0) weights
//   ks: sum over MM2 clusters of the forward and backward lists (Quartic)
// `lane` and `stride`: this thread's first cluster and the step (a warp: lane, 32; a block:
// thread index, block size).
template <bool kQuartic>
__device__ __forceinline__ JumpAcc EvalJump(const DevTables &t, int slot, const int8_t *st, const int8_t *rm,
                                            const int8_t *rf, const int8_t *rb, const uint32_t *s_de,
                                            const uint32_t *s_mmm, const uint32_t *s_mm2, const int8_t *s_pt,
                                            int lane, int stride = 32) {
  JumpAcc a{0, 0, 0, 0u};
  AccumulateDe(t, st, s_de, lane, stride, &a);
  const long long *__restrict__ wd = (kQuartic ? t.w_d : t.w_e0) + static_cast<long long>(slot) * t.f_mmm;
  for (int c = lane; c < t.n_mmm_cl; c += stride) {
    const uint32_t w = s_mmm[c];
    const int ia = w & 63, ib = (w >> 6) & 63, mode = (w >> 12) & 3, base = w >> 14;
    const int ra = rm[ia];
    const int rbv = ib == 63 ? 0 : rm[ib];
    const int tt = s_pt[(mode * 8 + ra) * 8 + rbv];
    if (tt >= 0) a.d += __ldg(&wd[base + tt]);
    else a.bad |= kStatusXInEnv;
  }
  if (kQuartic) {
    const long long *__restrict__ wk = t.w_ks + static_cast<long long>(slot) * t.f_mm2;
    for (int c = lane; c < t.n_mm2_cl; c += stride) {
      const uint32_t w = s_mm2[c];
      const int ia = w & 63, ib = (w >> 6) & 63, mode = (w >> 12) & 3, base = w >> 14;
      const int fa = rf[ia], ba = rb[ia];
      const int fb = ib == 63 ? 0 : rf[ib];
      const int bb = ib == 63 ? 0 : rb[ib];
      const int tf = s_pt[(mode * 8 + fa) * 8 + fb];
      const int tb = s_pt[(mode * 8 + ba) * 8 + bb];
      if (tf >= 0) a.ks += __ldg(&wk[base + tf]);
      else a.bad |= kStatusXInEnv;
      if (tb >= 0) a.ks += __ldg(&wk[base + tb]);
      else a.bad |= kStatusXInEnv;
    }
  }
  return a;
}

// FP64 epilogue of one jump. With P = Ks * D^2 the reference's closed form
// (VacancyMigrationPredictorQuartic.cpp:269-274) is exactly
//   Ea = (P + 12 dE)^2 (P^2 + 8 P dE - 48 dE^2) / (64 P^3)
// because its sqrt argument 9b^2 - 32ac equals 4 a Ks > 0, i.e. delta = Ks / D.
struct JumpOut {
  double ea, de, d_or_e0, ks;
};
__device__ __forceinline__ JumpOut JumpEpilogue(const DevTables &t, const ExpConsts &ec, int kind, int slot,
                                                long long acc_de, long long acc_d, long long acc_ks) {
  JumpOut o;
  o.de = static_cast<double>(acc_de) * t.de_scale;
  const double *f = t.form + slot * 12;
  // log D (quartic) or log e0 from the MMM sum, log Ks from the MM2 sum
  const double *fa = f + (kind == 0 ? 0 : 8);
  const double log_a = fa[2] * (static_cast<double>(acc_d) * fa[0] - fa[1]) + fa[3];
  const double log_ks = kind == 0 ? f[6] * (static_cast<double>(acc_ks) * f[4] - f[5]) + f[7] : 0.0;
  const double v = ExpFast(kind == 0 ? log_ks + 2.0 * log_a : log_a, ec);
  if (kind == 0) {
    const double p = v;
    const double q = p + 12.0 * o.de;
    o.ea = q * q * (p * p + 8.0 * p * o.de - 48.0 * o.de * o.de) * RcpFast(64.0 * p * p * p);
    o.d_or_e0 = log_a;
    o.ks = log_ks;
  } else {
    o.ea = fmax(0.0, v + o.de / 2);
    o.d_or_e0 = v;
    o.ks = 0.0;
  }
  return o;
}

// Exact-to-rounding int64 -> float on the FP32 / integer pipes: v = hi 2^32 + lo with a signed
// low half (|lo| <= 2^31), so small values convert exactly and large ones within 1.5 ulp.
__device__ __forceinline__ float I64ToFloat(long long v) {
  const int lo = static_cast<int>(static_cast<unsigned>(v));
  const int hi = static_cast<int>((v - lo) >> 32);
  return fmaf(static_cast<float>(hi), 4294967296.0f, static_cast<float>(lo));
}

// FP32 epilogue of one jump for the production streams (barriers within 1e-6 relative of the
// FP64 epilogue): the integer sums are centred exactly (S - C), so only the small deviations
// are rounded, and P = Ks D^2 = P0 exp(a_D (S_D - C_D) + a_Ks (S_Ks - C_Ks)). With x = dE / P
// the closed form above is Ea = P / 64 (1 + 12 x)^2 (1 + 8 x - 48 x^2).
struct JumpOutF {
  float ea, de;
};
__device__ __forceinline__ JumpOutF JumpEpilogueF32(const DevTables &t, int kind, int slot, long long acc_de,
                                                    long long acc_d, long long acc_ks) {
  const float *f = t.form32 + slot * 8;
  const long long *c = t.form32_c + slot * 3;
  JumpOutF o;
  o.de = I64ToFloat(acc_de) * f[7];
  if (kind == 0) {
    const float dev = fmaf(f[0], I64ToFloat(acc_d - c[0]), f[1] * I64ToFloat(acc_ks - c[1]));
    const float p = f[2] * expf(dev);
    const float x = o.de * __frcp_rn(p);
    const float a = fmaf(12.0f, x, 1.0f);
    const float b = fmaf(x, fmaf(-48.0f, x, 8.0f), 1.0f);
    o.ea = p * 0.015625f * a * a * b;
  } else {
    const float e0 = f[4] * expf(f[3] * I64ToFloat(acc_d - c[2]));
    o.ea = fmaxf(0.0f, fmaf(0.5f, o.de, e0));  // VacancyMigrationPredictorE0.cpp:153-159
  }
  return o;
}

// ---------------------------------------------------------------------------
// K1: batched barriers, one warp per pair.
// ---------------------------------------------------------------------------
struct JumpSmem {
  uint32_t *de, *mmm, *mm2;
  SmallTables *small;
  int8_t *arr;
};
__device__ __forceinline__ JumpSmem CarveJumpSmem(const DevTables &t, unsigned char *smem) {
  JumpSmem s;
  s.de = reinterpret_cast<uint32_t *>(smem);
  s.mmm = s.de + t.n_de_cl;
  s.mm2 = s.mmm + t.n_mmm_cl;
  s.small = reinterpret_cast<SmallTables *>(s.mm2 + t.n_mm2_cl);
  s.arr = reinterpret_cast<int8_t *>(s.small + 1);
  return s;
}
__device__ __forceinline__ void StageJump(const DevTables &t, const JumpSmem &s) {
  StageArray(t.de_cl, s.de, t.n_de_cl);
  StageArray(t.mmm_cl, s.mmm, t.n_mmm_cl);
  StageArray(t.mm2_cl, s.mm2, t.n_mm2_cl);
  StageSmall(t, s.small);
}
size_t JumpSmemBytes(const DevTables &t, int warps) {
  size_t b = 4u * (t.n_de_cl + t.n_mmm_cl + t.n_mm2_cl) + sizeof(SmallTables) + static_cast<size_t>(warps) * kArr;
  return (b + 15) & ~size_t(15);
}

// Resolves a (first, second) pair: returns the direction index of second - first
// and of first - second, or a status bit.
__device__ __forceinline__ int ResolvePair(const int8_t *dir_of, long long i, long long j, int n, H3 *hi, H3 *hj,
                                           int *di, int *db) {
  const long long nsites = 4LL * n * n * n;
  if (i < 0 || j < 0 || i >= nsites || j >= nsites) return kStatusBadSite;
  *hi = SiteCoord(i, n);
  *hj = SiteCoord(j, n);
  const int dx = MinImage(hj->x - hi->x, n), dy = MinImage(hj->y - hi->y, n), dz = MinImage(hj->z - hi->z, n);
  *di = DirIndex(dir_of, dx, dy, dz);
  *db = DirIndex(dir_of, -dx, -dy, -dz);
  return *di < 0 ? kStatusNotNeighbor : 0;
}

// Gathers the sorted arrays of jump (hi -> hj) straight from the lattice.
__device__ __forceinline__ void GatherJump(const DevTables &t, const int8_t *species, int n, H3 hi, H3 hj, int di,
                                           int db, const SmallTables *sm, int8_t *st, int8_t *rm, int8_t *rf,
                                           int8_t *rb, int lane) {
  for (int k = lane; k < kStateSites; k += 32) {
    const int8_t *o = t.state_off + (di * kStateSites + k) * 4;
    st[k] = species[NeighborId(hi, o[0], o[1], o[2], n)];
  }
  for (int k = lane; k < kEnvSites; k += 32) {
    const int8_t *a = t.mmm_off + (di * kEnvSites + k) * 4;
    const int8_t *b = t.mm2_off + (di * kEnvSites + k) * 4;
    const int8_t *c = t.mm2_off + (db * kEnvSites + k) * 4;
    rm[k] = sm->rank[species[NeighborId(hi, a[0], a[1], a[2], n)]];
    rf[k] = sm->rank[species[NeighborId(hi, b[0], b[1], b[2], n)]];
    rb[k] = sm->rank[species[NeighborId(hj, c[0], c[1], c[2], n)]];
  }
}

// m_dev (nullable): the number of pairs lives on the device (m is then its upper bound).
// One jump pair by the whole warp over the sorted state / MMM / MM2 lists (the
// dense cluster sums); writes pair p's outputs and returns its status bits.
__device__ __forceinline__ unsigned DensePairBarrier(const DevTables &t, const int8_t *__restrict__ species, int n,
                                                     const long long *__restrict__ pairs, long long p, int kind,
                                                     const uint32_t *s_de, const uint32_t *s_mmm,
                                                     const uint32_t *s_mm2, const SmallTables *small, int8_t *st,
                                                     int8_t *rm, int8_t *rf, int8_t *rb, double *ea, double *de,
                                                     double *d_or_e0, double *ks, int lane) {
  H3 hi, hj;
  int di = -1, db = -1;
  unsigned bad = ResolvePair(t.dir_of, pairs[2 * p], pairs[2 * p + 1], n, &hi, &hj, &di, &db);
  int slot = -1;
  if (!bad) {
    GatherJump(t, species, n, hi, hj, di, db, small, st, rm, rf, rb, lane);
    __syncwarp();
    slot = small->slot[st[t.pos_second]];
    if (slot < 0 || (kind == 0 ? !small->has_quartic[slot] : !small->has_e0[slot])) bad = kStatusNoCoefficients;
  }
  if (bad) {
    if (lane == 0) {
      ea[p] = nan("");
      de[p] = nan("");
    }
    __syncwarp();
    return bad;
  }
  JumpAcc a = kind == 0 ? EvalJump<true>(t, slot, st, rm, rf, rb, s_de, s_mmm, s_mm2, small->pairtype, lane)
                        : EvalJump<false>(t, slot, st, rm, rf, rb, s_de, s_mmm, s_mm2, small->pairtype, lane);
  const long long acc_de = WarpSum(a.de), acc_d = WarpSum(a.d), acc_ks = WarpSum(a.ks);
  unsigned b = __reduce_or_sync(0xffffffffu, a.bad);
  if (lane == 0) {
    const JumpOut o = JumpEpilogue(t, ExpConsts{t.exp_tab, t.exp_l1, t.exp_l2}, kind, slot, acc_de, acc_d, acc_ks);
    ea[p] = o.ea;
    de[p] = o.de;
    if (d_or_e0) d_or_e0[p] = kind == 0 ? exp(o.d_or_e0) : o.d_or_e0;
    if (ks) ks[p] = kind == 0 ? exp(o.ks) : 0.0;
    if (!isfinite(o.ea)) b |= kStatusNumeric;
  }
  __syncwarp();
  return b;
}

__global__ void barrier_batch_kernel(DevTables t, const int8_t *__restrict__ species, int n,
                                     const long long *__restrict__ pairs, int m, const int *m_dev, int kind,
                                     double *ea, double *de, double *d_or_e0, double *ks, int *status) {
  extern __shared__ __align__(16) unsigned char smem[];
  if (m_dev) m = min(m, *m_dev);
  const JumpSmem s = CarveJumpSmem(t, smem);
  StageJump(t, s);
  __syncthreads();
  const int warps = blockDim.x >> 5;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int8_t *st = s.arr + warp * kArr;
  int8_t *rm = st + kStateSites, *rf = rm + kEnvSites, *rb = rf + kEnvSites;
  unsigned bad_all = 0;
  for (int p = blockIdx.x * warps + warp; p < m; p += gridDim.x * warps)
    bad_all |= DensePairBarrier(t, species, n, pairs, p, kind, s.de, s.mmm, s.mm2, s.small, st, rm, rf, rb, ea, de,
                                d_or_e0, ks, lane);
  if (bad_all && lane == 0) atomicOr(status, static_cast<int>(bad_all));
}

// ---------------------------------------------------------------------------
// K1e: integer encodings (ElementCluster start/end counts, one-hot numerators).
// ---------------------------------------------------------------------------
__global__ void encode_batch_kernel(DevTables t, const int8_t *__restrict__ species, int n,
                                    const long long *__restrict__ pairs, int m, int *state_start, int *state_end,
                                    int *mmm, int *mm2f, int *mm2b, int *status) {
  extern __shared__ __align__(16) unsigned char smem[];
  const JumpSmem s = CarveJumpSmem(t, smem);
  StageJump(t, s);
  __syncthreads();
  const int warps = blockDim.x >> 5;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int8_t *st = s.arr + warp * kArr;
  int8_t *rm = st + kStateSites, *rf = rm + kEnvSites, *rb = rf + kEnvSites;
  const int e = t.num_species;
  for (int p = blockIdx.x * warps + warp; p < m; p += gridDim.x * warps) {
    H3 hi, hj;
    int di = -1, db = -1;
    unsigned bad = ResolvePair(t.dir_of, pairs[2 * p], pairs[2 * p + 1], n, &hi, &hj, &di, &db);
    if (bad) {
      if (lane == 0) atomicOr(status, static_cast<int>(bad));
      continue;
    }
    GatherJump(t, species, n, hi, hj, di, db, s.small, st, rm, rf, rb, lane);
    __syncwarp();
    const int sj = st[t.pos_second];
    int *cs = state_start + static_cast<long long>(p) * t.num_theta;
    int *ce = state_end + static_cast<long long>(p) * t.num_theta;
    for (int c = lane; c < t.n_state_all; c += 32) {
      const uint32_t w = t.state_all[c];
      const int label = w & 7, size = (w >> 3) & 3;
      int k[3] = {static_cast<int>((w >> 5) & 63), static_cast<int>((w >> 11) & 63), static_cast<int>((w >> 17) & 63)};
      int a[3] = {0, 0, 0}, b[3] = {0, 0, 0};
      for (int q = 0; q < size; ++q) {
        a[q] = st[k[q]];
        b[q] = k[q] == t.pos_first ? sj : (k[q] == t.pos_second ? t.x_code : a[q]);
      }
      const int ia = t.cluster_index[((label * e + a[0]) * e + a[1]) * e + a[2]];
      const int ib = t.cluster_index[((label * e + b[0]) * e + b[1]) * e + b[2]];
      if (ia < 0 || ib < 0) {
        atomicOr(status, kStatusBadCluster);
        continue;
      }
      atomicAdd(&cs[ia], 1);
      atomicAdd(&ce[ib], 1);
    }
    int *om = mmm + static_cast<long long>(p) * t.f_mmm;
    for (int c = lane; c < t.n_mmm_cl; c += 32) {
      const uint32_t w = s.mmm[c];
      const int ia = w & 63, ib = (w >> 6) & 63, mode = (w >> 12) & 3, base = w >> 14;
      const int tt = s.small->pairtype[(mode * 8 + rm[ia]) * 8 + (ib == 63 ? 0 : rm[ib])];
      if (tt >= 0) atomicAdd(&om[base + tt], 1);
      else atomicOr(status, kStatusXInEnv);
    }
    int *of = mm2f + static_cast<long long>(p) * t.f_mm2;
    int *ob = mm2b + static_cast<long long>(p) * t.f_mm2;
    for (int c = lane; c < t.n_mm2_cl; c += 32) {
      const uint32_t w = s.mm2[c];
      const int ia = w & 63, ib = (w >> 6) & 63, mode = (w >> 12) & 3, base = w >> 14;
      const int tf = s.small->pairtype[(mode * 8 + rf[ia]) * 8 + (ib == 63 ? 0 : rf[ib])];
      const int tb = s.small->pairtype[(mode * 8 + rb[ia]) * 8 + (ib == 63 ? 0 : rb[ib])];
      if (tf >= 0) atomicAdd(&of[base + tf], 1);
      else atomicOr(status, kStatusXInEnv);
      if (tb >= 0) atomicAdd(&ob[base + tb], 1);
      else atomicOr(status, kStatusXInEnv);
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------
// K2: PairSite energy change of swapping the species of two sites.
//   dE = sum over clusters c of site(a) with b not in c of W(c; a -> s_b) - W(c)
//      + sum over clusters c of site(b) with a not in c of W(c; b -> s_a) - W(c)
// which equals both the uncoupled (two site terms) and the coupled (pair
// mapping, GetClusterParametersMappingStatePairOf) branches of the reference:
// clusters containing both sites keep their multiset and cancel.
// ---------------------------------------------------------------------------
struct SiteSmem {
  uint32_t *cl;
  int8_t *off;   // [43][4]
  int8_t *arr;   // per warp 2 x 44
};
__device__ __forceinline__ SiteSmem CarveSiteSmem(const DevTables &t, unsigned char *smem) {
  SiteSmem s;
  s.cl = reinterpret_cast<uint32_t *>(smem);
  s.off = reinterpret_cast<int8_t *>(s.cl + t.n_site_cl);
  s.arr = s.off + kSiteSites * 4;
  return s;
}
size_t SiteSmemBytes(const DevTables &t, int warps) {
  size_t b = 4u * t.n_site_cl + kSiteSites * 4 + static_cast<size_t>(warps) * 88;
  return (b + 15) & ~size_t(15);
}

// Partial (per-lane) fixed-point dE of swapping the species at the centres of
// the site arrays sa / sb. pa / pb: index of the other centre in each list or -1.
__device__ __forceinline__ long long SwapDePartial(const DevTables &t, const uint32_t *cl, const int8_t *sa,
                                                   const int8_t *sb, int pa, int pb, int lane) {
  const int e = t.num_species;
  const int ca = sa[t.site_center], cb = sb[t.site_center];
  const long long *__restrict__ w = t.w_de;
  long long acc = 0;
  for (int c = lane; c < t.n_site_cl; c += 32) {
    const uint32_t d = cl[c];
    const int label = d & 7, o1 = (d >> 3) & 63, o2 = (d >> 9) & 63;
    const int base = label * e;
    if (o1 != pb && o2 != pb) {
      const int tail = (o1 == 63 ? 0 : sa[o1]) * e + (o2 == 63 ? 0 : sa[o2]);
      acc += __ldg(&w[(base + cb) * e * e + tail]) - __ldg(&w[(base + ca) * e * e + tail]);
    }
    if (o1 != pa && o2 != pa) {
      const int tail = (o1 == 63 ? 0 : sb[o1]) * e + (o2 == 63 ? 0 : sb[o2]);
      acc += __ldg(&w[(base + ca) * e * e + tail]) - __ldg(&w[(base + cb) * e * e + tail]);
    }
  }
  return acc;
}

// Gathers the 43-site lists of a and b and locates each centre in the other list.
__device__ __forceinline__ void GatherSwap(const int8_t *off, const int8_t *species, int n, H3 ha, H3 hb,
                                           int8_t *sa, int8_t *sb, int *pa, int *pb, int lane) {
  const int dx = MinImage(hb.x - ha.x, n), dy = MinImage(hb.y - ha.y, n), dz = MinImage(hb.z - ha.z, n);
  int found_b = -1, found_a = -1;
  for (int k = lane; k < kSiteSites; k += 32) {
    const int8_t *o = off + k * 4;
    sa[k] = species[NeighborId(ha, o[0], o[1], o[2], n)];
    sb[k] = species[NeighborId(hb, o[0], o[1], o[2], n)];
    if (o[0] == dx && o[1] == dy && o[2] == dz) found_b = k;
    if (o[0] == -dx && o[1] == -dy && o[2] == -dz) found_a = k;
  }
  *pb = __reduce_max_sync(0xffffffffu, found_b);
  *pa = __reduce_max_sync(0xffffffffu, found_a);
  __syncwarp();
}

// Single-site substitution dE (EnergyChangePredictorPairSite::GetDeFromLatticeIdSite,
// EnergyChangePredictorPairSite.cpp:154-192), one warp per query: the species at `site`
// taken as from[q] (the lattice's own when from is null) and replaced by to[q]; the
// lattice read with `fill_site` (if >= 0) holding fill_code. Folded int64 weights over
// the site's clusters: sum W(c; centre -> to) - W(c; centre = from).
__global__ void site_de_kernel(DevTables t, const int8_t *__restrict__ species, int n,
                               const long long *__restrict__ sites, const int8_t *__restrict__ from,
                               const int8_t *__restrict__ to, long long m, long long fill_site, int fill_code,
                               double *de) {
  extern __shared__ __align__(16) unsigned char smem[];
  const SiteSmem s = CarveSiteSmem(t, smem);
  StageArray(t.site_cl, s.cl, t.n_site_cl);
  StageArray(t.site_off, s.off, kSiteSites * 4);
  __syncthreads();
  const int warps = blockDim.x >> 5;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int8_t *sa = s.arr + warp * 88;
  const int e = t.num_species;
  for (long long q = static_cast<long long>(blockIdx.x) * warps + warp; q < m;
       q += static_cast<long long>(gridDim.x) * warps) {
    const long long site = sites[q];
    const H3 h = SiteCoord(site, n);
    for (int k = lane; k < kSiteSites; k += 32) {
      const int8_t *o = s.off + k * 4;
      const long long id = NeighborId(h, o[0], o[1], o[2], n);
      sa[k] = id == fill_site ? static_cast<int8_t>(fill_code) : species[id];
    }
    __syncwarp();
    const int ca = from ? from[q] : sa[t.site_center], cb = to[q];
    long long acc = 0;
    if (ca != cb) {
      const long long *__restrict__ w = t.w_de;
      for (int c = lane; c < t.n_site_cl; c += 32) {
        const uint32_t d = s.cl[c];
        const int label = d & 7, o1 = (d >> 3) & 63, o2 = (d >> 9) & 63;
        const int tail = (o1 == 63 ? 0 : sa[o1]) * e + (o2 == 63 ? 0 : sa[o2]);
        acc += __ldg(&w[(label * e + cb) * e * e + tail]) - __ldg(&w[(label * e + ca) * e * e + tail]);
      }
    }
    acc = WarpSum(acc);
    if (lane == 0) de[q] = static_cast<double>(acc) * t.de_scale;
    __syncwarp();
  }
}

// ExitTime::GetBindingEnergy and GetProfileEnergy (ExitTime.cpp:401-511) for every site, one warp
// per site: the neighbourhood gathered once (the vacancy `vac`, if >= 0, read as the solvent), then in
// one pass over the site's clusters the substitution sums of every element e -> X; binding[k][i] =
// dE(e_k -> X) - (mu_X - mu_e_k) over the non-X codes e_k in ascending order, profile[i] = dE(own ->
// X) + mu_own - mu_X, and at the vacancy the largest dE(e -> X) + mu_e - mu_X.
constexpr int kExitMaxElements = 5;
__global__ void exit_energy_kernel(DevTables t, const int8_t *__restrict__ species, int n, long long vac, int solvent,
                                   const double *__restrict__ mu, double *binding, double *profile) {
  extern __shared__ __align__(16) unsigned char smem[];
  const SiteSmem s = CarveSiteSmem(t, smem);
  StageArray(t.site_cl, s.cl, t.n_site_cl);
  StageArray(t.site_off, s.off, kSiteSites * 4);
  __syncthreads();
  const int warps = blockDim.x >> 5;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int8_t *sa = s.arr + warp * 88;
  const int e = t.num_species, x = t.x_code;
  const long long nsites = 4LL * n * n * n;
  for (long long site = static_cast<long long>(blockIdx.x) * warps + warp; site < nsites;
       site += static_cast<long long>(gridDim.x) * warps) {
    const H3 h = SiteCoord(site, n);
    for (int k = lane; k < kSiteSites; k += 32) {
      const int8_t *o = s.off + k * 4;
      const long long id = NeighborId(h, o[0], o[1], o[2], n);
      sa[k] = id == vac ? static_cast<int8_t>(solvent) : species[id];
    }
    __syncwarp();
    long long acc[kExitMaxElements] = {0, 0, 0, 0, 0};  // indexed by the element's rank among non-X codes
    const long long *__restrict__ w = t.w_de;
    for (int c = lane; c < t.n_site_cl; c += 32) {
      const uint32_t d = s.cl[c];
      const int label = d & 7, o1 = (d >> 3) & 63, o2 = (d >> 9) & 63;
      const int tail = (o1 == 63 ? 0 : sa[o1]) * e + (o2 == 63 ? 0 : sa[o2]);
      const long long wx = __ldg(&w[(label * e + x) * e * e + tail]);
#pragma unroll
      for (int k = 0; k < kExitMaxElements; ++k) {
        const int code = k < x ? k : k + 1;
        if (code < e) acc[k] += wx - __ldg(&w[(label * e + code) * e * e + tail]);
      }
    }
    double best = -1e300;
    const int own = sa[t.site_center];
#pragma unroll
    for (int k = 0; k < kExitMaxElements; ++k) {
      const int code = k < x ? k : k + 1;
      if (code >= e) continue;
      const double de = static_cast<double>(WarpSum(acc[k])) * t.de_scale;
      if (lane == 0) binding[k * nsites + site] = de - (mu[x] - mu[code]);
      best = fmax(best, de + mu[code] - mu[x]);
      if (code == own && lane == 0 && site != vac) profile[site] = de + mu[code] - mu[x];
    }
    if (lane == 0 && site != vac && own == x) profile[site] = 0.0;  // another vacancy: X -> X
    if (lane == 0 && site == vac) profile[site] = best;
    __syncwarp();
  }
}

__global__ void de_pairs_kernel(DevTables t, const int8_t *__restrict__ species, int n,
                                const long long *__restrict__ pairs, int m, double *de, int *status) {
  extern __shared__ __align__(16) unsigned char smem[];
  const SiteSmem s = CarveSiteSmem(t, smem);
  StageArray(t.site_cl, s.cl, t.n_site_cl);
  StageArray(t.site_off, s.off, kSiteSites * 4);
  __syncthreads();
  const int warps = blockDim.x >> 5;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int8_t *sa = s.arr + warp * 88, *sb = sa + 44;
  const long long nsites = 4LL * n * n * n;
  for (int p = blockIdx.x * warps + warp; p < m; p += gridDim.x * warps) {
    const long long a = pairs[2 * p], b = pairs[2 * p + 1];
    if (a < 0 || b < 0 || a >= nsites || b >= nsites) {
      if (lane == 0) {
        de[p] = nan("");
        atomicOr(status, kStatusBadSite);
      }
      continue;
    }
    if (species[a] == species[b]) {
      if (lane == 0) de[p] = 0.0;
      continue;
    }
    int pa, pb;
    GatherSwap(s.off, species, n, SiteCoord(a, n), SiteCoord(b, n), sa, sb, &pa, &pb, lane);
    const long long acc = WarpSum(SwapDePartial(t, s.cl, sa, sb, pa, pb, lane));
    if (lane == 0) de[p] = static_cast<double>(acc) * t.de_scale;
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------
// K3: full-lattice cluster census. One thread per site, shared-memory
// histogram; clusters made only of the dominant species are counted in
// registers per label and merged once per warp (they are most of the lattice).
// ---------------------------------------------------------------------------
// kCheckCodes: the species array comes straight from the caller (lmc_energy_noalloc) rather than
// from a context lattice validated at upload, so every code is range-checked before it indexes
// the shared tables; a site whose 43-site neighbourhood holds a code outside [0, e) is skipped
// and counted in *bad_codes.
constexpr int kCensusThreads = 256;
template <bool kCheckCodes>
__global__ void __launch_bounds__(kCensusThreads) census_kernel(DevTables t, const int8_t *__restrict__ species, int n,
                                                                int base_code, unsigned long long *counts,
                                                                unsigned long long *bad_codes) {
  __shared__ unsigned int hist[512];
  __shared__ uint32_t s_tri[160];
  __shared__ int8_t s_off[kSiteSites * 4];
  __shared__ int8_t s_label[kSiteSites];
  __shared__ int16_t s_idx[8 * 6 * 6 * 6];
  __shared__ int8_t s_sp[kCensusThreads * 44];
  const int e = t.num_species;
  for (int i = threadIdx.x; i < 512; i += blockDim.x) hist[i] = 0;
  StageArray(t.census_tri, s_tri, t.n_census_tri);
  StageArray(t.site_off, s_off, kSiteSites * 4);
  StageArray(t.cluster_index, s_idx, 8 * e * e * e);
  __syncthreads();
  for (int k = threadIdx.x; k < kSiteSites; k += blockDim.x) {
    const int x = s_off[k * 4], y = s_off[k * 4 + 1], z = s_off[k * 4 + 2];
    const int n2 = x * x + y * y + z * z;
    s_label[k] = n2 == 2 ? 1 : (n2 == 4 ? 2 : (n2 == 6 ? 3 : 0));
  }
  __syncthreads();
  const long long nsites = 4LL * n * n * n;
  int8_t *sp = s_sp + threadIdx.x * 44;
  unsigned base_count[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (long long site = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; site < nsites;
       site += static_cast<long long>(gridDim.x) * blockDim.x) {
    const H3 h = SiteCoord(site, n);
    bool all_base = true;
    for (int k = 0; k < kSiteSites; ++k) {
      const int8_t v = species[NeighborId(h, s_off[k * 4], s_off[k * 4 + 1], s_off[k * 4 + 2], n)];
      sp[k] = v;
      all_base &= v == base_code;
    }
    const int c0 = sp[t.site_center];
    if (all_base) {
      base_count[0] += 1;
      base_count[1] += 12;
      base_count[2] += 6;
      base_count[3] += 24;
      for (int q = 0; q < t.n_census_tri; ++q) base_count[s_tri[q] & 7] += 1;
      continue;
    }
    if constexpr (kCheckCodes) {
      bool ok = true;
      for (int k = 0; k < kSiteSites; ++k) ok &= static_cast<unsigned>(static_cast<int>(sp[k])) < static_cast<unsigned>(e);
      if (!ok) {
        atomicAdd(bad_codes, 1ull);
        continue;
      }
    }
    // clusters whose multiset has no index (two or more vacancies) count nothing
    atomicAdd(&hist[s_idx[(0 * e + c0) * e * e]], 1u);
    for (int k = 0; k < kSiteSites; ++k) {
      const int l = s_label[k];
      if (l == 0) continue;
      const int c1 = sp[k];
      if (c0 == base_code && c1 == base_code) {
        base_count[l] += 1;
      } else {
        const int idx = s_idx[((l * e + c0) * e + c1) * e];
        if (idx >= 0) atomicAdd(&hist[idx], 1u);
      }
    }
    for (int q = 0; q < t.n_census_tri; ++q) {
      const uint32_t w = s_tri[q];
      const int l = w & 7;
      const int c1 = sp[(w >> 3) & 63], c2 = sp[(w >> 9) & 63];
      if (c0 == base_code && c1 == base_code && c2 == base_code) {
        base_count[l] += 1;
      } else {
        const int idx = s_idx[((l * e + c0) * e + c1) * e + c2];
        if (idx >= 0) atomicAdd(&hist[idx], 1u);
      }
    }
  }
  // merge the per-label dominant-species counts
  for (int l = 0; l < 8; ++l) {
    unsigned v = base_count[l];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0 && v) {
      const int idx = l == 0 ? s_idx[(0 * e + base_code) * e * e]
                             : (l <= 3 ? s_idx[((l * e + base_code) * e + base_code) * e]
                                       : s_idx[((l * e + base_code) * e + base_code) * e + base_code]);
      atomicAdd(&hist[idx], v);
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < t.num_theta; i += blockDim.x)
    if (hist[i]) atomicAdd(&counts[i], static_cast<unsigned long long>(hist[i]));
}

// Energy = sum_idx theta_idx * (count_idx / bonds_idx), sequential in index
// order without contraction, as the reference's GetEncode + dot
// (EnergyPredictor.cpp:87-95,173-177).
// With bad_codes set, a nonzero count of skipped sites gives NaN instead of an energy.
__global__ void census_energy_kernel(DevTables t, const unsigned long long *counts, double *energy,
                                     const unsigned long long *bad_codes) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  if (bad_codes != nullptr && *bad_codes != 0) {
    *energy = nan("");
    return;
  }
  double s = 0.0;
  for (int i = 0; i < t.num_theta; ++i) {
    const double enc = __ddiv_rn(static_cast<double>(counts[i]), t.census_bonds[i]);
    s = __dadd_rn(s, __dmul_rn(t.theta[i], enc));
  }
  *energy = s;
}

// ---------------------------------------------------------------------------
// Random numbers.
//  * std::mt19937_64 with libstdc++'s generate_canonical<double, 53> and
//    uniform_int_distribution (Lemire's multiply-and-reject, Lemire 2019),
//    so device draws equal the reference's for the same seed.
//  * Philox4x32-10 (Salmon et al., SC'11) for production streams.
// ---------------------------------------------------------------------------
struct Mt {
  unsigned long long *mt;  // 312 words
  unsigned *idx;
};
// mt19937_64's output tempering.
__device__ __forceinline__ unsigned long long MtTemperOut(unsigned long long y) {
  y ^= (y >> 29) & 0x5555555555555555ULL;
  y ^= (y << 17) & 0x71D67FFFEDA60000ULL;
  y ^= (y << 37) & 0xFFF7EEE000000000ULL;
  return y ^ (y >> 43);
}
__device__ __forceinline__ unsigned long long MtNext(Mt s) {
  constexpr int kN = 312, kM = 156;
  constexpr unsigned long long kUpper = 0xFFFFFFFF80000000ULL, kLower = 0x7FFFFFFFULL;
  constexpr unsigned long long kA = 0xB5026F5AA96619E9ULL;
  unsigned i = *s.idx;
  if (i >= kN) {
    for (int k = 0; k < kN; ++k) {
      const unsigned long long x = (s.mt[k] & kUpper) | (s.mt[(k + 1) % kN] & kLower);
      s.mt[k] = s.mt[(k + kM) % kN] ^ (x >> 1) ^ ((x & 1ULL) ? kA : 0ULL);
    }
    i = 0;
  }
  const unsigned long long y = s.mt[i];
  *s.idx = i + 1;
  return MtTemperOut(y);
}
// generate_canonical<double, 53>(mt19937_64): one draw scaled by 2^-64, values
// that round up to 1 become the largest double below 1.
__device__ __forceinline__ double MtCanonical(unsigned long long x) {
  const double u = __ull2double_rn(x) * 5.421010862427522170e-20;  // 2^-64
  return u >= 1.0 ? 0.99999999999999988898 : u;
}
__device__ __forceinline__ double MtUniform(Mt s) { return MtCanonical(MtNext(s)); }
// MtNext's in-place twist of the 312 state words, by a whole warp, 32 words at a time:
// every lane reads its word's three inputs before any lane of the chunk writes. Word k reads
// words k + 1 and k + 156 (mod 312); the serial loop sees the new values of the words below k
// and the old ones above, and so does this order: a chunk's inputs below it were written by
// earlier chunks, those above it (and inside it, read before the writes) are still old.
__device__ __forceinline__ void MtTwistInPlaceWarp(unsigned long long *mt, int lane) {
  constexpr unsigned long long kUpper = 0xFFFFFFFF80000000ULL, kLower = 0x7FFFFFFFULL;
  constexpr unsigned long long kA = 0xB5026F5AA96619E9ULL;
  for (int b = 0; b < 312; b += 32) {
    const int k = b + lane;
    unsigned long long v = 0;
    if (k < 312) {
      const unsigned long long x = (mt[k] & kUpper) | (mt[k + 1 < 312 ? k + 1 : 0] & kLower);
      v = mt[k + 156 < 312 ? k + 156 : k - 156] ^ (x >> 1) ^ ((x & 1ULL) ? kA : 0ULL);
    }
    __syncwarp();
    if (k < 312) mt[k] = v;
    __syncwarp();
  }
}

struct Philox {
  uint32_t c[4], k[2];
};
__device__ __forceinline__ uint4 PhiloxRound10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0,
                                               uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint32_t hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
    const uint32_t hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
    const uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return make_uint4(c0, c1, c2, c3);
}
// 53-bit uniform in [0, 1) from two 32-bit words; the (0, 1] variant adds one ulp.
__device__ __forceinline__ double U01(uint32_t hi, uint32_t lo) {
  const unsigned long long v = ((static_cast<unsigned long long>(hi) << 32) | lo) >> 11;
  return static_cast<double>(v) * 1.1102230246251565404e-16;  // 2^-53
}
__device__ __forceinline__ double U01Open(uint32_t hi, uint32_t lo) {
  const unsigned long long v = ((static_cast<unsigned long long>(hi) << 32) | lo) >> 11;
  return static_cast<double>(v + 1) * 1.1102230246251565404e-16;
}

// ---------------------------------------------------------------------------
// K6: surrogate training data and features.
//
// Features of a jump (MLP input, bf16 row of in_pad values): for each of the 58
// MMM-ordered environment sites, then the migrant, `width` channels, one of which
// is 1 (FeatEnc: the one-hot rank, or a solute channel with the base species as
// the all-zero site); zero padded.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void WriteFeatures(const int8_t *rm, int mig_rank, const FeatEnc &f, int in_pad,
                                              __nv_bfloat16 *row, int lane) {
  const int w = f.width, env = kEnvSites * w;
  for (int idx = lane; idx < in_pad; idx += 32) {
    bool one = false;
    if (idx < env) one = FeatChannel(f, rm[idx / w]) == idx % w;
    else if (idx < env + w) one = FeatChannel(f, mig_rank) == idx - env;
    row[idx] = __float2bfloat16(one ? 1.0f : 0.0f);
  }
}

// One warp per sample: a 135-site neighbourhood drawn with Philox (counter =
// (sample, lane, round), key = seed): the centre is the vacancy, every other
// site a solute with probability f ~ U(solute_lo, solute_hi) (solutes equally
// likely) and the base species otherwise; jump direction = sample mod 12. The
// label is the plain predictor's barrier (dense cluster sums + FP64 epilogue).
__global__ void surrogate_dataset_kernel(DevTables t, SurrogateGen g) {
  extern __shared__ __align__(16) unsigned char smem[];
  const JumpSmem s = CarveJumpSmem(t, smem);
  StageJump(t, s);
  const int warps = blockDim.x >> 5;
  int8_t *locals = reinterpret_cast<int8_t *>(s.arr + warps * kArr);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int8_t *st = s.arr + warp * kArr;
  int8_t *rm = st + kStateSites, *rf = rm + kEnvSites, *rb = rf + kEnvSites;
  int8_t *local = locals + warp * 144;
  const int e = t.num_species;
  // solutes: every non-vacancy species other than the base
  int solutes[8], ns = 0;
  for (int c = 0; c < e; ++c)
    if (c != t.x_code && c != g.base_code) solutes[ns++] = c;
  unsigned bad_all = 0;
  for (long long i = static_cast<long long>(blockIdx.x) * warps + warp; i < g.count;
       i += static_cast<long long>(gridDim.x) * warps) {
    const uint32_t k0 = static_cast<uint32_t>(g.seed), k1 = static_cast<uint32_t>(g.seed >> 32);
    const uint4 head = PhiloxRound10(static_cast<uint32_t>(i), static_cast<uint32_t>(i >> 32), 0xFFFFu, 0x53u, k0, k1);
    const float f = g.solute_lo + (g.solute_hi - g.solute_lo) * (head.x * 2.3283064365386963e-10f);
    const int c = static_cast<int>(i % 12);
    for (int r = 0; r < 2; ++r) {
      const uint4 x = PhiloxRound10(static_cast<uint32_t>(i), static_cast<uint32_t>(i >> 32), lane, r, k0, k1);
      const uint32_t v[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int site = lane + 32 * (4 * r + q);
        if (site >= kLocalSites) continue;
        const float u = (v[q] >> 8) * 5.9604644775390625e-8f;  // 24-bit uniform
        int code = g.base_code;
        if (u < f && ns > 0) code = solutes[min(ns - 1, static_cast<int>(u / f * ns))];
        local[site] = static_cast<int8_t>(code);
      }
    }
    __syncwarp();
    const uint8_t *lst = t.local_st + c * kStateSites;
    if (lane == 0) local[lst[t.pos_first]] = static_cast<int8_t>(t.x_code);
    __syncwarp();
    for (int k = lane; k < kStateSites; k += 32) st[k] = local[lst[k]];
    for (int k = lane; k < kEnvSites; k += 32) {
      rm[k] = s.small->rank[local[t.local_mmm[c * kEnvSites + k]]];
      rf[k] = s.small->rank[local[t.local_mm2f[c * kEnvSites + k]]];
      rb[k] = s.small->rank[local[t.local_mm2b[c * kEnvSites + k]]];
    }
    __syncwarp();
    const int mig = st[t.pos_second];
    const int slot = s.small->slot[mig];
    const bool ok = slot >= 0 && (g.kind == 0 ? s.small->has_quartic[slot] : s.small->has_e0[slot]);
    JumpAcc a{0, 0, 0, 0u};
    if (ok)
      a = g.kind == 0 ? EvalJump<true>(t, slot, st, rm, rf, rb, s.de, s.mmm, s.mm2, s.small->pairtype, lane)
                      : EvalJump<false>(t, slot, st, rm, rf, rb, s.de, s.mmm, s.mm2, s.small->pairtype, lane);
    const long long acc_de = WarpSum(a.de), acc_d = WarpSum(a.d), acc_ks = WarpSum(a.ks);
    bad_all |= __reduce_or_sync(0xffffffffu, a.bad) | (ok ? 0u : kStatusNoCoefficients);
    if (lane == 0) {
      double ea = nan(""), de = nan("");
      if (ok) {
        const JumpOut o = JumpEpilogue(t, ExpConsts{t.exp_tab, t.exp_l1, t.exp_l2}, g.kind, slot, acc_de, acc_d, acc_ks);
        ea = o.ea;
        de = o.de;
      }
      g.ea[i] = static_cast<float>(ea);
      if (g.ea64) g.ea64[i] = ea;
      if (g.de64) g.de64[i] = de;
    }
    WriteFeatures(rm, s.small->rank[mig], g.enc, g.in_pad, g.features + i * g.in_pad, lane);
    __syncwarp();
  }
  if (bad_all && lane == 0) atomicOr(g.status, static_cast<int>(bad_all));
}

// Features of lattice jumps, one thread per pair (channels per site kEh known at
// compile time): the 58 MMM-ordered sites are gathered with independent loads
// and the row of in_pad bf16 values (a multiple of 8, 16-byte aligned) is
// written as 16-byte stores, 8 features at a time. Same values as the warp
// kernel below, which serves other row layouts.
template <int kEh>
__global__ void __launch_bounds__(256) surrogate_features_thread_kernel(
    DevTables t, const int8_t *__restrict__ species, int n, const long long *__restrict__ pairs, int m, int in_pad,
    FeatEnc enc, __nv_bfloat16 *features, int *status) {
  __shared__ int8_t s_off[12 * kEnvSites * 4];
  __shared__ int8_t s_rank[8];
  __shared__ int8_t s_dir_of[27];
  StageArray(t.mmm_off, s_off, 12 * kEnvSites * 4);
  if (threadIdx.x < 8) s_rank[threadIdx.x] = static_cast<int8_t>(FeatChannel(enc, t.onehot_rank[threadIdx.x]));
  if (threadIdx.x < 27) s_dir_of[threadIdx.x] = t.dir_of[threadIdx.x];
  __syncthreads();
  const long long nsites = 4LL * n * n * n;
  unsigned bad_all = 0;
  for (long long p = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; p < m;
       p += static_cast<long long>(gridDim.x) * blockDim.x) {
    const long long a = pairs[2 * p], b = pairs[2 * p + 1];
    unsigned bad = (a < 0 || b < 0 || a >= nsites || b >= nsites) ? kStatusBadSite : 0u;
    int di = -1;
    H3 hi{0, 0, 0};
    if (!bad) {
      hi = SiteCoord(a, n);
      const H3 hj = SiteCoord(b, n);
      const int dx = WrapDelta(hj.x - hi.x, n), dy = WrapDelta(hj.y - hi.y, n), dz = WrapDelta(hj.z - hi.z, n);
      if (dx >= -1 && dx <= 1 && dy >= -1 && dy <= 1 && dz >= -1 && dz <= 1)
        di = s_dir_of[(dx + 1) * 9 + (dy + 1) * 3 + (dz + 1)];
      if (di < 0) bad = kStatusNotNeighbor;
    }
    bad_all |= bad;
    int8_t rk[kEnvSites + 1];
    if (!bad) {
      const int8_t *o = s_off + di * kEnvSites * 4;
#pragma unroll
      for (int k = 0; k < kEnvSites; ++k) rk[k] = species[NeighborId(hi, o[4 * k], o[4 * k + 1], o[4 * k + 2], n)];
      rk[kEnvSites] = species[b];
#pragma unroll
      for (int k = 0; k <= kEnvSites; ++k) rk[k] = s_rank[rk[k]];
    } else {
#pragma unroll
      for (int k = 0; k <= kEnvSites; ++k) rk[k] = kMaxOnehot - 1;  // matches no rank: a zero row
    }
    uint4 *row = reinterpret_cast<uint4 *>(features + p * in_pad);
    constexpr int kFeat = (kEnvSites + 1) * kEh;
#pragma unroll
    for (int c = 0; c < (kFeat + 7) / 8; ++c) {
      uint32_t w[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        uint32_t word = 0;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int idx = 8 * c + 2 * e + h;
          if (idx < kFeat && rk[idx / kEh] == idx % kEh) word |= h ? 0x3F800000u : 0x3F80u;  // bf16 1.0
        }
        w[e] = word;
      }
      row[c] = make_uint4(w[0], w[1], w[2], w[3]);
    }
    for (int c = (kFeat + 7) / 8; c < in_pad / 8; ++c) row[c] = make_uint4(0, 0, 0, 0);
  }
  if (bad_all) atomicOr(status, static_cast<int>(bad_all));
}

// Features of lattice jumps (pairs first -> second), one warp per pair. The
// direction is found among the 12 neighbours of the first site (lanes 0-11),
// the 58 MMM-ordered sites are gathered into shared memory, and lane l writes
// features [8 l, 8 l + 8) as one 16-byte store (rows of a multiple of 8 values,
// 16-byte aligned; other layouts take the scalar writer).
__global__ void surrogate_features_kernel(DevTables t, const int8_t *__restrict__ species, int n,
                                          const long long *__restrict__ pairs, int m, int in_pad, FeatEnc enc,
                                          __nv_bfloat16 *features, int *status) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ int8_t s_ch[8];  // feature channel of each species code (-1: none)
  int8_t *arr = reinterpret_cast<int8_t *>(smem);
  if (threadIdx.x < 8) s_ch[threadIdx.x] = static_cast<int8_t>(FeatChannel(enc, t.onehot_rank[threadIdx.x]));
  __syncthreads();
  const int warps = blockDim.x >> 5;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int8_t *rm = arr + warp * 64;  // [0, 58) environment channels, [58] migrant channel, [59] padding (never matches)
  const int eh = enc.width;
  const long long nsites = 4LL * n * n * n;
  const bool vec = (in_pad % 8) == 0 && (reinterpret_cast<uintptr_t>(features) & 15) == 0 && in_pad <= 256;
  // this lane's 8 features: (source slot in rm, one-hot rank)
  int src[8], rk[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const int idx = 8 * lane + j;
    const int site = idx / eh;
    src[j] = idx < (kEnvSites + 1) * eh ? site : kEnvSites + 1;
    rk[j] = idx - site * eh;
  }
  const int8_t *dirs = t.dir;
  unsigned bad_all = 0;
  for (int p = blockIdx.x * warps + warp; p < m; p += gridDim.x * warps) {
    const long long a = pairs[2 * p], b = pairs[2 * p + 1];
    unsigned bad = (a < 0 || b < 0 || a >= nsites || b >= nsites) ? kStatusBadSite : 0u;
    int di = -1;
    H3 hi{0, 0, 0};
    if (!bad) {
      hi = SiteCoord(a, n);
      bool hit = false;
      if (lane < 12) {
        const int8_t *o = dirs + lane * 4;
        hit = NeighborId(hi, o[0], o[1], o[2], n) == b;
      }
      const unsigned mk = __ballot_sync(0xffffffffu, hit);
      di = mk ? __ffs(mk) - 1 : -1;
      if (di < 0) bad = kStatusNotNeighbor;
    }
    if (!bad) {
      for (int k = lane; k < kEnvSites; k += 32) {
        const int8_t *o = t.mmm_off + (di * kEnvSites + k) * 4;
        rm[k] = s_ch[species[NeighborId(hi, o[0], o[1], o[2], n)]];
      }
      if (lane == 0) rm[kEnvSites] = s_ch[species[b]];
    } else {
      for (int k = lane; k <= kEnvSites; k += 32) rm[k] = -1;
    }
    if (lane == 0) rm[kEnvSites + 1] = -1;
    bad_all |= bad;
    __syncwarp();
    __nv_bfloat16 *row = features + static_cast<long long>(p) * in_pad;
    if (vec) {
      if (8 * lane < in_pad) {
        uint32_t w[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const bool lo = rm[src[2 * e]] == rk[2 * e], hi2 = rm[src[2 * e + 1]] == rk[2 * e + 1];
          w[e] = (lo ? 0x3F80u : 0u) | (hi2 ? 0x3F800000u : 0u);  // bf16 1.0 in the low / high half
        }
        *reinterpret_cast<uint4 *>(row + 8 * lane) = make_uint4(w[0], w[1], w[2], w[3]);
      }
    } else {
      // rm already holds channels: write them through the identity encoding of this width
      const FeatEnc id{0x0706050403020100ull, eh};
      WriteFeatures(rm, rm[kEnvSites], id, in_pad, row, lane);
    }
    __syncwarp();
  }
  if (bad_all && lane == 0) atomicOr(status, static_cast<int>(bad_all));
}

// ---------------------------------------------------------------------------
// K4: persistent batched-replica KMC. A block owns R replicas with G warps
// each; per step: gather the 135-site neighbourhood of the vacancy, evaluate
// the 12 jumps (warp g takes jumps g, g+G, ...), then warp 0 of the replica
// turns them into rates, draws (u1, u2), selects the event and updates the
// lattice, clock and energy.
// ---------------------------------------------------------------------------
struct KmcShared {
  int8_t local[kLocalSites + 1];
  int8_t pad0[7];
  long long acc[12][3];
  int slot[12];
  long long ids[12];
  double beta;
  double corr;
  float beta_f;                     // beta rounded to FP32 (FP32 rates)
  int stop;
  int dsel;                         // direction index of the selected jump
  int escaped;                      // early stop: this step's vacancy had only solvent in its 1-3NN shells
  int nbk;                          // non-base sites in the neighbourhood (sparse evaluation)
  int has_x;                        // one of them is a vacancy (the checked sparse sums)
  int npairs;                       // pairs of them that share a cluster in some jump
  uint8_t nb_l[kMaxSparseSites + 1];    // their local indices; padding: kLocalSites (in no list)
  int8_t nb_code[kMaxSparseSites + 1];  // and species; padding: the base species
  uint16_t pairs[kMaxSparsePairs];      // (k | k2 << 8), k2 < k indices into nb_l; padding: (32, 32)
};

// 1 / kT and the vacancy-concentration time correction at temperature `temp`
// (RateCorrector::GetTimeCorrectionFactor, RateCorrector.hpp:17-24; 1 without one).
__device__ __noinline__ void TemperatureFactors(const KmcDevState &s, int r, double temp, double *beta,
                                                   double *corr) {
  *beta = 1.0 / kBoltzmannEv / temp;
  double c = 1.0;
  if (s.corr_cvac[r] >= 0.0) {
    const double cv = 1.64 * exp(-(0.66 / kBoltzmannEv / temp - 0.7));
    c = s.corr_cvac[r] / cv / (1 - 13 * s.corr_csol[r]);
  }
  *corr = c;
}

__device__ __forceinline__ double InterpT(const double *tt, const double *tv, int len, double time) {
  // TimeTemperatureInterpolator::GetTemperature (TimeTemperatureInterpolator.cpp:44-65)
  int lo = 0, hi = len;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (tt[mid] < time) lo = mid + 1;
    else hi = mid;
  }
  if (lo == len) return tv[len - 1];
  if (lo == 0 && time <= tt[0]) return tv[0];
  const double ux = tt[lo], uy = tv[lo], lx = tt[lo - 1], ly = tv[lo - 1];
  return ly + ((time - lx) / (ux - lx)) * (uy - ly);
}

// Pair term of one environment pair cluster (see KmcSparse): the cluster's
// entry minus the two entries with one site at the base species. "No cluster"
// lookups address a block of zeros. A site of rank kMaxOnehot - 1 (a vacancy
// or an element without a one-hot slot) is flagged by the single-site terms;
// its pair type is clamped so the loads stay in bounds.
__device__ __forceinline__ long long EnvPairTerm(uint32_t v, const long long *__restrict__ w, int p, int q, int rp,
                                                 int rq, int rb0, const int8_t *pt) {
  const int fb = v & 0xFFFFF, mode = (v >> 20) & 3;
  const bool lower_first = (v >> 22) & 1;
  const bool first = (p < q) == lower_first;  // p is the cluster's first site
  const int ra = first ? rp : rq, rb = first ? rq : rp;
  const int8_t *row = pt + mode * 64;
  const int t_ab = max(0, static_cast<int>(row[ra * 8 + rb]));
  const int t_a0 = max(0, static_cast<int>(row[ra * 8 + rb0]));
  const int t_0b = max(0, static_cast<int>(row[rb0 * 8 + rb]));
  return __ldg(&w[fb + t_ab]) - __ldg(&w[fb + t_a0]) - __ldg(&w[fb + t_0b]);
}

struct LaneAcc {
  long long a, b;
  unsigned bad;
};

// Sparse evaluation of one half of jump c over the replica's non-base sites
// and their interacting pairs (lists padded to multiples of 4 with entries
// that fall outside every list). Part 0 sums the energy change (list A =
// state) and the D or e0 form (list B = MMM); part 1 sums the Ks form over MM2
// forward (A) and backward (B). Branch-free, four entries at a time, so the
// table loads of independent entries overlap. Returns the corrections to the
// all-base constants.
// kCheckX: a listed site may be a vacancy (then the status bits of the reference's exceptions are
// formed); without one, no site lacks a one-hot rank and the checks are skipped.
template <bool kCheckX>
__device__ __forceinline__ LaneAcc EvalJumpPairsT(const KmcSparse &sp, const uint8_t *s_pos, const uint16_t *s_pxst,
                                                 const uint32_t *s_pxenv, const SmallTables *sm, const KmcShared &rs,
                                                 int e, int x, int c, int part, int mig, int slot, bool quartic) {
  long long acc_a = 0, acc_b = 0;
  unsigned bad = 0;
  const int rb0 = sm->rank[sp.base_code];
  const uint8_t *pos_a = s_pos + ((part == 0 ? 0 : 2) * 12 + c) * 136;
  const uint8_t *pos_b = s_pos + ((part == 0 ? 1 : 3) * 12 + c) * 136;
  constexpr int kEnvRows = kEnvSites + 1, kStateRows = kStateSites + 1;
  const long long *__restrict__ sg_a =
      part == 0 ? sp.s_de + mig * kStateRows * e : sp.s_env + (slot * 3 + 1) * kEnvRows * 8;
  const long long *__restrict__ sg_b = sp.s_env + (slot * 3 + (part == 1 ? 1 : (quartic ? 0 : 2))) * kEnvRows * 8;
  const int stride_a = part == 0 ? e : 8, zero_a = part == 0 ? kStateSites : kEnvSites;
  const long long *__restrict__ w_a = sp.dw_ks + static_cast<long long>(slot) * sp.dw_stride_mm2;
  const long long *__restrict__ w_b =
      part == 1 ? w_a : (quartic ? sp.dw_d : sp.dw_e0) + static_cast<long long>(slot) * sp.dw_stride_mmm;
  const uint32_t *px_a = s_pxenv + (kTriEnv + 1);
  const uint32_t *px_b = s_pxenv + (part == 1 ? kTriEnv + 1 : 0);
  const long long *__restrict__ pde = sp.p_de + mig * e * e;
  // single-site terms
  const int k_sites = rs.nbk;
  for (int k0 = 0; k0 < k_sites; k0 += 4) {
    long long va[4], vb[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int l = rs.nb_l[k0 + u], code = rs.nb_code[k0 + u];
      const int rp = sm->rank[code];
      const int pa = pos_a[l], pb = pos_b[l];
      const bool in_a = pa != 255, in_b = pb != 255;
      va[u] = __ldg(&sg_a[(in_a ? pa : zero_a) * stride_a + (part == 0 ? code : rp)]);
      vb[u] = __ldg(&sg_b[(in_b ? pb : kEnvSites) * 8 + rp]);
      if constexpr (kCheckX) {  // only a vacancy lacks a one-hot rank
        const bool bad_rank = rp == kMaxOnehot - 1;
        bad |= (part == 0 && in_a && code == x) ? kStatusBadCluster : 0u;
        bad |= (((part == 1 && in_a) || in_b) && bad_rank) ? kStatusXInEnv : 0u;
      }
    }
    acc_a += (va[0] + va[1]) + (va[2] + va[3]);
    acc_b += (vb[0] + vb[1]) + (vb[2] + vb[3]);
  }
  // pair terms over the pairs that share a cluster in some jump
  const int n_pairs = rs.npairs;
  for (int i0 = 0; i0 < n_pairs; i0 += 2) {
    long long va[2], vb[2];
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const unsigned pk = rs.pairs[i0 + u];
      const int k = pk & 0xFF, k2 = pk >> 8;
      const int l = rs.nb_l[k], l2 = rs.nb_l[k2];
      const int code = rs.nb_code[k], c2 = rs.nb_code[k2];
      const int pa = pos_a[l], qa = pos_a[l2], pb = pos_b[l], qb = pos_b[l2];
      const int rp = sm->rank[code], rq = sm->rank[c2];
      const bool both_a = pa != 255 && qa != 255, both_b = pb != 255 && qb != 255;
      if (part == 0) {
        const unsigned v = s_pxst[both_a ? Tri(pa, qa) : kTriState];
        const unsigned t0 = v & 0xFF, t1 = v >> 8;
        const long long f0 = __ldg(&pde[((t0 & 7) * e * e) * e + code * e + c2]);
        const long long f1 = __ldg(&pde[((t1 & 7) * e * e) * e + code * e + c2]);
        va[u] = ((t0 & 8) ? -f0 : f0) + ((t1 & 8) ? -f1 : f1);
      } else {
        va[u] = EnvPairTerm(px_a[both_a ? Tri(pa, qa) : kTriEnv], w_a, pa, qa, rp, rq, rb0, sm->pairtype);
      }
      vb[u] = EnvPairTerm(px_b[both_b ? Tri(pb, qb) : kTriEnv], w_b, pb, qb, rp, rq, rb0, sm->pairtype);
    }
    acc_a += va[0] + va[1];
    acc_b += vb[0] + vb[1];
  }
  return {acc_a, acc_b, bad};
}

// EvalJumpPairsT over the work units first, first + stride, ... of the item only (unit u < Gs:
// the four listed sites from 4u; unit Gs + v: the two pairs from 2v; Gs = the site groups), so
// that `stride` threads share the item and their partial sums add up to the whole (int64, exact).
template <bool kCheckX>
__device__ __forceinline__ LaneAcc EvalJumpPairsStrided(const KmcSparse &sp, const uint8_t *s_pos,
                                                       const uint16_t *s_pxst, const uint32_t *s_pxenv,
                                                       const SmallTables *sm, const KmcShared &rs, int e, int x,
                                                       int c, int part, int mig, int slot, bool quartic, int first,
                                                       int stride) {
  long long acc_a = 0, acc_b = 0;
  unsigned bad = 0;
  const int rb0 = sm->rank[sp.base_code];
  const uint8_t *pos_a = s_pos + ((part == 0 ? 0 : 2) * 12 + c) * 136;
  const uint8_t *pos_b = s_pos + ((part == 0 ? 1 : 3) * 12 + c) * 136;
  constexpr int kEnvRows = kEnvSites + 1, kStateRows = kStateSites + 1;
  const long long *__restrict__ sg_a =
      part == 0 ? sp.s_de + mig * kStateRows * e : sp.s_env + (slot * 3 + 1) * kEnvRows * 8;
  const long long *__restrict__ sg_b = sp.s_env + (slot * 3 + (part == 1 ? 1 : (quartic ? 0 : 2))) * kEnvRows * 8;
  const int stride_a = part == 0 ? e : 8, zero_a = part == 0 ? kStateSites : kEnvSites;
  const long long *__restrict__ w_a = sp.dw_ks + static_cast<long long>(slot) * sp.dw_stride_mm2;
  const long long *__restrict__ w_b =
      part == 1 ? w_a : (quartic ? sp.dw_d : sp.dw_e0) + static_cast<long long>(slot) * sp.dw_stride_mmm;
  const uint32_t *px_a = s_pxenv + (kTriEnv + 1);
  const uint32_t *px_b = s_pxenv + (part == 1 ? kTriEnv + 1 : 0);
  const long long *__restrict__ pde = sp.p_de + mig * e * e;
  // single-site terms
  const int k_sites = rs.nbk;
  // the four listed sites from k0
  auto site_group = [&](int k0) {
    long long va[4], vb[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int l = rs.nb_l[k0 + i], code = rs.nb_code[k0 + i];
      const int rp = sm->rank[code];
      const int pa = pos_a[l], pb = pos_b[l];
      const bool in_a = pa != 255, in_b = pb != 255;
      va[i] = __ldg(&sg_a[(in_a ? pa : zero_a) * stride_a + (part == 0 ? code : rp)]);
      vb[i] = __ldg(&sg_b[(in_b ? pb : kEnvSites) * 8 + rp]);
      if constexpr (kCheckX) {  // only a vacancy lacks a one-hot rank
        const bool bad_rank = rp == kMaxOnehot - 1;
        bad |= (part == 0 && in_a && code == x) ? kStatusBadCluster : 0u;
        bad |= (((part == 1 && in_a) || in_b) && bad_rank) ? kStatusXInEnv : 0u;
      }
    }
    acc_a += (va[0] + va[1]) + (va[2] + va[3]);
    acc_b += (vb[0] + vb[1]) + (vb[2] + vb[3]);
  };
  // pair terms over the pairs that share a cluster in some jump: the two pairs from i0
  auto pair_group = [&](int i0) {
    long long va[2], vb[2];
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      const unsigned pk = rs.pairs[i0 + i];
      const int k = pk & 0xFF, k2 = pk >> 8;
      const int l = rs.nb_l[k], l2 = rs.nb_l[k2];
      const int code = rs.nb_code[k], c2 = rs.nb_code[k2];
      const int pa = pos_a[l], qa = pos_a[l2], pb = pos_b[l], qb = pos_b[l2];
      const int rp = sm->rank[code], rq = sm->rank[c2];
      const bool both_a = pa != 255 && qa != 255, both_b = pb != 255 && qb != 255;
      if (part == 0) {
        const unsigned tv = s_pxst[both_a ? Tri(pa, qa) : kTriState];
        const unsigned t0 = tv & 0xFF, t1 = tv >> 8;
        const long long f0 = __ldg(&pde[((t0 & 7) * e * e) * e + code * e + c2]);
        const long long f1 = __ldg(&pde[((t1 & 7) * e * e) * e + code * e + c2]);
        va[i] = ((t0 & 8) ? -f0 : f0) + ((t1 & 8) ? -f1 : f1);
      } else {
        va[i] = EnvPairTerm(px_a[both_a ? Tri(pa, qa) : kTriEnv], w_a, pa, qa, rp, rq, rb0, sm->pairtype);
      }
      vb[i] = EnvPairTerm(px_b[both_b ? Tri(pb, qb) : kTriEnv], w_b, pb, qb, rp, rq, rb0, sm->pairtype);
    }
    acc_a += va[0] + va[1];
    acc_b += vb[0] + vb[1];
  };
  const int n_pairs = rs.npairs;
  int u = first;
  for (; 4 * u < k_sites; u += stride) site_group(4 * u);
  for (int v = u - (k_sites + 3) / 4; 2 * v < n_pairs; v += stride) pair_group(2 * v);
  return {acc_a, acc_b, bad};
}

// Shared-memory layout of the KMC kernels: jump cluster tables, small tables,
// local-index tables of the 12 jumps, the 135-site neighbourhood offsets, the
// ExpFast table, one KmcShared per replica, per-warp sorted arrays, then the
// sparse-evaluation tables (KmcSharedBytes gives the size).
struct KmcSmem {
  uint32_t *de, *mmm, *mm2;
  SmallTables *small;
  uint8_t *lst, *lmmm, *lmm2f, *lmm2b;  // [12][60], [12][58] x 3
  int8_t *loff;                         // [135][4]
  double *exp;                          // [kExpTableSize]
  KmcShared *rep;                       // [replicas per block]
  int8_t *arr;                          // [warps][kArr]
  uint8_t *pos;                         // [4][12][136]
  uint32_t *pxenv;                      // [2][kTriEnv + 1]
  uint32_t *inter;                      // [135][kInterWords]
  uint16_t *pxst;                       // [kTriState + 1]
  unsigned char *end;
};
__device__ __forceinline__ KmcSmem CarveKmcSmem(const DevTables &t, unsigned char *smem, int rpb, int g_per) {
  KmcSmem m;
  m.de = reinterpret_cast<uint32_t *>(smem);
  m.mmm = m.de + t.n_de_cl;
  m.mm2 = m.mmm + t.n_mmm_cl;
  m.small = reinterpret_cast<SmallTables *>(m.mm2 + t.n_mm2_cl);
  m.lst = reinterpret_cast<uint8_t *>(m.small + 1);
  m.lmmm = m.lst + 12 * kStateSites;
  m.lmm2f = m.lmmm + 12 * kEnvSites;
  m.lmm2b = m.lmm2f + 12 * kEnvSites;
  m.loff = reinterpret_cast<int8_t *>(m.lmm2b + 12 * kEnvSites);
  size_t off = reinterpret_cast<size_t>(m.loff + kLocalSites * 4);
  off = (off + 15) & ~size_t(15);
  m.exp = reinterpret_cast<double *>(off);
  m.rep = reinterpret_cast<KmcShared *>(m.exp + kExpTableSize);
  m.arr = reinterpret_cast<int8_t *>(m.rep + rpb);
  m.pos = reinterpret_cast<uint8_t *>(m.arr + rpb * g_per * kArr);
  m.pxenv = reinterpret_cast<uint32_t *>(m.pos + 4 * 12 * 136);
  m.inter = m.pxenv + 2 * (kTriEnv + 1);
  m.pxst = reinterpret_cast<uint16_t *>(m.inter + kLocalSites * kInterWords);
  m.end = reinterpret_cast<unsigned char *>(m.pxst + kTriState + 1);
  return m;
}
__device__ __forceinline__ void StageKmcSmem(const DevTables &t, const KmcSparse &sp, const KmcSmem &m, bool sparse) {
  if (sparse) {
    StageArray(sp.pos, m.pos, 4 * 12 * 136);
    StageArray(sp.px_st, m.pxst, kTriState + 1);
    StageArray(sp.px_env, m.pxenv, 2 * (kTriEnv + 1));
    StageArray(sp.inter, m.inter, kLocalSites * kInterWords);
  }
  StageArray(t.de_cl, m.de, t.n_de_cl);
  StageArray(t.mmm_cl, m.mmm, t.n_mmm_cl);
  StageArray(t.mm2_cl, m.mm2, t.n_mm2_cl);
  StageSmall(t, m.small);
  StageArray(t.local_st, m.lst, 12 * kStateSites);
  StageArray(t.local_mmm, m.lmmm, 12 * kEnvSites);
  StageArray(t.local_mm2f, m.lmm2f, 12 * kEnvSites);
  StageArray(t.local_mm2b, m.lmm2b, 12 * kEnvSites);
  StageArray(t.local_off, m.loff, kLocalSites * 4);
  StageArray(t.exp_tab, m.exp, kExpTableSize);
}

// Sparse evaluation, listing step (one warp): the non-base sites of the
// neighbourhood in rs.local (except the centre) with their species, padded to
// a multiple of 4, then the pairs of them that share a cluster in some jump
// (interaction table rows), padded to a multiple of 4. rs.nbk / rs.npairs above
// kMaxSparseSites / kMaxSparsePairs mean the lists are incomplete.
__device__ __forceinline__ void SparseList(KmcShared &rs, const uint32_t *s_inter, const KmcSparse &sp, int lane) {
  int k_sites = 0;
  bool any_x = false;
#pragma unroll
  for (int w = 0; w < 5; ++w) {
    const int k = w * 32 + lane;
    const int code = k < kLocalSites ? rs.local[k] : sp.base_code;
    const bool nb = code != sp.base_code && k != sp.center;
    any_x |= nb && code == sp.x_code;
    const unsigned mk = __ballot_sync(0xffffffffu, nb);
    const int idx = k_sites + __popc(mk & ((1u << lane) - 1u));
    if (nb && idx < kMaxSparseSites) {
      rs.nb_l[idx] = static_cast<uint8_t>(k);
      rs.nb_code[idx] = static_cast<int8_t>(code);
    }
    k_sites += __popc(mk);
  }
  // padding up to the next multiple of 4 (and the fixed entry 32)
  if (lane >= k_sites && lane < ((k_sites + 3) & ~3)) {
    rs.nb_l[lane] = static_cast<uint8_t>(kLocalSites);
    rs.nb_code[lane] = static_cast<int8_t>(sp.base_code);
  }
  if (lane == 0) {
    rs.nb_l[kMaxSparseSites] = static_cast<uint8_t>(kLocalSites);
    rs.nb_code[kMaxSparseSites] = static_cast<int8_t>(sp.base_code);
  }
  __syncwarp();
  // interacting pairs (k2 < k): lane k tests its row of the interaction table
  unsigned pm = 0;
  if (k_sites <= kMaxSparseSites && lane < k_sites) {
    const uint32_t *row = s_inter + rs.nb_l[lane] * kInterWords;
    for (int k2 = 0; k2 < lane; ++k2) {
      const int l2 = rs.nb_l[k2];
      pm |= ((row[l2 >> 5] >> (l2 & 31)) & 1u) << k2;
    }
  }
  const int cnt = __popc(pm);
  int pre = cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, pre, o);
    if (lane >= o) pre += v;
  }
  const int n_pairs = __shfl_sync(0xffffffffu, pre, 31);
  pre -= cnt;
  if (n_pairs <= kMaxSparsePairs) {
    while (pm) {
      const int k2 = __ffs(pm) - 1;
      pm &= pm - 1;
      rs.pairs[pre++] = static_cast<uint16_t>(lane | (k2 << 8));
    }
    if (lane < ((n_pairs + 3) & ~3) - n_pairs)
      rs.pairs[n_pairs + lane] = static_cast<uint16_t>(kMaxSparseSites | (kMaxSparseSites << 8));
  }
  const bool has_x = __any_sync(0xffffffffu, any_x);
  if (lane == 0) {
    rs.nbk = k_sites;
    rs.npairs = n_pairs;
    rs.has_x = has_x ? 1 : 0;
  }
}

// Sparse evaluation, one lane's item (0..23; larger items idle): jump c =
// item % 12, half item / 12 (0: energy change and the D / e0 sum, 1: the Ks
// sums). Writes rs.acc / rs.slot of its jump; returns the warp's status bits.
__device__ __forceinline__ unsigned SparseItem(const DevTables &t, const KmcSparse &sp, const uint8_t *s_lst,
                                               const uint8_t *s_pos, const uint16_t *s_pxst, const uint32_t *s_pxenv,
                                               const SmallTables *s_small, KmcShared &rs, int barrier_kind, int item) {
  const int c = item % 12, part = item / 12;
  LaneAcc la{0, 0, 0u};
  if (item < 24) {
    const int mig = rs.local[s_lst[c * kStateSites + t.pos_second]];
    const int slot = s_small->slot[mig];
    const bool quartic = barrier_kind == 0;
    const bool ok = slot >= 0 && (quartic ? s_small->has_quartic[slot] : s_small->has_e0[slot]);
    if (ok && (part == 0 || quartic))
      la = rs.has_x ? EvalJumpPairsT<true>(sp, s_pos, s_pxst, s_pxenv, s_small, rs, t.num_species, t.x_code, c,
                                           part, mig, slot, quartic)
                    : EvalJumpPairsT<false>(sp, s_pos, s_pxst, s_pxenv, s_small, rs, t.num_species, t.x_code, c,
                                            part, mig, slot, quartic);
    if (ok) {
      const long long *bf = sp.base_form + slot * 3;
      if (part == 0) {
        rs.acc[c][0] = sp.base_de[mig] + la.a;
        rs.acc[c][1] = (quartic ? bf[0] : bf[2]) + la.b;
      } else {
        rs.acc[c][2] = bf[1] + la.a + la.b;
      }
    }
    if (part == 0) rs.slot[c] = ok ? slot : (mig == t.x_code ? -2 : -1);
  }
  return __reduce_or_sync(0xffffffffu, la.bad);
}

// The 24 items of SparseItem shared by `subs` threads each (subs a power of two up to 16):
// thread tid of the group takes item tid / subs and every subs-th work unit of it, the subs
// partial sums meet by shuffles within their aligned lane group (int64: the same bits as one
// lane per item) and the group's first thread writes rs.acc / rs.slot. Every thread of a warp
// calls it (threads with tid >= 24 subs only take part in the shuffles). Returns the warp's
// status bits.
__device__ __forceinline__ unsigned SparseItemGroup(const DevTables &t, const KmcSparse &sp, const uint8_t *s_lst,
                                                    const uint8_t *s_pos, const uint16_t *s_pxst,
                                                    const uint32_t *s_pxenv, const SmallTables *s_small,
                                                    KmcShared &rs, int barrier_kind, int tid, int subs) {
  const int item = tid / subs, sub = tid - item * subs;
  const int c = item % 12, part = item / 12;
  LaneAcc la{0, 0, 0u};
  int mig = 0, slot = -1;
  bool ok = false;
  const bool quartic = barrier_kind == 0;
  if (item < 24) {
    mig = rs.local[s_lst[c * kStateSites + t.pos_second]];
    slot = s_small->slot[mig];
    ok = slot >= 0 && (quartic ? s_small->has_quartic[slot] : s_small->has_e0[slot]);
    if (ok && (part == 0 || quartic))
      la = rs.has_x ? EvalJumpPairsStrided<true>(sp, s_pos, s_pxst, s_pxenv, s_small, rs, t.num_species, t.x_code,
                                                 c, part, mig, slot, quartic, sub, subs)
                    : EvalJumpPairsStrided<false>(sp, s_pos, s_pxst, s_pxenv, s_small, rs, t.num_species, t.x_code,
                                                  c, part, mig, slot, quartic, sub, subs);
  }
  for (int o = subs >> 1; o > 0; o >>= 1) {
    la.a += __shfl_xor_sync(0xffffffffu, la.a, o);
    la.b += __shfl_xor_sync(0xffffffffu, la.b, o);
  }
  if (item < 24 && sub == 0) {
    if (ok) {
      const long long *bf = sp.base_form + slot * 3;
      if (part == 0) {
        rs.acc[c][0] = sp.base_de[mig] + la.a;
        rs.acc[c][1] = (quartic ? bf[0] : bf[2]) + la.b;
      } else {
        rs.acc[c][2] = bf[1] + la.a + la.b;
      }
    }
    if (part == 0) rs.slot[c] = ok ? slot : (mig == t.x_code ? -2 : -1);
  }
  return __reduce_or_sync(0xffffffffu, la.bad);
}

// Dense evaluation of the replica's 12 jumps (warp g takes jumps g, g + G, ...):
// gathers each jump's sorted state / MMM / MM2 lists into the warp's arrays and
// sums the cluster tables. Returns the status bits.
struct DenseArgs {
  const uint8_t *lst, *lmmm, *lmm2f, *lmm2b;
  const uint32_t *de, *mmm, *mm2;
  const SmallTables *small;
  int8_t *st, *rm, *rf, *rb;
};
__device__ __forceinline__ unsigned DenseJumps(const DevTables &t, KmcShared &rs, const DenseArgs &d, int kind, int g,
                                               int g_per, int lane) {
  unsigned bad_all = 0;
  for (int c = g; c < 12; c += g_per) {
    const uint8_t *lst = d.lst + c * kStateSites;
    for (int k = lane; k < kStateSites; k += 32) d.st[k] = rs.local[lst[k]];
    for (int k = lane; k < kEnvSites; k += 32) {
      d.rm[k] = d.small->rank[rs.local[d.lmmm[c * kEnvSites + k]]];
      d.rf[k] = d.small->rank[rs.local[d.lmm2f[c * kEnvSites + k]]];
      d.rb[k] = d.small->rank[rs.local[d.lmm2b[c * kEnvSites + k]]];
    }
    __syncwarp();
    const int mig = d.st[t.pos_second];
    const int slot = d.small->slot[mig];
    const bool ok = slot >= 0 && (kind == 0 ? d.small->has_quartic[slot] : d.small->has_e0[slot]);
    JumpAcc a{0, 0, 0, 0u};
    if (ok) {
      a = kind == 0 ? EvalJump<true>(t, slot, d.st, d.rm, d.rf, d.rb, d.de, d.mmm, d.mm2, d.small->pairtype, lane)
                    : EvalJump<false>(t, slot, d.st, d.rm, d.rf, d.rb, d.de, d.mmm, d.mm2, d.small->pairtype, lane);
    }
    const long long v0 = WarpSum(a.de), v1 = WarpSum(a.d), v2 = WarpSum(a.ks);
    bad_all |= __reduce_or_sync(0xffffffffu, a.bad);
    if (lane == 0) {
      rs.acc[c][0] = v0;
      rs.acc[c][1] = v1;
      rs.acc[c][2] = v2;
      // a jump onto another vacancy has no coefficients: rate 0
      rs.slot[c] = ok ? slot : (mig == t.x_code ? -2 : -1);
    }
    __syncwarp();
  }
  return bad_all;
}
// Out-of-line copy for kernels where the dense evaluation is the rare path.
__device__ __noinline__ unsigned DenseJumpsCold(const DevTables &t, KmcShared &rs, const DenseArgs &d, int kind, int g,
                                                int g_per, int lane) {
  return DenseJumps(t, rs, d, kind, g, g_per, lane);
}

// The reference's two draws per step on its mt19937_64 stream: u1 for the
// clock (returned as -log(u1)), then u2 for the selection.
__device__ __noinline__ double2 MtStepDraws(Mt mt) {
  const double nlog = -log(MtUniform(mt));  // KineticMcFirstOmp::CalculateTime draws first
  const double u2 = MtUniform(mt);          // then KineticMcFirstAbstract::SelectEvent
  return make_double2(nlog, u2);
}

// Time increment of a step with FP32 rates: the 12 rates are exp(lmin - Ea_i beta), relative to
// the fastest event (lmin = min Ea_i beta), and `total` is their FP64 sum, so
//   dt = -log(u1) / (total exp(-lmin) 1e13) * corr,
// with exp(lmin) = 2^yi 2^(y - yi), y = lmin log2(e): 2^yi exact in FP64, the rest in FP32.
__device__ __noinline__ double KmcDtWide(double nlog_u1, double total, float lmin, double corr) {
  return nlog_u1 * exp(static_cast<double>(lmin)) / (total * kPrefactor) * corr;
}
__device__ __forceinline__ double KmcDtF32(double nlog_u1, double total, float lmin, double corr) {
  const float y = lmin * 1.44269504088896341f;
  if (!(fabsf(y) < 1000.0f)) return KmcDtWide(nlog_u1, total, lmin, corr);
  const float yi = floorf(y);
  const float f = exp2f(y - yi) * __frcp_rn(__double2float_rn(total) * 1e13f);
  const double p2 = __hiloint2double((static_cast<int>(yi) + 1023) << 20, 0);
  return nlog_u1 * static_cast<double>(f) * p2 * corr;
}

// Synchronises the warps of one replica only: nothing for a single warp
// (beyond the warp itself), a named barrier (id 1 + replica slot) otherwise,
// so replicas sharing a block never wait for one another.
__device__ __forceinline__ void ReplicaSync(int g_per, int rl) {
  if (g_per == 1) {
    __syncwarp();
  } else {
    asm volatile("bar.sync %0, %1;" ::"r"(1 + rl), "r"(g_per * 32) : "memory");
  }
}

// Block shapes (kShape): 0 up to 256 threads with a register budget for 4
// resident blocks per SM; 1 up to 384 threads (12 warps per replica), 2
// resident blocks; 2 one block per SM of up to 28 single-warp replicas (one
// copy of the staged tables per SM, 72 registers per thread).
// kF32 (production Philox streams only): barriers and rates in FP32 (JumpEpilogueF32, rates
// relative to the fastest event), the rate sum and the clock in FP64, the energy in exact
// fixed point. Without it (and always on the reference's mt19937_64 stream) the epilogue,
// rates, sum and clock are FP64 as in the reference.
constexpr int kShapeThreads[3] = {256, 384, 896};
constexpr int kShapeBlocks[3] = {4, 2, 1};
template <bool kSparse, int kShape, bool kMt, bool kF32>
__global__ void __launch_bounds__(kShapeThreads[kShape], kShapeBlocks[kShape])
    kmc_kernel(const __grid_constant__ DevTables t, int8_t *species, const __grid_constant__ KmcDevState s,
               const __grid_constant__ KmcLaunch l) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int g_per = l.warps_per_replica;
  const int rpb = l.replicas_per_block;
  const KmcSmem sm = CarveKmcSmem(t, smem, rpb, g_per);
  StageKmcSmem(t, l.sp, sm, kSparse);
  __syncthreads();
  uint32_t *s_de = sm.de, *s_mmm = sm.mmm, *s_mm2 = sm.mm2;
  SmallTables *s_small = sm.small;
  uint8_t *s_lst = sm.lst, *s_lmmm = sm.lmmm, *s_lmm2f = sm.lmm2f, *s_lmm2b = sm.lmm2b;
  int8_t *s_loff = sm.loff, *s_arr = sm.arr;
  KmcShared *s_rep = sm.rep;
  uint8_t *s_pos = sm.pos;
  uint32_t *s_pxenv = sm.pxenv, *s_inter = sm.inter;
  uint16_t *s_pxst = sm.pxst;
  const ExpConsts ec{sm.exp, t.exp_l1, t.exp_l2};

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int rl = warp / g_per;         // replica within block
  const int g = warp - rl * g_per;     // warp within replica
  const int r = blockIdx.x * rpb + rl;
  const bool active = r < s.num_replicas;
  KmcShared &rs = s_rep[rl];
  int8_t *st = s_arr + warp * kArr;
  int8_t *rm = st + kStateSites, *rf = rm + kEnvSites, *rb = rf + kEnvSites;
  const int n = active ? s.lat_n[r] : 6;
  int8_t *lat = species + (active ? s.lat_off[r] : 0);
  long long vac = active ? s.vacancy[r] : 0;
  const bool leader = g == 0 && lane == 0;
  static_assert(!(kMt && kF32), "the reference's stream keeps the FP64 epilogue");
  using Real = typename std::conditional<kF32, float, double>::type;
  unsigned bad_all = 0;
  double time = 0, energy = 0;
  long long energy_fix = 0;  // FP32 mode: this launch's energy change in the dE fixed point (exact)
  unsigned long long step0 = 0, steps_done = 0;
  if (active && leader) {
    time = s.time[r];
    energy = s.energy[r];
  }
  if (active && g == 0) step0 = s.steps[r];
  uint32_t key0 = 0, key1 = 0;  // Philox key of the replica
  if (active && g == 0 && !kMt) {
    key0 = s.rng[r * kRngWords];
    key1 = s.rng[r * kRngWords + 1];
  }
  // Philox draws for 32 steps at a time: lane j holds -log(u1) and u2 of
  // step (it & ~31) + j, so the FP64 logarithm runs once per 32 steps
  double nlog_blk = 0.0, u2_blk = 0.0;
  Mt mt{nullptr, nullptr};
  int mt_left = 0, mt_pos = 0;  // steps of draws left in the warp's batch, the next one
  unsigned mt_base = 0;         // stream position of the batch's first draw
  if (active && kMt) {
    uint32_t *w = s.rng + static_cast<long long>(r) * kRngWords;
    mt.mt = reinterpret_cast<unsigned long long *>(w);
    mt.idx = w + 2 * 312;
  }
  if (!active || (s.early_stop && s.escaped[r])) return;  // no block-wide barrier below this point
  if (leader && s.tt_len == 0) {
    TemperatureFactors(s, r, s.temperature[r], &rs.beta, &rs.corr);
    rs.beta_f = static_cast<float>(rs.beta);
  }
  H3 hv = SiteCoord(vac, n);  // vacancy coordinates, advanced by the selected direction each step
  // threads per sparse item when several warps share a replica: the largest power of two (up to
  // 16) with 24 items x item_subs <= the replica's threads
  int item_subs = 1;
  while (item_subs < 16 && 48 * item_subs <= 32 * g_per) item_subs *= 2;
  for (unsigned long long it = 0; it < l.steps; ++it) {
    // ---- phase 1: neighbourhood gather, neighbour ids, temperature ----
    if (active) {
      const H3 h = hv;
      for (int k = g * 32 + lane; k < kLocalSites; k += g_per * 32) {
        const int8_t *o = s_loff + k * 4;
        rs.local[k] = lat[NeighborId(h, o[0], o[1], o[2], n)];
      }
      if (g == 0 && lane < 12) {
        const int8_t *o = t.dir + lane * 4;
        rs.ids[lane] = NeighborId(h, o[0], o[1], o[2], n);
      }
      if (leader) {
        if (s.tt_len > 0) {
          TemperatureFactors(s, r, InterpT(s.tt_time, s.tt_temp, s.tt_len, time), &rs.beta, &rs.corr);
          rs.beta_f = static_cast<float>(rs.beta);
        }
        rs.stop = (l.stop_flag && (it & 63) == 0 && *l.stop_flag) ? 1 : 0;
      }
    }
    ReplicaSync(g_per, rl);
    if (rs.stop) {
      bad_all |= kStatusStopped;
      break;
    }
    // ---- phase 2: the 12 jump evaluations ----
    if (kSparse) {
      // list the non-base sites of the neighbourhood (warp 0)
      if (g == 0) SparseList(rs, s_inter, l.sp, lane);
      ReplicaSync(g_per, rl);
    }
    const bool sparse_step = kSparse && rs.nbk <= kMaxSparseSites && rs.npairs <= kMaxSparsePairs;
    if (sparse_step) {
      if (kShape == 2 || g_per == 1) {
        // one lane per (jump, half): item = lane * G + g, items 0..23
        bad_all |= SparseItem(t, l.sp, s_lst, s_pos, s_pxst, s_pxenv, s_small, rs, s.barrier_kind, lane * g_per + g);
      } else {
        // the replica's warps share the 24 items, item_subs threads each
        bad_all |= SparseItemGroup(t, l.sp, s_lst, s_pos, s_pxst, s_pxenv, s_small, rs, s.barrier_kind,
                                   g * 32 + lane, item_subs);
      }
    }
    if (!sparse_step) {
      const DenseArgs da{s_lst, s_lmmm, s_lmm2f, s_lmm2b, s_de, s_mmm, s_mm2, s_small, st, rm, rf, rb};
      bad_all |= kSparse ? DenseJumpsCold(t, rs, da, s.barrier_kind, g, g_per, lane)
                         : DenseJumps(t, rs, da, s.barrier_kind, g, g_per, lane);
    }
    ReplicaSync(g_per, rl);
    // ---- phase 3: rates, selection, update (warp 0 of the replica) ----
    if (active && g == 0) {
      Real ea = 0, de = 0;
      double k = 0;
      float lmin = 0.0f;  // FP32 mode: min Ea beta over the 12 events
      long long id = 0x7fffffffffffffffLL;
      if constexpr (kF32) {
        bool ok = false;
        if (lane < 12) {
          const int slot = rs.slot[lane];
          id = rs.ids[lane];
          if (slot >= 0) {
            const JumpOutF o =
                JumpEpilogueF32(t, s.barrier_kind, slot, rs.acc[lane][0], rs.acc[lane][1], rs.acc[lane][2]);
            ea = o.ea;
            de = o.de;
            ok = true;
          } else if (slot == -1) {
            bad_all |= kStatusNoCoefficients;
          }
        }
        const float lb = ok ? ea * rs.beta_f : INFINITY;
        lmin = lb;
#pragma unroll
        for (int o = 8; o > 0; o >>= 1) lmin = fminf(lmin, __shfl_xor_sync(0xffffffffu, lmin, o));
        lmin = __shfl_sync(0xffffffffu, lmin, 0);
        // JumpEvent forward rate (JumpEvent.cpp:6-13), relative to exp(-lmin)
        k = ok ? static_cast<double>(expf(lmin - lb)) : 0.0;
      } else {
        if (lane < 12) {
          const int slot = rs.slot[lane];
          id = rs.ids[lane];
          if (slot >= 0) {
            const JumpOut o =
                JumpEpilogue(t, ec, s.barrier_kind, slot, rs.acc[lane][0], rs.acc[lane][1], rs.acc[lane][2]);
            ea = o.ea;
            de = o.de;
            k = ExpFast(-ea * rs.beta, ec);  // JumpEvent forward rate (JumpEvent.cpp:6-13)
          } else if (slot == -1) {
            bad_all |= kStatusNoCoefficients;
          }
        }
      }
      // lane q takes the event of rank q in the id-sorted 1NN list: the order depends only on
      // which axes of the vacancy lie on the periodic boundary (t.id_order)
      const int m2 = 2 * n - 1;
      const int bcase = (hv.x == 0 ? 9 : (hv.x == m2 ? 18 : 0)) + (hv.y == 0 ? 3 : (hv.y == m2 ? 6 : 0)) +
                        (hv.z == 0 ? 1 : (hv.z == m2 ? 2 : 0));
      const int src = lane < 12 ? __ldg(&t.id_order[bcase * 12 + lane]) : lane;
      const double k_s = __shfl_sync(0xffffffffu, k, src);
      const Real ea_s = __shfl_sync(0xffffffffu, ea, src);
      const Real de_s = __shfl_sync(0xffffffffu, de, src);
      const long long id_s = __shfl_sync(0xffffffffu, id, src);
      // total rate and prefix sums, sequential in id order (the reference's
      // single-thread reduction, KineticMcFirstOmp.cpp:55-68)
      double total = 0.0, mycum = 0.0;
      if (kMt) {
        for (int q = 0; q < 12; ++q) {
          total += __shfl_sync(0xffffffffu, k_s, q);
          if (lane == q) mycum = total;
        }
      } else {
        // production streams: inclusive scan in log2(16) = 4 shuffle steps
        mycum = lane < 12 ? k_s : 0.0;
#pragma unroll
        for (int o = 1; o < 16; o <<= 1) {
          const double v = __shfl_up_sync(0xffffffffu, mycum, o);
          if (lane >= o) mycum += v;
        }
        total = __shfl_sync(0xffffffffu, mycum, 11);
      }
      double nlog_u1 = 0, u2 = 0;  // -log(u1) for the clock, u2 for the selection
      if (kMt) {
        // the step's two draws; up to 32 steps' draws are read by the warp at once (lane j:
        // step j), within the current 312-word block, the index stored after every step
        if (mt_left == 0) {
          unsigned i = *mt.idx;
          if (i >= 312) {  // the serial generator twists on its next draw
            MtTwistInPlaceWarp(mt.mt, lane);
            i = 0;
          }
          if ((i & 1u) == 0) {
            mt_left = static_cast<int>(min(32u, (312u - i) / 2u));
            mt_base = i;
            mt_pos = 0;
            if (lane < mt_left) {
              nlog_blk = -log(MtCanonical(MtTemperOut(mt.mt[i + 2 * lane])));  // CalculateTime draws first
              u2_blk = MtCanonical(MtTemperOut(mt.mt[i + 2 * lane + 1]));      // then SelectEvent
            }
          } else if (lane == 0) {
            *mt.idx = i;  // an odd position: this step's draws one at a time
          }
          __syncwarp();
        }
        if (mt_left > 0) {
          nlog_u1 = __shfl_sync(0xffffffffu, nlog_blk, mt_pos);
          u2 = __shfl_sync(0xffffffffu, u2_blk, mt_pos);
          ++mt_pos;
          --mt_left;
          if (lane == 0) *mt.idx = mt_base + 2u * static_cast<unsigned>(mt_pos);
        } else {
          if (lane == 0) {
            const double2 d = MtStepDraws(mt);
            nlog_u1 = d.x;
            u2 = d.y;
          }
          u2 = __shfl_sync(0xffffffffu, u2, 0);
        }
      } else {
        if ((it & 31) == 0) {
          const unsigned long long ctr = step0 + it + lane;
          const uint4 x = PhiloxRound10(static_cast<uint32_t>(ctr), static_cast<uint32_t>(ctr >> 32),
                                        static_cast<uint32_t>(r), 0x4b4d43u, key0, key1);
          nlog_blk = -log(U01Open(x.x, x.y));
          u2_blk = U01(x.z, x.w);
        }
        nlog_u1 = __shfl_sync(0xffffffffu, nlog_blk, static_cast<int>(it & 31));
        u2 = __shfl_sync(0xffffffffu, u2_blk, static_cast<int>(it & 31));
      }
      bool hit;
      if (kMt) {
        // cumulative probabilities k_i / total summed in order, first one >= u2
        // (std::lower_bound in KineticMcFirstAbstract::SelectEvent); the sum stops there
        const double p = k_s / total;
        double cp = 0.0;
        int first = 11;  // none: the last event
        for (int q = 0; q < 12; ++q) {
          cp += __shfl_sync(0xffffffffu, p, q);
          if (cp >= u2) {
            first = q;
            break;
          }
        }
        hit = lane == first;
      } else {
        hit = lane < 12 && mycum >= u2 * total;
      }
      const unsigned ballot = __ballot_sync(0xffffffffu, hit);
      const int sel = ballot ? __ffs(ballot) - 1 : 11;  // past the end: the last event
      const int dsel = __shfl_sync(0xffffffffu, src, sel);
      const long long tgt = __shfl_sync(0xffffffffu, id_s, sel);
      const Real ea_sel = __shfl_sync(0xffffffffu, ea_s, sel);
      const Real de_sel = __shfl_sync(0xffffffffu, de_s, sel);
      if (lane == 0) {
        if (!(total > 0.0) || !isfinite(total)) bad_all |= kStatusNumeric;
        double dt;
        if constexpr (kF32) {
          dt = KmcDtF32(nlog_u1, total, lmin, rs.corr);
          energy_fix += rs.acc[dsel][0];
        } else {
          dt = nlog_u1 * RcpFast(total * kPrefactor) * rs.corr;
          energy += de_sel;
        }
        time += dt;
        lat[vac] = lat[tgt];  // Config::LatticeJump: the migrating atom takes the vacancy site
        lat[tgt] = static_cast<int8_t>(t.x_code);
        if (r == l.trace_replica && l.trace) {
          KmcTraceRec rec;
          rec.vacancy = vac;
          rec.target = tgt;
          rec.selected = sel;
          rec.slot = 0;
          rec.ea = ea_sel;
          rec.de = de_sel;
          rec.total_rate = kF32 ? total * exp(-static_cast<double>(lmin)) : total;
          rec.time = time;
          rec.energy = kF32 ? energy + static_cast<double>(energy_fix) * t.de_scale : energy;
          l.trace[it] = rec;
        }
        rs.ids[0] = tgt;
        rs.dsel = dsel;
      }
      if (s.early_stop) {
        // IsEscaped on the configuration before the jump (rs.local is this step's gather)
        const int sv = s.solvent[r];
        bool solvent_only = rs.local[t.shell_local[lane]] == sv;
        if (lane < 10) solvent_only = solvent_only && rs.local[t.shell_local[32 + lane]] == sv;
        const bool esc = __all_sync(0xffffffffu, solvent_only);
        if (lane == 0) rs.escaped = esc ? 1 : 0;
      }
      if (r == l.trace_replica && l.events12 && lane < 12) {
        double *ev = l.events12 + it * 36 + lane * 3;
        ev[0] = static_cast<double>(id_s);
        ev[1] = ea_s;
        ev[2] = de_s;
      }
      vac = tgt;
    }
    ReplicaSync(g_per, rl);
    if (active && g != 0) vac = rs.ids[0];
    {
      const int8_t *o = t.dir + rs.dsel * 4;
      hv = WrapCoord(hv, o[0], o[1], o[2], n);
    }
    ++steps_done;
    const bool escaped_now = s.early_stop && rs.escaped;
    ReplicaSync(g_per, rl);
    if (escaped_now) {
      if (leader) s.escaped[r] = 1;
      break;
    }
  }
  if (active && leader) {
    s.vacancy[r] = vac;
    s.time[r] = time;
    s.energy[r] = kF32 ? energy + static_cast<double>(energy_fix) * t.de_scale : energy;
    s.steps[r] = step0 + steps_done;
  }
  bad_all = __reduce_or_sync(0xffffffffu, bad_all);  // a jump's status bits may sit in lanes 1-11
  if (bad_all && lane == 0) atomicOr(l.status, static_cast<int>(bad_all));
}

// ---------------------------------------------------------------------------
// K4c: second-order "chain" KMC (KineticMcChainOmpi.cpp:56-152): one block of 12
// warps per replica. Per step, warp d takes the neighbour i = k + dir[d] of the
// vacancy k, builds the neighbourhood of i as it is after the jump k -> i (the
// vacancy at i, the migrant at k) and evaluates the 12 jumps i -> l (the same
// sparse / dense evaluation as kmc_kernel): their rate sum and the barrier and
// energy change of i -> k. Warp 0 then forms, in the id order of the 12
// neighbours, the reverse events k -> i (barrier Ea(i->k) - dE(i->k), energy
// change -dE(i->k)), their rates and the second-order probabilities and time of
// KineticMcChainOmpi::CalculateTime (sums sequential in that order), draws one
// uniform (the time is deterministic), selects and moves the vacancy.
// ---------------------------------------------------------------------------
struct ChainShared {
  double total_i[kChainWarps];  // per direction: rate sum of the 12 jumps out of i
  double ea_ik[kChainWarps], de_ik[kChainWarps];
  long long id_i[kChainWarps];
  int opp[kChainWarps];  // local index of -dir[d] (where the migrant lands)
  int sel_dir;
  int stop;
};

size_t ChainSharedBytes(const DevTables &t, bool sparse) {
  KmcLaunch l{};
  l.warps_per_replica = 1;
  l.replicas_per_block = kChainWarps;
  l.sparse = sparse ? 1 : 0;
  size_t b = KmcSharedBytes(t, l);
  if (!sparse) b += 4 * 12 * 136 + 4 * 2 * (kTriEnv + 1) + 4 * kLocalSites * kInterWords + 2 * (kTriState + 1);
  b = (b + 15) & ~size_t(15);
  return b + ((sizeof(ChainShared) + 15) & ~size_t(15));
}

template <bool kSparse>
__global__ void __launch_bounds__(kChainWarps * 32, 2)
    kmc_chain_kernel(const __grid_constant__ DevTables t, int8_t *species, const __grid_constant__ KmcDevState s,
                     const __grid_constant__ KmcLaunch l) {
  extern __shared__ __align__(16) unsigned char smem[];
  const KmcSmem sm = CarveKmcSmem(t, smem, kChainWarps, 1);
  ChainShared *cs = reinterpret_cast<ChainShared *>((reinterpret_cast<size_t>(sm.end) + 15) & ~size_t(15));
  const int r = blockIdx.x;
  if (r >= s.num_replicas) return;  // block-uniform, before any barrier
  StageKmcSmem(t, l.sp, sm, kSparse);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // local index of the offset opposite to each direction
  {
    const int8_t *o = t.dir + warp * 4;
    __syncthreads();
    int found = -1;
    for (int k = lane; k < kLocalSites; k += 32) {
      const int8_t *q = sm.loff + k * 4;
      if (q[0] == -o[0] && q[1] == -o[1] && q[2] == -o[2]) found = k;
    }
    found = __reduce_max_sync(0xffffffffu, found);
    if (lane == 0) cs->opp[warp] = found;
  }
  const ExpConsts ec{sm.exp, t.exp_l1, t.exp_l2};
  KmcShared &rs = sm.rep[warp];
  int8_t *st = sm.arr + warp * kArr;
  int8_t *rm = st + kStateSites, *rf = rm + kEnvSites, *rb = rf + kEnvSites;
  const int n = s.lat_n[r];
  int8_t *lat = species + s.lat_off[r];
  const int center = sm.lst[t.pos_first];
  long long vac = s.vacancy[r], prev = s.prev[r];
  const bool leader = warp == 0 && lane == 0;
  unsigned bad_all = 0;
  double time = 0, energy = 0;
  unsigned long long step0 = s.steps[r], steps_done = 0;
  if (leader) {
    time = s.time[r];
    energy = s.energy[r];
  }
  uint32_t key0 = 0, key1 = 0;
  if (s.rng_kind != 0) {
    key0 = s.rng[r * kRngWords];
    key1 = s.rng[r * kRngWords + 1];
  }
  double u_blk = 0.0;
  Mt mt{nullptr, nullptr};
  if (s.rng_kind == 0) {
    uint32_t *w = s.rng + static_cast<long long>(r) * kRngWords;
    mt.mt = reinterpret_cast<unsigned long long *>(w);
    mt.idx = w + 2 * 312;
  }
  if (leader && s.tt_len == 0) TemperatureFactors(s, r, s.temperature[r], &sm.rep[0].beta, &sm.rep[0].corr);
  __syncthreads();
  H3 hk = SiteCoord(vac, n);
  for (unsigned long long it = 0; it < l.steps; ++it) {
    if (leader) {
      if (s.tt_len > 0)
        TemperatureFactors(s, r, InterpT(s.tt_time, s.tt_temp, s.tt_len, time), &sm.rep[0].beta, &sm.rep[0].corr);
      cs->stop = (l.stop_flag && (it & 63) == 0 && *l.stop_flag) ? 1 : 0;
    }
    __syncthreads();
    if (cs->stop) {
      bad_all |= kStatusStopped;
      break;
    }
    const double beta = sm.rep[0].beta;
    // ---- phase 1: warp d, the configuration after the jump k -> i ----
    {
      const int8_t *o = t.dir + warp * 4;
      const H3 hi = WrapCoord(hk, o[0], o[1], o[2], n);
      const long long id_i = NeighborId(hk, o[0], o[1], o[2], n);
      const int8_t mig = lat[id_i];
      for (int k = lane; k < kLocalSites; k += 32) {
        const int8_t *q = sm.loff + k * 4;
        rs.local[k] = lat[NeighborId(hi, q[0], q[1], q[2], n)];
      }
      __syncwarp();
      if (lane == 0) {
        rs.local[center] = static_cast<int8_t>(t.x_code);
        rs.local[cs->opp[warp]] = mig;
      }
      if (lane < 12) {
        const int8_t *q = t.dir + lane * 4;
        rs.ids[lane] = NeighborId(hi, q[0], q[1], q[2], n);
      }
      __syncwarp();
      bool sparse_v = false;
      if (kSparse) {
        SparseList(rs, sm.inter, l.sp, lane);
        __syncwarp();
        sparse_v = rs.nbk <= kMaxSparseSites && rs.npairs <= kMaxSparsePairs;
      }
      if (sparse_v) {
        bad_all |= SparseItem(t, l.sp, sm.lst, sm.pos, sm.pxst, sm.pxenv, sm.small, rs, s.barrier_kind, lane);
      } else {
        const DenseArgs da{sm.lst, sm.lmmm, sm.lmm2f, sm.lmm2b, sm.de, sm.mmm, sm.mm2, sm.small, st, rm, rf, rb};
        bad_all |= DenseJumpsCold(t, rs, da, s.barrier_kind, 0, 1, lane);
      }
      __syncwarp();
      double ea = 0, de = 0, k = 0;
      long long id = 0x7fffffffffffffffLL;
      if (lane < 12) {
        const int slot = rs.slot[lane];
        id = rs.ids[lane];
        if (slot >= 0) {
          const JumpOut jo = JumpEpilogue(t, ec, s.barrier_kind, slot, rs.acc[lane][0], rs.acc[lane][1], rs.acc[lane][2]);
          ea = jo.ea;
          de = jo.de;
          k = ExpFast(-ea * beta, ec);
        } else if (slot == -1) {
          bad_all |= kStatusNoCoefficients;
        }
      }
      // rate sum in id order (sequential), and the jump back to k
      int rank = 0;
      for (int q = 0; q < 12; ++q) {
        const long long oid = __shfl_sync(0xffffffffu, id, q);
        rank += (q != lane) && (oid < id);
      }
      int src = 0;
      for (int q = 0; q < 12; ++q)
        if (__shfl_sync(0xffffffffu, rank, q) == lane) src = q;
      const double k_s = __shfl_sync(0xffffffffu, k, src);
      double total = 0.0;
      for (int q = 0; q < 12; ++q) total += __shfl_sync(0xffffffffu, k_s, q);
      const unsigned back = __ballot_sync(0xffffffffu, lane < 12 && id == vac);
      const int bl = back ? __ffs(back) - 1 : 0;
      const double ea_ik = __shfl_sync(0xffffffffu, ea, bl), de_ik = __shfl_sync(0xffffffffu, de, bl);
      if (lane == 0) {
        cs->total_i[warp] = total;
        cs->ea_ik[warp] = ea_ik;
        cs->de_ik[warp] = de_ik;
        cs->id_i[warp] = id_i;
      }
    }
    __syncthreads();
    // ---- phase 2: second-order probabilities and time, selection, move (warp 0) ----
    if (warp == 0) {
      // lane q holds the neighbour of rank q in id order
      long long idd = lane < 12 ? cs->id_i[lane] : 0x7fffffffffffffffLL;
      int rank = 0;
      for (int q = 0; q < 12; ++q) {
        const long long oid = __shfl_sync(0xffffffffu, idd, q);
        rank += (q != lane) && (oid < idd);
      }
      int src = 0;
      for (int q = 0; q < 12; ++q)
        if (__shfl_sync(0xffffffffu, rank, q) == lane) src = q;
      const int d = lane < 12 ? src : 0;
      const long long id_i = cs->id_i[d];
      const double tot_i = cs->total_i[d];
      const double barrier_ki = cs->ea_ik[d] - cs->de_ik[d];  // JumpEvent::GetReverseJumpEvent
      const double de_ki = -cs->de_ik[d];
      const double rate_ki = lane < 12 ? ExpFast(-barrier_ki * beta, ec) : 0.0;
      const double back_ki = lane < 12 ? ExpFast((de_ki - barrier_ki) * beta, ec) : 0.0;
      double total_k = 0.0;
      for (int q = 0; q < 12; ++q) total_k += __shfl_sync(0xffffffffu, rate_ki, q);
      const double t_1 = 1 / total_k / kPrefactor;
      const double p_ki = rate_ki / total_k;
      const double p_ik = lane < 12 ? back_ki / tot_i : 0.0;
      const double bb = p_ki * p_ik, bk = p_ki * (1 - p_ik);
      const bool is_prev = lane < 12 && id_i == prev;
      const double t_i = lane < 12 ? 1 / tot_i / kPrefactor : 0.0;
      double beta_bar_k = 0, beta_k = 0, gamma_bar_k_j = 0, gamma_k_j = 0, beta_k_j = 0, alpha_k_j = 0, ts_num = 0,
             ts_j_num = 0;
      for (int q = 0; q < 12; ++q) {
        const double bbq = __shfl_sync(0xffffffffu, bb, q), bkq = __shfl_sync(0xffffffffu, bk, q);
        const double pq = __shfl_sync(0xffffffffu, p_ki, q), tq = __shfl_sync(0xffffffffu, t_i, q);
        const bool prq = __shfl_sync(0xffffffffu, is_prev ? 1 : 0, q) != 0;
        beta_bar_k += bbq;
        beta_k += bkq;
        gamma_bar_k_j += prq ? 0.0 : bbq;
        gamma_k_j += prq ? 0.0 : bkq;
        beta_k_j += prq ? bkq : 0.0;
        alpha_k_j += prq ? pq : 0.0;
        ts_num += (t_1 + tq) * bbq;
        ts_j_num += prq ? 0.0 : (t_1 + tq) * bbq;
      }
      const double ts = ts_num / beta_bar_k;
      const double ts_j = ts_j_num / gamma_bar_k_j;
      const double one_over = 1 / (1 - alpha_k_j);
      const double t_2 = one_over * (gamma_k_j * t_1 + gamma_bar_k_j * (ts_j + t_1 + beta_bar_k / beta_k * ts));
      const double pr = is_prev ? one_over * (gamma_bar_k_j / beta_k) * beta_k_j
                                : one_over * (1 + gamma_bar_k_j / beta_k) * bk;
      double cum = 0.0, mycum = 0.0;
      for (int q = 0; q < 12; ++q) {
        cum += __shfl_sync(0xffffffffu, pr, q);
        if (lane == q) mycum = cum;
      }
      double u = 0.0;
      if (s.rng_kind == 0) {
        if (lane == 0) u = MtUniform(mt);
        u = __shfl_sync(0xffffffffu, u, 0);
      } else {
        if ((it & 31) == 0) {
          const unsigned long long ctr = step0 + it + lane;
          const uint4 x = PhiloxRound10(static_cast<uint32_t>(ctr), static_cast<uint32_t>(ctr >> 32),
                                        static_cast<uint32_t>(r), 0x4b4d43u, key0, key1);
          u_blk = U01(x.z, x.w);
        }
        u = __shfl_sync(0xffffffffu, u_blk, static_cast<int>(it & 31));
      }
      const unsigned hit = __ballot_sync(0xffffffffu, lane < 12 && !(mycum < u));
      const int sel = hit ? __ffs(hit) - 1 : 11;
      const int sel_dir = __shfl_sync(0xffffffffu, d, sel);
      const long long tgt = __shfl_sync(0xffffffffu, id_i, sel);
      const double b_sel = __shfl_sync(0xffffffffu, barrier_ki, sel), de_sel = __shfl_sync(0xffffffffu, de_ki, sel);
      const double tot_sel = total_k;
      if (lane == 0) {
        if (!(total_k > 0.0) || !isfinite(total_k) || !isfinite(t_2) || !(t_2 >= 0.0)) bad_all |= kStatusNumeric;
        time += t_2 * sm.rep[0].corr;
        energy += de_sel;
        lat[vac] = lat[tgt];
        lat[tgt] = static_cast<int8_t>(t.x_code);
        if (r == l.trace_replica && l.trace) {
          KmcTraceRec rec;
          rec.vacancy = vac;
          rec.target = tgt;
          rec.selected = sel;
          rec.slot = 0;
          rec.ea = b_sel;
          rec.de = de_sel;
          rec.total_rate = tot_sel;
          rec.time = time;
          rec.energy = energy;
          l.trace[it] = rec;
        }
        cs->sel_dir = sel_dir;
      }
    }
    __syncthreads();
    {
      const int8_t *o = t.dir + cs->sel_dir * 4;
      prev = vac;
      vac = NeighborId(hk, o[0], o[1], o[2], n);
      hk = WrapCoord(hk, o[0], o[1], o[2], n);
    }
    ++steps_done;
  }
  if (leader) {
    s.vacancy[r] = vac;
    s.prev[r] = prev;
    s.time[r] = time;
    s.energy[r] = energy;
    s.steps[r] = step0 + steps_done;
  }
  bad_all = __reduce_or_sync(0xffffffffu, bad_all);  // a jump's status bits may sit in lanes 1-11
  if (bad_all && lane == 0) atomicOr(l.status, static_cast<int>(bad_all));
}

// ---------------------------------------------------------------------------
// K1b: jump energetics of a vacancy placed on each listed site, one warp per
// site (ansys::ExitTime::GetJumpEnergetics, ExitTime.cpp:257-310, and
// GetBarrierListAndExitTime, :217-255): the lattice's own vacancy becomes the
// solvent, the site becomes X, and its 12 jumps are evaluated with the sparse /
// dense code of kmc_kernel. Outputs per site: (Ea, dE, neighbour) in id order,
// the mean barrier and the exit time 1 / sum exp(-Ea beta) / prefactor, both
// summed over the barriers in ascending order as the reference does after its sort.
// ---------------------------------------------------------------------------
constexpr int kSiteJumpWarps = 8;
template <bool kSparse>
__global__ void __launch_bounds__(kSiteJumpWarps * 32)
    site_jumps_kernel(const __grid_constant__ DevTables t, const int8_t *__restrict__ species,
                      const __grid_constant__ SiteJumpArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const KmcSmem sm = CarveKmcSmem(t, smem, kSiteJumpWarps, 1);
  StageKmcSmem(t, a.sp, sm, kSparse);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  KmcShared &rs = sm.rep[warp];
  int8_t *st = sm.arr + warp * kArr;
  int8_t *rm = st + kStateSites, *rf = rm + kEnvSites, *rb = rf + kEnvSites;
  const ExpConsts ec{sm.exp, t.exp_l1, t.exp_l2};
  const int n = a.n;
  const int center = sm.lst[t.pos_first];
  unsigned bad_all = 0;
  for (long long q = static_cast<long long>(blockIdx.x) * kSiteJumpWarps + warp; q < a.m;
       q += static_cast<long long>(gridDim.x) * kSiteJumpWarps) {
    const long long site = a.sites ? a.sites[q] : q;
    const H3 h = SiteCoord(site, n);
    for (int k = lane; k < kLocalSites; k += 32) {
      const int8_t *o = sm.loff + k * 4;
      const long long id = NeighborId(h, o[0], o[1], o[2], n);
      rs.local[k] = k == center ? static_cast<int8_t>(t.x_code)
                                : (id == a.vacancy ? static_cast<int8_t>(a.solvent) : species[id]);
    }
    if (lane < 12) {
      const int8_t *o = t.dir + lane * 4;
      rs.ids[lane] = NeighborId(h, o[0], o[1], o[2], n);
    }
    __syncwarp();
    bool sparse_v = false;
    if (kSparse) {
      SparseList(rs, sm.inter, a.sp, lane);
      __syncwarp();
      sparse_v = rs.nbk <= kMaxSparseSites && rs.npairs <= kMaxSparsePairs;
    }
    if (sparse_v) {
      bad_all |= SparseItem(t, a.sp, sm.lst, sm.pos, sm.pxst, sm.pxenv, sm.small, rs, a.barrier_kind, lane);
    } else {
      const DenseArgs da{sm.lst, sm.lmmm, sm.lmm2f, sm.lmm2b, sm.de, sm.mmm, sm.mm2, sm.small, st, rm, rf, rb};
      bad_all |= DenseJumpsCold(t, rs, da, a.barrier_kind, 0, 1, lane);
    }
    __syncwarp();
    double ea = 0, de = 0;
    long long id = 0x7fffffffffffffffLL;
    if (lane < 12) {
      const int slot = rs.slot[lane];
      id = rs.ids[lane];
      if (slot >= 0) {
        const JumpOut o = JumpEpilogue(t, ec, a.barrier_kind, slot, rs.acc[lane][0], rs.acc[lane][1], rs.acc[lane][2]);
        ea = o.ea;
        de = o.de;
      } else {
        bad_all |= slot == -1 ? kStatusNoCoefficients : kStatusXInEnv;
      }
    }
    // id order (the reference's adjacency list) for the per-jump outputs
    int rank = 0, rank_ea = 0;
    for (int k2 = 0; k2 < 12; ++k2) {
      const long long oid = __shfl_sync(0xffffffffu, id, k2);
      const double oea = __shfl_sync(0xffffffffu, ea, k2);
      rank += (k2 != lane) && (oid < id);
      rank_ea += (k2 != lane) && (oea < ea || (oea == ea && k2 < lane));
    }
    if (lane < 12) {
      const long long o = q * 12 + rank;
      if (a.ea12) a.ea12[o] = ea;
      if (a.de12) a.de12[o] = de;
      if (a.nb12) a.nb12[o] = id;
    }
    // ascending barriers: sum and rate sum in that order (std::sort then the loop)
    int src = 0;
    for (int k2 = 0; k2 < 12; ++k2)
      if (__shfl_sync(0xffffffffu, rank_ea, k2) == lane) src = k2;
    const double ea_sorted = __shfl_sync(0xffffffffu, ea, src);
    if (a.average || a.exit_time) {
      double sum = 0.0, rate = 0.0;
      for (int k2 = 0; k2 < 12; ++k2) {
        const double b = __shfl_sync(0xffffffffu, ea_sorted, k2);
        sum += b;
        rate += exp(-b * a.beta_escape);
      }
      if (lane == 0) {
        if (a.average) a.average[q] = sum / 12.0;
        if (a.exit_time) a.exit_time[q] = 1.0 / rate / kPrefactor;
      }
    }
    __syncwarp();
  }
  if (bad_all && lane == 0) atomicOr(a.status, static_cast<int>(bad_all));
}

// ---------------------------------------------------------------------------
// K1s: batched barriers with the sparse evaluation. A vacancy's jumps are usually
// asked together (KineticMcFirstOmp::BuildEventList asks for all 12,
// KineticMcFirstOmp.cpp:57-64), so each warp takes 12 consecutive pairs and, for
// every run of pairs that share a first site holding a vacancy, gathers that
// site's 135-site neighbourhood once and evaluates its 12 jumps with the sparse
// sums of the KMC kernel (bit-identical to the dense sums); every other pair, a
// run whose neighbourhood is too rich for the sparse lists, or a run whose
// sparse items report anything, takes the dense per-pair path.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kSiteJumpWarps * 32)
    barrier_group_kernel(const __grid_constant__ DevTables t, const int8_t *__restrict__ species,
                         const __grid_constant__ BarrierGroupArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const KmcSmem sm = CarveKmcSmem(t, smem, kSiteJumpWarps, 1);
  StageKmcSmem(t, a.sp, sm, true);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  KmcShared &rs = sm.rep[warp];
  int8_t *st = sm.arr + warp * kArr;
  int8_t *rm = st + kStateSites, *rf = rm + kEnvSites, *rb = rf + kEnvSites;
  const ExpConsts ec{sm.exp, t.exp_l1, t.exp_l2};
  const int n = a.n;
  const long long nsites = 4LL * n * n * n;
  const long long m = a.m_dev ? min(a.m, static_cast<long long>(*a.m_dev)) : a.m;
  const long long *__restrict__ pairs = a.pairs;
  unsigned bad_all = 0;
  for (long long c0 = (static_cast<long long>(blockIdx.x) * kSiteJumpWarps + warp) * 12; c0 < m;
       c0 += static_cast<long long>(gridDim.x) * kSiteJumpWarps * 12) {
    const long long cend = min(c0 + 12, m);
    long long p = c0;
    while (p < cend) {
      const long long i = pairs[2 * p];
      long long q = p + 1;
      while (q < cend && pairs[2 * q] == i) ++q;
      bool group = i >= 0 && i < nsites && species[i] == t.x_code;
      if (group) {
        const H3 h = SiteCoord(i, n);
        for (int k = lane; k < kLocalSites; k += 32) {
          const int8_t *o = sm.loff + k * 4;
          rs.local[k] = species[NeighborId(h, o[0], o[1], o[2], n)];
        }
        __syncwarp();
        SparseList(rs, sm.inter, a.sp, lane);
        __syncwarp();
        group = rs.nbk <= kMaxSparseSites && rs.npairs <= kMaxSparsePairs &&
                SparseItem(t, a.sp, sm.lst, sm.pos, sm.pxst, sm.pxenv, sm.small, rs, a.kind, lane) == 0u;
        __syncwarp();
      }
      if (group) {
        // lane k writes pair p + k from the jump of its direction
        if (lane < q - p) {
          const long long pk = p + lane;
          H3 hi, hj;
          int di = -1, db = -1;
          unsigned bad = ResolvePair(t.dir_of, pairs[2 * pk], pairs[2 * pk + 1], n, &hi, &hj, &di, &db);
          const int slot = bad ? -1 : rs.slot[di];
          if (!bad && (slot < 0 || (a.kind == 0 ? !sm.small->has_quartic[slot] : !sm.small->has_e0[slot])))
            bad = kStatusNoCoefficients;
          if (bad) {
            a.ea[pk] = nan("");
            a.de[pk] = nan("");
            bad_all |= bad;
          } else {
            const JumpOut o = JumpEpilogue(t, ec, a.kind, slot, rs.acc[di][0], rs.acc[di][1], rs.acc[di][2]);
            a.ea[pk] = o.ea;
            a.de[pk] = o.de;
            if (a.d_or_e0) a.d_or_e0[pk] = a.kind == 0 ? exp(o.d_or_e0) : o.d_or_e0;
            if (a.ks) a.ks[pk] = a.kind == 0 ? exp(o.ks) : 0.0;
            if (!isfinite(o.ea)) bad_all |= kStatusNumeric;
          }
        }
        __syncwarp();
      } else {
        for (long long r = p; r < q; ++r)
          bad_all |= DensePairBarrier(t, species, n, pairs, r, a.kind, sm.de, sm.mmm, sm.mm2, sm.small, st, rm, rf, rb,
                                      a.ea, a.de, a.d_or_e0, a.ks, lane);
      }
      p = q;
    }
  }
  bad_all = __reduce_or_sync(0xffffffffu, bad_all);
  if (bad_all && lane == 0) atomicOr(a.status, static_cast<int>(bad_all));
}

// ---------------------------------------------------------------------------
// K3b: solute clusters (ansys::SoluteCluster, SoluteCluster.cpp:277-410).
// Connected components of the non-solvent sites under 1NN bonds by lock-free
// union-find: every root is hooked under a smaller root (so a parent id never
// exceeds its child's and every chain ends), finds halve their paths; a final
// read-only pass stores each site's root. Then one block per cluster evaluates
// EnergyPredictor::GetEnergyOfCluster (EnergyPredictor.cpp:97-184) on the
// cluster's sorted site set S (members and their 1-3NN shells) twice: with the
// members' own species on a solvent background, and with the solvent everywhere.
// ---------------------------------------------------------------------------
constexpr uint32_t kNoCluster = 0xFFFFFFFFu;
constexpr int kUnionLimit = 1 << 22;  // retries of one union (bounded; each retry follows progress elsewhere)

__global__ void solute_label_init_kernel(const int8_t *__restrict__ species, long long nsites, int solvent,
                                         uint32_t *parent) {
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < nsites;
       i += static_cast<long long>(gridDim.x) * blockDim.x)
    parent[i] = species[i] != solvent ? static_cast<uint32_t>(i) : kNoCluster;
}
// Root of x while unions run: parent[x] < x below the root, so at most x + 1 steps; path halving
// (g is an ancestor of x in the same tree, and only non-roots are written).
__device__ __forceinline__ uint32_t ClusterRoot(uint32_t *parent, uint32_t x) {
  volatile uint32_t *vp = parent;
  for (uint32_t it = 0, x0 = x; it <= x0; ++it) {
    const uint32_t p = vp[x];
    if (p == x) return x;
    const uint32_t g = vp[p];
    if (g != p) vp[x] = g;
    x = p;
  }
  return x;
}
// Root of x once the forest is final (read-only: a concurrent flatten writes only roots).
__device__ __forceinline__ uint32_t ClusterRootRead(const uint32_t *parent, uint32_t x) {
  const volatile uint32_t *vp = parent;
  for (uint32_t it = 0, x0 = x; it <= x0; ++it) {
    const uint32_t p = vp[x];
    if (p == x) return x;
    x = p;
  }
  return x;
}
__global__ void solute_hook_kernel(DevTables t, const int8_t *__restrict__ species, int n, int solvent,
                                   uint32_t *parent, int *status) {
  __shared__ int8_t s_dir[12 * 4];
  StageArray(t.dir, s_dir, 12 * 4);
  __syncthreads();
  const long long nsites = 4LL * n * n * n;
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < nsites;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    if (species[i] == solvent) continue;
    const H3 h = SiteCoord(i, n);
    for (int d = 0; d < 12; ++d) {
      const long long j = NeighborId(h, s_dir[d * 4], s_dir[d * 4 + 1], s_dir[d * 4 + 2], n);
      if (j < i || species[j] == solvent) continue;  // each bond once, from its smaller end
      int it = 0;
      for (; it < kUnionLimit; ++it) {
        uint32_t ra = ClusterRoot(parent, static_cast<uint32_t>(i)), rb = ClusterRoot(parent, static_cast<uint32_t>(j));
        if (ra == rb) break;
        if (ra < rb) {
          const uint32_t tmp = ra;
          ra = rb;
          rb = tmp;
        }
        if (atomicCAS(&parent[ra], ra, rb) == ra) break;
      }
      if (it == kUnionLimit) atomicOr(status, kStatusNumeric);
    }
  }
}
__global__ void solute_flatten_kernel(long long nsites, uint32_t *parent) {
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < nsites;
       i += static_cast<long long>(gridDim.x) * blockDim.x)
    if (parent[i] != kNoCluster) parent[i] = ClusterRootRead(parent, static_cast<uint32_t>(i));
}

__device__ __forceinline__ bool SortedHas(const long long *a, long long len, long long v) {
  long long lo = 0, hi = len;
  while (lo < hi) {
    const long long mid = (lo + hi) >> 1;
    if (a[mid] < v) lo = mid + 1;
    else hi = mid;
  }
  return lo < len && a[lo] == v;
}
constexpr int kClusterThreads = 128;
__global__ void __launch_bounds__(kClusterThreads) cluster_census_kernel(DevTables t, const int8_t *__restrict__ species,
                                                                          int n, int solvent, const long long *s_off,
                                                                          const long long *s_ids, const long long *l_off,
                                                                          const long long *l_ids, double *de) {
  __shared__ unsigned int hist[2][512];  // solute configuration, solvent configuration
  __shared__ uint32_t s_tri[160];
  __shared__ int8_t s_off4[kSiteSites * 4];
  __shared__ int8_t s_label[kSiteSites];
  __shared__ int16_t s_idx[8 * 6 * 6 * 6];
  const int e = t.num_species;
  const int k = blockIdx.x;
  for (int i = threadIdx.x; i < 1024; i += blockDim.x) (&hist[0][0])[i] = 0;
  StageArray(t.census_tri, s_tri, t.n_census_tri);
  StageArray(t.site_off, s_off4, kSiteSites * 4);
  StageArray(t.cluster_index, s_idx, 8 * e * e * e);
  __syncthreads();
  for (int q = threadIdx.x; q < kSiteSites; q += blockDim.x) {
    const int x = s_off4[q * 4], y = s_off4[q * 4 + 1], z = s_off4[q * 4 + 2];
    const int n2 = x * x + y * y + z * z;
    s_label[q] = n2 == 2 ? 1 : (n2 == 4 ? 2 : (n2 == 6 ? 3 : 0));
  }
  __syncthreads();
  const long long *S = s_ids + s_off[k], *L = l_ids + l_off[k];
  const long long ns = s_off[k + 1] - s_off[k], nl = l_off[k + 1] - l_off[k];
  const int8_t sv = static_cast<int8_t>(solvent);
  for (long long t1 = threadIdx.x; t1 < ns; t1 += blockDim.x) {
    const long long site = S[t1];
    const H3 h = SiteCoord(site, n);
    int8_t sp[kSiteSites];
    uint64_t in_s = 0;  // bit q: neighbour q lies in S
    for (int q = 0; q < kSiteSites; ++q) {
      const long long j = NeighborId(h, s_off4[q * 4], s_off4[q * 4 + 1], s_off4[q * 4 + 2], n);
      const bool ins = q == t.site_center || SortedHas(S, ns, j);
      in_s |= static_cast<uint64_t>(ins) << q;
      sp[q] = ins && SortedHas(L, nl, j) ? species[j] : sv;
    }
    const int c0 = sp[t.site_center];
    int idx = s_idx[(0 * e + c0) * e * e];
    if (idx >= 0) atomicAdd(&hist[0][idx], 1u);
    const int i0 = s_idx[(0 * e + sv) * e * e];
    if (i0 >= 0) atomicAdd(&hist[1][i0], 1u);
    for (int q = 0; q < kSiteSites; ++q) {
      const int l = s_label[q];
      if (l == 0 || !((in_s >> q) & 1)) continue;
      idx = s_idx[((l * e + c0) * e + sp[q]) * e];
      if (idx >= 0) atomicAdd(&hist[0][idx], 1u);
      const int i1 = s_idx[((l * e + sv) * e + sv) * e];
      if (i1 >= 0) atomicAdd(&hist[1][i1], 1u);
    }
    for (int q = 0; q < t.n_census_tri; ++q) {
      const uint32_t w = s_tri[q];
      const int l = w & 7, o1 = (w >> 3) & 63, o2 = (w >> 9) & 63;
      if (!((in_s >> o1) & 1) || !((in_s >> o2) & 1)) continue;
      idx = s_idx[((l * e + c0) * e + sp[o1]) * e + sp[o2]];
      if (idx >= 0) atomicAdd(&hist[0][idx], 1u);
      const int i2 = s_idx[((l * e + sv) * e + sv) * e + sv];
      if (i2 >= 0) atomicAdd(&hist[1][i2], 1u);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    // sequential in index order without contraction, as GetEncodeOfCluster + dot
    double ea = 0.0, eb = 0.0;
    for (int i = 0; i < t.num_theta; ++i) {
      ea = __dadd_rn(ea, __dmul_rn(t.theta[i], __ddiv_rn(static_cast<double>(hist[0][i]), t.census_bonds[i])));
      eb = __dadd_rn(eb, __dmul_rn(t.theta[i], __ddiv_rn(static_cast<double>(hist[1][i]), t.census_bonds[i])));
    }
    de[2 * k] = ea;
    de[2 * k + 1] = eb;
  }
}

// ---------------------------------------------------------------------------
// K4b: multi-vacancy KMC, one block of kMultiWarps warps per lattice.
// Every vacancy of the lattice is tracked (slots 0..V-1). Per step:
//  1. the warps re-evaluate the 12 events of each vacancy whose 135-site
//     neighbourhood changed, with the sparse / dense evaluation of kmc_kernel:
//     a single such vacancy (the usual step: only the moved one) by the whole
//     block (gather by all threads, the 24 sparse items shared by kMultiItemSubs
//     threads each), several by one warp each. A neighbourhood holding a second vacancy takes
//     the dense sums in which that vacancy contributes nothing: clusters with two
//     vacancies have no coefficients and a vacancy has no one-hot slot (the
//     reference throws there; this is the defined extension). A jump onto a
//     vacancy has rate 0. Per slot: the 12 rates in id order and their inclusive
//     scan in 4 shuffle steps (16 lanes, lanes 12-15 zero), K_v = scan[11];
//  2. warp 0 forms the inclusive prefix of K_v over the slots, 32 slots at a time
//     (inclusive scan in 5 shuffle steps, plus the running total of the previous
//     chunks), draws (-log u1, u2) from the lattice's Philox stream (counter =
//     step, lattice), takes x = u2 * total, the first slot v with prefix >= x and
//     K_v > 0, then y = x - prefix(v - 1) and the first event with scan >= y and a
//     positive rate (past the end: the last positive one); dt = -log(u1) / (total
//     * prefactor); the vacancy moves (the migrating atom's species comes from the
//     slot tables, filled at the slot's evaluation) and the slots whose
//     neighbourhoods contain one of the two changed sites are marked for step 1.
// The oracle restates exactly these operations (orc_kmc_multi). kF32 (production
// arithmetic, KmcMultiArgs::f32): FP32 barriers and rates (MultiSlotRates), the
// rate sums and the clock in FP64 as above, the energy as an exact fixed-point sum.
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool InLocal(const uint32_t *bits, int dx, int dy, int dz) {
  if (dx < -4 || dx > 4 || dy < -4 || dy > 4 || dz < -4 || dz > 4) return false;
  const int b = ((dx + 4) * kLocalSpan + (dy + 4)) * kLocalSpan + (dz + 4);
  return (bits[b >> 5] >> (b & 31)) & 1u;
}

size_t MultiSharedBytes(const DevTables &t, bool sparse) {
  KmcLaunch l{};
  l.warps_per_replica = 1;
  l.replicas_per_block = kMultiWarps;
  l.sparse = sparse ? 1 : 0;
  size_t b = KmcSharedBytes(t, l);
  // sparse tables are always carved (the layout is shared); add them when not counted
  if (!sparse) b += 4 * 12 * 136 + 4 * 2 * (kTriEnv + 1) + 4 * kLocalSites * kInterWords + 2 * (kTriState + 1);
  b = (b + 15) & ~size_t(15);
  b += sizeof(double) * kMaxMultiVac * 12;  // rate scans
  b += (2 * sizeof(double) + sizeof(long long)) * kMaxMultiVac * 12;  // Ea, dE, target of every event
  b += sizeof(double) * kMaxMultiVac;       // slot prefix
  b += sizeof(long long) * kMaxMultiVac;    // positions
  b += sizeof(H3) * kMaxMultiVac;           // coordinates
  b += sizeof(int) * kMaxMultiVac;          // dirty list
  b += sizeof(uint16_t) * kMaxMultiVac;     // positive-rate masks
  b += kMaxMultiVac * 12;                   // target species
  b += sizeof(int) * 4 + sizeof(uint32_t) * kLocalBitWords;
  return (b + 15) & ~size_t(15);
}

// Multi-vacancy KMC: rates of slot v from the sums in q (one warp): the 12 events in id order
// (the sorted 1NN list; the order depends only on which axes of the vacancy lie on the periodic
// boundary), their inclusive scan in FP64 (4 shuffle steps over 16 lanes), Ea, dE, targets, the
// targets' species (mig_local[d * kStateSites]: local index of direction d's migrant) and the
// positive-rate mask into the slot tables. Returns the status bits.
// kF32: JumpEpilogueF32 (barriers within 1e-6 relative of the FP64 epilogue) and rates
// 2^64 exp(-Ea / kT) = exp2(64 - Ea log2(e) / kT) in FP32 (the power-of-two scale keeps barriers
// up to about 130 kT above zero; the clock divides it out exactly); ea holds FP32 barriers (as
// float), de the energy change's exact fixed-point sum (as long long). Otherwise FP64 throughout.
struct MultiSlotTables {
  double *cum, *ea, *de;
  long long *tgt;
  uint16_t *kmask;
  int8_t *tsp;  // species on each target site (the migrating atom)
};
constexpr double kMultiRateScale = 18446744073709551616.0;  // 2^64, the FP32 rates' scale
template <bool kF32>
__device__ __forceinline__ unsigned MultiSlotRates(const DevTables &t, const ExpConsts &ec, int kind, double beta,
                                                   float beta_l2e, const KmcShared &q, H3 h, int n, int v,
                                                   const uint8_t *mig_local, const MultiSlotTables &o, int lane) {
  unsigned bad = 0;
  double ea = 0.0, de = 0.0, k = 0.0;
  float ea_f = 0.0f;
  long long de_fix = 0, id = 0x7fffffffffffffffLL;
  if (lane < 12) {
    const int slot = q.slot[lane];
    id = q.ids[lane];
    if (slot >= 0) {
      if constexpr (kF32) {
        const JumpOutF jo = JumpEpilogueF32(t, kind, slot, q.acc[lane][0], q.acc[lane][1], q.acc[lane][2]);
        ea_f = jo.ea;
        de_fix = q.acc[lane][0];
        const float kf = exp2f(fmaf(-ea_f, beta_l2e, 64.0f));
        if (!(kf < INFINITY)) bad |= kStatusNumeric;  // a barrier below -44 kT
        k = FloatToDouble(kf);
      } else {
        const JumpOut jo = JumpEpilogue(t, ec, kind, slot, q.acc[lane][0], q.acc[lane][1], q.acc[lane][2]);
        ea = jo.ea;
        de = jo.de;
        k = ExpFast(-ea * beta, ec);
      }
    } else if (slot == -1) {
      bad |= kStatusNoCoefficients;
    }
  }
  const int m2 = 2 * n - 1;
  const int bcase = (h.x == 0 ? 9 : (h.x == m2 ? 18 : 0)) + (h.y == 0 ? 3 : (h.y == m2 ? 6 : 0)) +
                    (h.z == 0 ? 1 : (h.z == m2 ? 2 : 0));
  const int src = lane < 12 ? __ldg(&t.id_order[bcase * 12 + lane]) : lane;
  const double k_s = __shfl_sync(0xffffffffu, k, src);
  const long long id_s = __shfl_sync(0xffffffffu, id, src);
  double cum = lane < 12 ? k_s : 0.0;
#pragma unroll
  for (int off = 1; off < 16; off <<= 1) {
    const double u = __shfl_up_sync(0xffffffffu, cum, off);
    if (lane >= off) cum += u;
  }
  const unsigned kpos = __ballot_sync(0xffffffffu, lane < 12 && k_s > 0.0);
  if constexpr (kF32) {
    const float ea_s = __shfl_sync(0xffffffffu, ea_f, src);
    const long long de_s = __shfl_sync(0xffffffffu, de_fix, src);
    if (lane < 12) {
      reinterpret_cast<float *>(o.ea)[v * 12 + lane] = ea_s;
      reinterpret_cast<long long *>(o.de)[v * 12 + lane] = de_s;
    }
  } else {
    const double ea_s = __shfl_sync(0xffffffffu, ea, src);
    const double de_s = __shfl_sync(0xffffffffu, de, src);
    if (lane < 12) {
      o.ea[v * 12 + lane] = ea_s;
      o.de[v * 12 + lane] = de_s;
    }
  }
  if (lane < 12) {
    o.cum[v * 12 + lane] = cum;
    o.tgt[v * 12 + lane] = id_s;
    o.tsp[v * 12 + lane] = q.local[mig_local[src * kStateSites]];
  }
  if (lane == 0) o.kmask[v] = static_cast<uint16_t>(kpos);
  __syncwarp();
  return bad;
}

template <bool kSparse, bool kF32>
__global__ void __launch_bounds__(kMultiWarps * 32, 1)
    kmc_multi_kernel(const __grid_constant__ DevTables t, int8_t *species, const __grid_constant__ KmcMultiArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const KmcSmem sm = CarveKmcSmem(t, smem, kMultiWarps, 1);
  size_t off = (reinterpret_cast<size_t>(sm.end) + 15) & ~size_t(15);
  double *s_cum = reinterpret_cast<double *>(off);                   // [kMaxMultiVac][12]
  double *s_ea = s_cum + kMaxMultiVac * 12;                           // [kMaxMultiVac][12], id order
  double *s_de = s_ea + kMaxMultiVac * 12;
  long long *s_tgt = reinterpret_cast<long long *>(s_de + kMaxMultiVac * 12);
  double *s_incl = reinterpret_cast<double *>(s_tgt + kMaxMultiVac * 12);  // [kMaxMultiVac]
  long long *s_pos = reinterpret_cast<long long *>(s_incl + kMaxMultiVac);
  H3 *s_h = reinterpret_cast<H3 *>(s_pos + kMaxMultiVac);
  int *s_list = reinterpret_cast<int *>(s_h + kMaxMultiVac);
  uint16_t *s_kmask = reinterpret_cast<uint16_t *>(s_list + kMaxMultiVac);
  int8_t *s_tsp = reinterpret_cast<int8_t *>(s_kmask + kMaxMultiVac);  // [kMaxMultiVac][12] target species
  int *s_ctl = reinterpret_cast<int *>(s_tsp + kMaxMultiVac * 12);     // [0] dirty count, [1] stop
  uint32_t *s_bits = reinterpret_cast<uint32_t *>(s_ctl + 4);
  const MultiSlotTables slot_tab{s_cum, s_ea, s_de, s_tgt, s_kmask, s_tsp};

  const int r = blockIdx.x;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int v0 = a.vac_off[r], nv = a.vac_off[r + 1] - v0;
  if (nv <= 0 || nv > kMaxMultiVac) return;  // block-uniform, before any barrier; the host rejects such lattices
  StageKmcSmem(t, a.sp, sm, kSparse);
  const int n = a.lat_n[r];
  int8_t *lat = species + a.lat_off[r];
  for (int i = threadIdx.x; i < kLocalBitWords; i += blockDim.x) s_bits[i] = a.local_bits[i];
  for (int i = threadIdx.x; i < nv; i += blockDim.x) {
    const long long p = a.vac_pos[v0 + i];
    s_pos[i] = p;
    s_h[i] = SiteCoord(p, n);
    s_list[i] = i;  // every slot is evaluated at the start of a launch
  }
  if (threadIdx.x == 0) {
    s_ctl[0] = nv;
    s_ctl[1] = 0;
  }
  __syncthreads();
  const ExpConsts ec{sm.exp, t.exp_l1, t.exp_l2};
  KmcShared &rs = sm.rep[warp];
  int8_t *st = sm.arr + warp * kArr;
  int8_t *rm = st + kStateSites, *rf = rm + kEnvSites, *rb = rf + kEnvSites;
  const int x_code = t.x_code;
  const int center = sm.lst[t.pos_first];  // local index of the vacancy site itself
  const double beta = 1.0 / kBoltzmannEv / a.temperature[r];
  const float beta_l2e = static_cast<float>(beta * 1.4426950408889634);  // FP32 rates: log2(e) / kT
  unsigned bad_all = 0;
  double time = 0.0, energy = 0.0;
  long long energy_fix = 0;  // FP32 mode: this launch's energy change in the dE fixed point (exact)
  unsigned long long step0 = 0, steps_done = 0;
  uint32_t key0 = 0, key1 = 0;
  if (warp == 0) {
    time = a.time[r];
    energy = a.energy[r];
    step0 = a.steps[r];
    key0 = a.key[2 * r];
    key1 = a.key[2 * r + 1];
  }
  double nlog_blk = 0.0, u2_blk = 0.0;
  for (unsigned long long it = 0; it < a.nsteps; ++it) {
    // ---- phase 1: re-evaluate the marked slots ----
    const int nd = s_ctl[0];
    if (kSparse && nd == 1) {
      // one slot (the usual step: only the moved vacancy): the block gathers its neighbourhood,
      // warp 0 lists the non-base sites, kMultiItemWarps warps share the 24 sparse items
      const int v = s_list[0];
      KmcShared &q = sm.rep[0];
      const H3 h = s_h[v];
      bool other = false;  // a second vacancy in the neighbourhood
      for (int k = threadIdx.x; k < kLocalSites; k += blockDim.x) {
        const int8_t *o = sm.loff + k * 4;
        const int8_t c = lat[NeighborId(h, o[0], o[1], o[2], n)];
        q.local[k] = c;
        other |= c == x_code && k != center;
      }
      if (threadIdx.x < 12) {
        const int8_t *o = t.dir + threadIdx.x * 4;
        q.ids[threadIdx.x] = NeighborId(h, o[0], o[1], o[2], n);
      }
      const bool extra_x = __syncthreads_or(other);
      if (!extra_x && warp == 0) SparseList(q, sm.inter, a.sp, lane);
      __syncthreads();
      const bool sparse_v = !extra_x && q.nbk <= kMaxSparseSites && q.npairs <= kMaxSparsePairs;
      if (sparse_v) {
        if (warp < kMultiItemWarps)
          bad_all |= SparseItemGroup(t, a.sp, sm.lst, sm.pos, sm.pxst, sm.pxenv, sm.small, q, a.barrier_kind,
                                     threadIdx.x, kMultiItemSubs);
      } else if (warp == 0) {
        const DenseArgs da{sm.lst, sm.lmmm, sm.lmm2f, sm.lmm2b, sm.de, sm.mmm, sm.mm2, sm.small, st, rm, rf, rb};
        unsigned b = DenseJumpsCold(t, q, da, a.barrier_kind, 0, 1, lane);
        if (extra_x) b &= ~static_cast<unsigned>(kStatusXInEnv | kStatusBadCluster);
        bad_all |= b;
      }
      __syncthreads();
      if (warp == 0)
        bad_all |= MultiSlotRates<kF32>(t, ec, a.barrier_kind, beta, beta_l2e, q, h, n, v, sm.lst + t.pos_second,
                                        slot_tab, lane);
    } else {
      // several slots (the first step, or a move next to another vacancy): one warp per slot
      for (int qi = warp; qi < nd; qi += kMultiWarps) {
        const int v = s_list[qi];
        const H3 h = s_h[v];
        bool other = false;  // a second vacancy in the neighbourhood
        for (int k = lane; k < kLocalSites; k += 32) {
          const int8_t *o = sm.loff + k * 4;
          const int8_t c = lat[NeighborId(h, o[0], o[1], o[2], n)];
          rs.local[k] = c;
          other |= c == x_code && k != center;
        }
        if (lane < 12) {
          const int8_t *o = t.dir + lane * 4;
          rs.ids[lane] = NeighborId(h, o[0], o[1], o[2], n);
        }
        const bool extra_x = __any_sync(0xffffffffu, other);
        __syncwarp();
        bool sparse_v = false;
        if (kSparse && !extra_x) {
          SparseList(rs, sm.inter, a.sp, lane);
          __syncwarp();
          sparse_v = rs.nbk <= kMaxSparseSites && rs.npairs <= kMaxSparsePairs;
        }
        if (sparse_v) {
          bad_all |= SparseItem(t, a.sp, sm.lst, sm.pos, sm.pxst, sm.pxenv, sm.small, rs, a.barrier_kind, lane);
        } else {
          const DenseArgs da{sm.lst, sm.lmmm, sm.lmm2f, sm.lmm2b, sm.de, sm.mmm, sm.mm2, sm.small, st, rm, rf, rb};
          unsigned b = DenseJumpsCold(t, rs, da, a.barrier_kind, 0, 1, lane);
          if (extra_x) b &= ~static_cast<unsigned>(kStatusXInEnv | kStatusBadCluster);
          bad_all |= b;
        }
        __syncwarp();
        bad_all |= MultiSlotRates<kF32>(t, ec, a.barrier_kind, beta, beta_l2e, rs, h, n, v, sm.lst + t.pos_second,
                                        slot_tab, lane);
      }
    }
    __syncthreads();
    // ---- phase 2: selection over all slots and the move (warp 0) ----
    if (warp == 0) {
      if (lane == 0) s_ctl[1] = (a.stop_flag && (it & 63) == 0 && *a.stop_flag) ? 1 : 0;
      __syncwarp();
      if (s_ctl[1] == 0) {
        if ((it & 31) == 0) {
          const unsigned long long ctr = step0 + it + lane;
          const uint4 xr = PhiloxRound10(static_cast<uint32_t>(ctr), static_cast<uint32_t>(ctr >> 32),
                                         static_cast<uint32_t>(r), 0x4b4d43u, key0, key1);
          nlog_blk = -log(U01Open(xr.x, xr.y));
          u2_blk = U01(xr.z, xr.w);
        }
        const double nlog_u1 = __shfl_sync(0xffffffffu, nlog_blk, static_cast<int>(it & 31));
        const double u2 = __shfl_sync(0xffffffffu, u2_blk, static_cast<int>(it & 31));
        const int chunks = (nv + 31) >> 5;
        double run = 0.0;
        for (int c = 0; c < chunks; c += 2) {
          // two chunks' scans side by side (the same additions as one after the other)
          const int v0 = c * 32 + lane, v1 = v0 + 32;
          double sc0 = v0 < nv ? s_cum[v0 * 12 + 11] : 0.0;
          if (c + 1 < chunks) {  // warp-uniform
            double sc1 = v1 < nv ? s_cum[v1 * 12 + 11] : 0.0;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
              const double u0 = __shfl_up_sync(0xffffffffu, sc0, o);
              const double u1 = __shfl_up_sync(0xffffffffu, sc1, o);
              if (lane >= o) {
                sc0 += u0;
                sc1 += u1;
              }
            }
            if (v0 < nv) s_incl[v0] = run + sc0;
            run = run + __shfl_sync(0xffffffffu, sc0, 31);
            if (v1 < nv) s_incl[v1] = run + sc1;
            run = run + __shfl_sync(0xffffffffu, sc1, 31);
          } else {
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
              const double u0 = __shfl_up_sync(0xffffffffu, sc0, o);
              if (lane >= o) sc0 += u0;
            }
            if (v0 < nv) s_incl[v0] = run + sc0;
            run = run + __shfl_sync(0xffffffffu, sc0, 31);
          }
        }
        const double total = run;
        __syncwarp();
        const double xs = __dmul_rn(u2, total);  // not contracted with the subtraction below
        int vsel = -1, vlast = -1;
        for (int c = 0; c < chunks; ++c) {
          const int v = c * 32 + lane;
          const bool pos = v < nv && s_kmask[v] != 0;
          const unsigned hit = __ballot_sync(0xffffffffu, pos && s_incl[v] >= xs);
          const unsigned any = __ballot_sync(0xffffffffu, pos);
          if (vsel < 0 && hit) vsel = c * 32 + __ffs(hit) - 1;
          if (any) vlast = c * 32 + 31 - __clz(any);
        }
        if (vsel < 0) vsel = vlast;
        if (vsel < 0 || !(total > 0.0) || !isfinite(total)) {
          bad_all |= kStatusNumeric;
          s_ctl[1] = 1;  // every lane writes the same value
        } else {
          const double y = __dsub_rn(xs, vsel > 0 ? s_incl[vsel - 1] : 0.0);
          const unsigned km = s_kmask[vsel];
          const bool pos = lane < 12 && ((km >> lane) & 1u);
          const unsigned hit = __ballot_sync(0xffffffffu, pos && s_cum[vsel * 12 + (lane < 12 ? lane : 0)] >= y);
          const int sel = hit ? __ffs(hit) - 1 : 31 - __clz(km);
          const int e = vsel * 12 + sel;
          const long long p_old = s_pos[vsel];
          const long long tgt = s_tgt[e];
          const int8_t mig = s_tsp[e];  // the migrating atom's species
          double ea_sel, de_sel;
          if constexpr (kF32) {
            // rates carry the 2^64 scale: dt = -log(u1) 2^64 / (total x prefactor)
            ea_sel = FloatToDouble(reinterpret_cast<const float *>(s_ea)[e]);
            const long long de_fix = reinterpret_cast<const long long *>(s_de)[e];
            energy_fix += de_fix;
            de_sel = static_cast<double>(de_fix) * t.de_scale;  // the trace only
            time += nlog_u1 * RcpFast(total * (kPrefactor / kMultiRateScale));
          } else {
            ea_sel = s_ea[e];
            de_sel = s_de[e];
            time += nlog_u1 * RcpFast(total * kPrefactor);
            energy += de_sel;
          }
          const H3 h_old = s_h[vsel];
          const H3 h_new = SiteCoord(tgt, n);
          __syncwarp();
          if (lane == 0) {
            lat[p_old] = mig;  // Config::LatticeJump
            lat[tgt] = static_cast<int8_t>(x_code);
            s_pos[vsel] = tgt;
            s_h[vsel] = h_new;
            if (r == a.trace_replica && a.trace) {
              KmcTraceRec rec;
              rec.vacancy = p_old;
              rec.target = tgt;
              rec.selected = sel;
              rec.slot = vsel;
              rec.ea = ea_sel;
              rec.de = de_sel;
              rec.total_rate = kF32 ? total / kMultiRateScale : total;
              rec.time = time;
              rec.energy = kF32 ? energy + static_cast<double>(energy_fix) * t.de_scale : energy;
              a.trace[it] = rec;
            }
          }
          // slots to re-evaluate: the moved one and those whose neighbourhood holds a changed site
          int nd2 = 0;
          for (int c = 0; c < chunks; ++c) {
            const int v = c * 32 + lane;
            bool d = false;
            if (v < nv) {
              const H3 hv = v == vsel ? h_new : s_h[v];
              d = v == vsel ||
                  InLocal(s_bits, WrapDelta(h_old.x - hv.x, n), WrapDelta(h_old.y - hv.y, n),
                          WrapDelta(h_old.z - hv.z, n)) ||
                  InLocal(s_bits, WrapDelta(h_new.x - hv.x, n), WrapDelta(h_new.y - hv.y, n),
                          WrapDelta(h_new.z - hv.z, n));
            }
            const unsigned m = __ballot_sync(0xffffffffu, d);
            if (d) s_list[nd2 + __popc(m & ((1u << lane) - 1u))] = v;
            nd2 += __popc(m);
          }
          if (lane == 0) s_ctl[0] = nd2;
        }
      }
    }
    __syncthreads();
    if (s_ctl[1]) {
      if (warp == 0 && !(bad_all & kStatusNumeric)) bad_all |= kStatusStopped;
      break;
    }
    ++steps_done;
  }
  if (warp == 0 && lane == 0) {
    a.time[r] = time;
    a.energy[r] = kF32 ? energy + static_cast<double>(energy_fix) * t.de_scale : energy;
    a.steps[r] = step0 + steps_done;
  }
  for (int i = threadIdx.x; i < nv; i += blockDim.x) a.vac_pos[v0 + i] = s_pos[i];
  bad_all = __reduce_or_sync(0xffffffffu, bad_all);
  if (bad_all && lane == 0) atomicOr(a.status, static_cast<int>(bad_all));
}

// ---------------------------------------------------------------------------
// K4s: surrogate-assisted multi-vacancy KMC of one lattice in one persistent CTA
// (kmc_surrogate_kernel): the step loop of kmc_multi_kernel with the barriers of the
// re-evaluated jumps taken from the compact ensemble on the tensor cores. The ensemble's
// weights are loaded into shared memory once per run and TMEM is allocated once; per step:
//  A. the listed jumps (12 per slot whose neighbourhood changed), 128 per tile: threads
//     0-255 gather the feature rows from the lattice (two threads per row), thread 0 issues
//     both members' layer-1 MMAs, the 16 warps turn D into H1 (GELU, packed half, tcgen05.st),
//     thread 0 issues layer 2 (A = H1 in TMEM), the warps fold GELU . w3 per column half and
//     member, warps 0-3 form each row's ensemble mean and spread (fused::* in mlp_fused.cuh);
//  B. the rows whose ensemble spread exceeds the threshold (or that the network does not
//     describe) by the plain predictor, the whole block per row (BlockPairBarrier);
//  C. per listed slot (one warp): rates, id order and inclusive scan, as kmc_multi_kernel;
//  D. warp 0 selects among all slots exactly as kmc_multi_kernel (Philox draw of counter =
//     step), the block evaluates the plain predictor's energy change of the selected jump
//     (before the move: the energy sums stay exact), warp 0 moves the vacancy and lists the
//     slots whose neighbourhood holds a changed site with their 12 jumps.
// With threshold 0 every jump takes the plain predictor and the trajectory is
// kmc_multi_kernel's. Phases are separated by __syncthreads; the MMA completions are
// mbarrier waits with a 2 s bound, after which the kernel records a status, drains its
// MMAs and copies, frees TMEM and returns.
// ---------------------------------------------------------------------------
// The plain predictor's barrier and energy change of jump a -> b on the current lattice,
// evaluated by the whole block: the sorted arrays gathered into shared memory, the cluster sums
// split over all threads (int64 sums, independent of their order: the same bits as one warp's),
// the FP64 epilogue by thread 0 into out[0] (barrier) and out[1] (energy change). With full =
// false only the energy change (state clusters; out[0] is NaN). Called by every thread of the
// block (it holds block-wide barriers); returns the status bits (thread 0).
__device__ unsigned BlockPairBarrier(const DevTables &t, const int8_t *lat, int n, long long a, long long b, int kind,
                                     bool full, const SmallTables *small, int8_t *st, int8_t *rm, int8_t *rf,
                                     int8_t *rb, long long *red, unsigned *red_bad, double *out) {
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, warps = blockDim.x >> 5;
  H3 hi, hj;
  int di = -1, db = -1;
  unsigned bad = ResolvePair(t.dir_of, a, b, n, &hi, &hj, &di, &db);  // block-uniform
  if (!bad) {
    for (int k = tid; k < kStateSites; k += blockDim.x) {
      const int8_t *o = t.state_off + (di * kStateSites + k) * 4;
      st[k] = lat[NeighborId(hi, o[0], o[1], o[2], n)];
    }
    for (int k = tid; full && k < kEnvSites; k += blockDim.x) {
      const int8_t *oa = t.mmm_off + (di * kEnvSites + k) * 4;
      const int8_t *ob = t.mm2_off + (di * kEnvSites + k) * 4;
      const int8_t *oc = t.mm2_off + (db * kEnvSites + k) * 4;
      rm[k] = small->rank[lat[NeighborId(hi, oa[0], oa[1], oa[2], n)]];
      rf[k] = small->rank[lat[NeighborId(hi, ob[0], ob[1], ob[2], n)]];
      rb[k] = small->rank[lat[NeighborId(hj, oc[0], oc[1], oc[2], n)]];
    }
  }
  __syncthreads();
  int slot = -1;
  if (!bad && full) {
    slot = small->slot[st[t.pos_second]];
    if (slot < 0 || (kind == 0 ? !small->has_quartic[slot] : !small->has_e0[slot])) bad = kStatusNoCoefficients;
  }
  if (!bad) {
    JumpAcc acc{0, 0, 0, 0u};
    if (!full)
      AccumulateDe(t, st, t.de_cl, tid, blockDim.x, &acc);
    else if (kind == 0)
      acc = EvalJump<true>(t, slot, st, rm, rf, rb, t.de_cl, t.mmm_cl, t.mm2_cl, small->pairtype, tid, blockDim.x);
    else
      acc = EvalJump<false>(t, slot, st, rm, rf, rb, t.de_cl, t.mmm_cl, t.mm2_cl, small->pairtype, tid, blockDim.x);
    const long long s_de = WarpSum(acc.de), s_d = WarpSum(acc.d), s_ks = WarpSum(acc.ks);
    const unsigned s_bad = __reduce_or_sync(0xffffffffu, acc.bad);
    if (lane == 0) {
      red[3 * warp] = s_de;
      red[3 * warp + 1] = s_d;
      red[3 * warp + 2] = s_ks;
      red_bad[warp] = s_bad;
    }
  }
  __syncthreads();
  if (tid == 0) {
    if (bad) {
      out[0] = nan("");
      out[1] = nan("");
    } else {
      long long acc_de = 0, acc_d = 0, acc_ks = 0;
      for (int w = 0; w < warps; ++w) {
        acc_de += red[3 * w];
        acc_d += red[3 * w + 1];
        acc_ks += red[3 * w + 2];
        bad |= red_bad[w];
      }
      if (full) {
        const JumpOut o = JumpEpilogue(t, ExpConsts{t.exp_tab, t.exp_l1, t.exp_l2}, kind, slot, acc_de, acc_d, acc_ks);
        out[0] = o.ea;
        out[1] = o.de;
        if (!isfinite(o.ea)) bad |= kStatusNumeric;
      } else {
        out[0] = nan("");
        out[1] = static_cast<double>(acc_de) * t.de_scale;  // as JumpEpilogue
      }
    }
  }
  __syncthreads();
  return bad;
}

constexpr int kSurWarps = 16;

struct SurShared {
  uint64_t w_full, mma, done;
  int abort, halt, rows, nfb;
  uint32_t tmem;
  uint32_t site_word[8];
  int8_t chan[8];
  uint32_t flag[4][4];                 // per row part and lane group: bit l, row 32 lg + l takes the plain predictor
  H3 h[kMaxMultiVac];                  // coordinates of each slot's vacancy
  float partial[2][fused::kMembers][fused::kRows];  // per column half and member: GELU . w3 of each row
  SmallTables small;
  int8_t arr[kArr];                    // the block's sorted arrays (BlockPairBarrier)
  uint32_t bits[kLocalBitWords];
  double incl[kMaxMultiVac];
  long long red[3 * kSurWarps];
  unsigned red_bad[kSurWarps];
  double out[2];
  long long sel[2];                    // the selected jump
  int sel_e, sel_v;
  double sel_total, sel_nlog;
  int16_t fb[kMaxMultiVac * 12];       // listed rows that take the plain predictor
};

template <int kC>
constexpr size_t SurrogateSmemBytes() {
  return static_cast<size_t>(fused::Shape<kC>::kW1Bytes) + fused::kW2Bytes + fused::Shape<kC>::kXBytes +
         sizeof(SurShared);
}
static_assert(SurrogateSmemBytes<3>() <= 232448, "the surrogate KMC kernel's shared memory exceeds 227 KB");

// Bounded wait by lane 0 (sleeping probes), its outcome broadcast to the warp.
__device__ __forceinline__ bool SurWarpWait(uint64_t *bar, uint32_t parity, volatile int *abort, int lane) {
  int ok = 1;
  if (lane == 0) ok = tc::WaitSleep(bar, parity, abort) ? 1 : 0;
  return __shfl_sync(0xffffffffu, ok, 0) != 0;
}

template <int kC>
__global__ void __launch_bounds__(kSurWarps * 32, 1)
    kmc_surrogate_kernel(const __grid_constant__ DevTables t, int8_t *species, const __grid_constant__ KmcSurrogateArgs a,
                         const __grid_constant__ MlpDev d, const __grid_constant__ FusedJumps j) {
  using S = fused::Shape<kC>;
  extern __shared__ __align__(1024) unsigned char smem[];
  unsigned char *sw1 = smem, *sw2 = sw1 + S::kW1Bytes, *sx = sw2 + fused::kW2Bytes;
  SurShared *sh = reinterpret_cast<SurShared *>(sx + S::kXBytes);
  volatile int *abort = &sh->abort;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int n = a.n, nv = a.nv;
  int8_t *lat = species + a.lat_off;
  const int x_code = t.x_code;
  const double beta = 1.0 / kBoltzmannEv / a.temperature;
  const ExpConsts ec{t.exp_tab, t.exp_l1, t.exp_l2};
  int8_t *st = sh->arr, *rm = st + kStateSites, *rf = rm + kEnvSites, *rb = rf + kEnvSites;
  constexpr unsigned kVacancyBits = kStatusXInEnv | kStatusBadCluster;  // a second vacancy contributes nothing

  if (tid == 0) {
    tc::BarInit(&sh->w_full, 1);
    tc::BarInit(&sh->mma, 1);
    tc::BarInit(&sh->done, 1);
    sh->abort = 0;
    sh->halt = 0;
    sh->rows = nv * 12;
    tc::FenceBarrierInit();
    tc::ArriveExpectTx(&sh->w_full, S::kW1Bytes + fused::kW2Bytes);
    tc::BulkCopy(sw1, d.w1_tiles, S::kW1Bytes, &sh->w_full);
    tc::BulkCopy(sw2, d.w2_tiles, fused::kW2Bytes, &sh->w_full);
  }
  if (tid < 8) {
    sh->site_word[tid] = j.site_word[tid];
    sh->chan[tid] = j.chan[tid];
  }
  StageSmall(t, &sh->small);
  for (int i = tid; i < kLocalBitWords; i += blockDim.x) sh->bits[i] = a.local_bits[i];
  // every slot listed at the start of the run, 12 jumps each in direction order
  for (int i = tid; i < nv * 12; i += blockDim.x) {
    const int v = i / 12, dd = i % 12;
    const long long pos = a.vac_pos[v];
    const H3 hv = SiteCoord(pos, n);
    const int8_t *o = t.dir + dd * 4;
    a.pairs[2 * i] = pos;
    a.pairs[2 * i + 1] = NeighborId(hv, o[0], o[1], o[2], n);
    if (dd == 0) {
      a.dirty[v] = v;
      sh->h[v] = hv;
    }
  }
  if (warp == 0) tc::TmemAlloc(&sh->tmem, fused::kCols);
  tc::FenceBeforeSync();
  __syncthreads();
  tc::FenceAfterSync();
  const uint32_t tmem = sh->tmem;
  const uint32_t a_x = tc::Smem(sx), a_w1 = tc::Smem(sw1), a_w2 = tc::Smem(sw2);
  // epilogue split: lane group (TMEM lanes 32 lg ..), member, column half
  const int lg = warp & 3, em = (warp >> 2) & 1, hh = warp >> 3;
  const uint32_t ecol = tmem + (static_cast<uint32_t>(lg * 32) << 16) + em * fused::kMemberCols;
  uint32_t mma_phase = 0;
  bool weights = false;
  unsigned bad_all = 0;
  unsigned long long nfb_total = 0;
  const unsigned long long step0 = *a.steps;
  // Philox draws for 32 steps at a time (warp 0): lane l holds -log(u1) and u2 of step (it & ~31) + l
  double nlog_blk = 0.0, u2_blk = 0.0;
  for (unsigned long long it = 0; it < a.nsteps; ++it) {
    const int rows = sh->rows;
    // ---- A: the network on the listed rows, 128 per tile ----
    for (int t0 = 0; t0 < rows; t0 += fused::kRows) {
      {
        // four threads per row: part = tid / 128 takes sites [16 part, 16 part + 16)
        const int part = tid >> 7, r = tid & 127, row = t0 + r;
        int code[16];
        bool fb = true;
        if (row < rows) {
          unsigned b = 0;
          fb = fused::LoadRowPart<4, false>(j, a.pairs[2 * row], a.pairs[2 * row + 1], part, code, &b);
          bad_all |= b;
        }
        if (fb) {
#pragma unroll
          for (int k = 0; k < 16; ++k) code[k] = -1;
        }
        fused::WriteRowPart<kC, 4>(code, sh->site_word, sh->chan, part, r, sx);
        const unsigned m = __ballot_sync(0xffffffffu, fb);
        if (lane == 0) sh->flag[part][(tid >> 5) & 3] = m;
        tc::FenceAsyncSmem();
      }
      __syncthreads();
      if (tid == 0) {
        if (!weights) weights = tc::WaitSleep(&sh->w_full, 0, abort);
        if (weights) {
          tc::FenceAfterSync();
          fused::IssueLayer1<kC>(tmem, a_x, a_w1, 0);
          fused::IssueLayer1<kC>(tmem, a_x, a_w1, 1);
          tc::Commit(&sh->mma);
        }
      }
      SurWarpWait(&sh->mma, mma_phase, abort, lane);
      mma_phase ^= 1;
      __syncthreads();
      if (*abort) break;
      tc::FenceAfterSync();
      // lane groups past the tile's last listed row hold no rows: their warps skip the epilogues
      const bool rows_here = lg * 32 < rows - t0;
      if (rows_here) {
        fused::Layer1Epilogue(ecol, hh * 64);
        fused::Layer1Epilogue(ecol, hh * 64 + 32);
      }
      tc::FenceBeforeSync();
      __syncthreads();
      if (tid == 0) {
        tc::FenceAfterSync();
        fused::IssueLayer2(tmem, a_w2, 0);
        fused::IssueLayer2(tmem, a_w2, 1);
        tc::Commit(&sh->mma);
      }
      SurWarpWait(&sh->mma, mma_phase, abort, lane);
      mma_phase ^= 1;
      __syncthreads();
      if (*abort) break;
      tc::FenceAfterSync();
      if (rows_here) {
        float v[32];
        float acc = 0.f;
#pragma unroll 1
        for (int cb = 0; cb < 2; ++cb) {
          const int col0 = hh * 64 + cb * 32;
          tc::TmemLoad32(ecol + col0, v);
          acc += fused::GeluDotHalf(v, d.b2h + em * fused::kHid + col0, d.w3h + em * fused::kHid + col0);
        }
        sh->partial[hh][em][lg * 32 + lane] = acc;
      }
      tc::FenceBeforeSync();
      __syncthreads();
      if (warp < 4) {
        const int r = warp * 32 + lane, row = t0 + r;
        if (row < rows) {
          const float y0 = sh->partial[0][0][r] + sh->partial[1][0][r] + __ldg(&d.b3[0]);
          const float y1 = sh->partial[0][1][r] + sh->partial[1][1][r] + __ldg(&d.b3[1]);
          const bool fb = (((sh->flag[0][warp] | sh->flag[1][warp] | sh->flag[2][warp] | sh->flag[3][warp]) >> lane) &
                           1u) != 0;
          a.mean[row] = j.mean_label + j.std_label * 0.5f * (y0 + y1);
          a.spread[row] = fb ? __int_as_float(0x7f800000) : j.std_label * fabsf(y0 - y1);
        }
      }
      __syncthreads();
    }
    if (*abort) break;
    // ---- B: the listed rows whose barrier the network does not give, by the plain predictor ----
    if (tid == 0) sh->nfb = 0;
    __syncthreads();
    const int listed = rows / 12;
    for (int q = warp; q < listed; q += kSurWarps) {
      const int row = q * 12 + lane;
      bool need = false;
      if (lane < 12) {
        const long long id = a.pairs[2 * row + 1];
        const float mu = a.mean[row], sp = a.spread[row];
        need = lat[id] != x_code && !(sp <= a.threshold && isfinite(mu));
      }
      const unsigned m = __ballot_sync(0xffffffffu, need);
      int base = 0;
      if (lane == 0 && m) base = atomicAdd(&sh->nfb, __popc(m));
      base = __shfl_sync(0xffffffffu, base, 0);
      if (need) sh->fb[base + __popc(m & ((1u << lane) - 1u))] = static_cast<int16_t>(row);
    }
    __syncthreads();
    const int nfb = sh->nfb;
    for (int i = 0; i < nfb; ++i) {
      const int row = sh->fb[i];
      const unsigned b = BlockPairBarrier(t, lat, n, a.pairs[2 * row], a.pairs[2 * row + 1], a.barrier_kind, true,
                                          &sh->small, st, rm, rf, rb, sh->red, sh->red_bad, sh->out);
      if (tid == 0) {
        bad_all |= b & ~kVacancyBits;
        a.pair_ea[row] = sh->out[0];
      }
    }
    if (tid == 0) nfb_total += nfb;
    __syncthreads();
    // ---- C: the listed slots' rates, id order and scan (one warp per slot) ----
    for (int q = warp; q < listed; q += kSurWarps) {
      const int v = a.dirty[q];
      const int row = q * 12 + (lane < 12 ? lane : 0);
      long long id = 0x7fffffffffffffffLL;
      double ea = 0.0, k = 0.0;
      if (lane < 12) {
        id = a.pairs[2 * row + 1];
        if (lat[id] != x_code) {
          const float mu = a.mean[row], sp = a.spread[row];
          ea = (sp <= a.threshold && isfinite(mu)) ? static_cast<double>(mu) : a.pair_ea[row];
          k = ExpFast(-ea * beta, ec);
        }
      }
      // events in id order (the sorted 1NN list), then their inclusive scan
      int rank = 0;
      for (int q2 = 0; q2 < 12; ++q2) {
        const long long oid = __shfl_sync(0xffffffffu, id, q2);
        rank += (q2 != lane) && (oid < id);
      }
      int src = 0;
      for (int q2 = 0; q2 < 12; ++q2)
        if (__shfl_sync(0xffffffffu, rank, q2) == lane) src = q2;
      const double k_s = __shfl_sync(0xffffffffu, k, src);
      const double ea_s = __shfl_sync(0xffffffffu, ea, src);
      const long long id_s = __shfl_sync(0xffffffffu, id, src);
      double cum = lane < 12 ? k_s : 0.0;
#pragma unroll
      for (int o = 1; o < 16; o <<= 1) {
        const double u = __shfl_up_sync(0xffffffffu, cum, o);
        if (lane >= o) cum += u;
      }
      const unsigned kpos = __ballot_sync(0xffffffffu, lane < 12 && k_s > 0.0);
      if (lane < 12) {
        a.cum[v * 12 + lane] = cum;
        a.ea[v * 12 + lane] = ea_s;
        a.tgt[v * 12 + lane] = id_s;
      }
      if (lane == 0) a.kmask[v] = kpos;
      __syncwarp();
    }
    __syncthreads();
    // ---- D: selection (warp 0) ----
    const unsigned long long step = step0 + it;
    if (warp == 0) {
      bool halt = false;
      if (a.stop_flag && (step & 63) == 0 && *a.stop_flag) {
        bad_all |= kStatusStopped;
        halt = true;
      }
      if (!halt) {
        if ((it & 31) == 0) {
          const unsigned long long ctr = step + lane;
          const uint4 xr = PhiloxRound10(static_cast<uint32_t>(ctr), static_cast<uint32_t>(ctr >> 32),
                                         static_cast<uint32_t>(a.replica), 0x4b4d43u, a.key0, a.key1);
          nlog_blk = -log(U01Open(xr.x, xr.y));
          u2_blk = U01(xr.z, xr.w);
        }
        const double nlog_u1 = __shfl_sync(0xffffffffu, nlog_blk, static_cast<int>(it & 31));
        const double u2 = __shfl_sync(0xffffffffu, u2_blk, static_cast<int>(it & 31));
        const int chunks = (nv + 31) >> 5;
        double run = 0.0;
        for (int c = 0; c < chunks; ++c) {
          const int v = c * 32 + lane;
          double sc = v < nv ? a.cum[v * 12 + 11] : 0.0;
#pragma unroll
          for (int o = 1; o < 32; o <<= 1) {
            const double u = __shfl_up_sync(0xffffffffu, sc, o);
            if (lane >= o) sc += u;
          }
          if (v < nv) sh->incl[v] = run + sc;
          run = run + __shfl_sync(0xffffffffu, sc, 31);
        }
        const double total = run;
        __syncwarp();
        const double xs = __dmul_rn(u2, total);  // not contracted with the subtraction below
        int vsel = -1, vlast = -1;
        for (int c = 0; c < chunks; ++c) {
          const int v = c * 32 + lane;
          const bool pos = v < nv && a.kmask[v] != 0;
          const unsigned hit = __ballot_sync(0xffffffffu, pos && sh->incl[v] >= xs);
          const unsigned any = __ballot_sync(0xffffffffu, pos);
          if (vsel < 0 && hit) vsel = c * 32 + __ffs(hit) - 1;
          if (any) vlast = c * 32 + 31 - __clz(any);
        }
        if (vsel < 0) vsel = vlast;
        if (vsel < 0 || !(total > 0.0) || !isfinite(total)) {
          bad_all |= kStatusNumeric;
          halt = true;
        } else {
          const double y = __dsub_rn(xs, vsel > 0 ? sh->incl[vsel - 1] : 0.0);
          const unsigned km = a.kmask[vsel];
          const bool pos = lane < 12 && ((km >> lane) & 1u);
          const unsigned hit = __ballot_sync(0xffffffffu, pos && a.cum[vsel * 12 + (lane < 12 ? lane : 0)] >= y);
          const int sel = hit ? __ffs(hit) - 1 : 31 - __clz(km);
          if (lane == 0) {
            sh->sel_e = vsel * 12 + sel;
            sh->sel_v = vsel;
            sh->sel[0] = a.vac_pos[vsel];
            sh->sel[1] = a.tgt[vsel * 12 + sel];
            sh->sel_total = total;
            sh->sel_nlog = nlog_u1;
          }
        }
      }
      if (lane == 0) sh->halt = halt ? 1 : 0;
    }
    __syncthreads();
    if (sh->halt) break;
    // ---- D: the plain predictor's energy change of the selected jump (before the move) ----
    const long long p_old = sh->sel[0], tgt = sh->sel[1];
    // the energy change alone, unless the run records the plain barrier of each selected event
    const unsigned b = BlockPairBarrier(t, lat, n, p_old, tgt, a.barrier_kind, a.plain_ea != nullptr, &sh->small, st,
                                        rm, rf, rb, sh->red, sh->red_bad, sh->out);
    if (tid == 0) bad_all |= b & ~kVacancyBits;
    // ---- D: the move and the next list (warp 0) ----
    if (warp == 0) {
      const int vsel = sh->sel_v, e = sh->sel_e;
      const double ea_plain = sh->out[0], de_sel = sh->out[1];
      const double time = *a.time + sh->sel_nlog * RcpFast(sh->sel_total * kPrefactor);
      const double energy = *a.energy + de_sel;
      const H3 h_old = sh->h[vsel], h_new = SiteCoord(tgt, n);
      if (lane == 0) {
        lat[p_old] = lat[tgt];  // Config::LatticeJump
        lat[tgt] = static_cast<int8_t>(x_code);
        a.vac_pos[vsel] = tgt;
        sh->h[vsel] = h_new;
        *a.time = time;
        *a.energy = energy;
        *a.steps = step + 1;
        const unsigned long long ti = step - a.trace_base;
        if (a.trace && ti < a.trace_len) {
          KmcTraceRec rec;
          rec.vacancy = p_old;
          rec.target = tgt;
          rec.selected = e - vsel * 12;
          rec.slot = vsel;
          rec.ea = a.ea[e];
          rec.de = de_sel;
          rec.total_rate = sh->sel_total;
          rec.time = time;
          rec.energy = energy;
          a.trace[ti] = rec;
          if (a.plain_ea) a.plain_ea[ti] = ea_plain;
        }
      }
      __syncwarp();
      // slots to re-evaluate: the moved one and those whose neighbourhood holds a changed
      // site, with their 12 jumps in direction order for the next step's network
      const int chunks = (nv + 31) >> 5;
      int nd2 = 0;
      for (int c = 0; c < chunks; ++c) {
        const int v = c * 32 + lane;
        bool dv = false;
        if (v < nv) {
          const H3 hv = v == vsel ? h_new : sh->h[v];
          dv = v == vsel ||
               InLocal(sh->bits, WrapDelta(h_old.x - hv.x, n), WrapDelta(h_old.y - hv.y, n),
                       WrapDelta(h_old.z - hv.z, n)) ||
               InLocal(sh->bits, WrapDelta(h_new.x - hv.x, n), WrapDelta(h_new.y - hv.y, n),
                       WrapDelta(h_new.z - hv.z, n));
        }
        const unsigned m = __ballot_sync(0xffffffffu, dv);
        if (dv) a.dirty[nd2 + __popc(m & ((1u << lane) - 1u))] = v;
        nd2 += __popc(m);
      }
      __syncwarp();
      for (int i = 0; i < nd2; ++i) {
        const int v = a.dirty[i];
        if (lane < 12) {
          const long long pv = v == vsel ? tgt : a.vac_pos[v];
          const int8_t *o = t.dir + lane * 4;
          a.pairs[2 * (i * 12 + lane)] = pv;
          a.pairs[2 * (i * 12 + lane) + 1] = NeighborId(v == vsel ? h_new : sh->h[v], o[0], o[1], o[2], n);
        }
      }
      if (lane == 0) sh->rows = nd2 * 12;
    }
    __syncthreads();
  }
  // drain: every MMA issued has completed when `done` does; the weight copies have landed
  if (tid == 0) {
    tc::Commit(&sh->done);
    if (!tc::WaitDrain(&sh->done, 0)) *abort = 1;
    if (!weights && !tc::WaitDrain(&sh->w_full, 0)) *abort = 1;
  }
  __syncthreads();
  const unsigned bad = __reduce_or_sync(0xffffffffu, bad_all);
  if (lane == 0 && bad) atomicOr(a.status, static_cast<int>(bad));
  if (tid == 0) {
    if (nfb_total) atomicAdd(a.fallbacks, nfb_total);
    if (*abort) atomicOr(a.net_status, 1);
    if (sh->halt || *abort) *a.halt = 1;
  }
  tc::FenceBeforeSync();
  __syncthreads();
  if (warp == 0) tc::TmemFree(tmem, fused::kCols);
}

constexpr int kCmcRefMaxBatch = 256;
// The reference's mt19937_64 stream read by a whole warp: the current block of
// 312 raw state words and the next one (twisted ahead, warp-parallel) sit in
// shared memory, so any lane can read any of the next 312 or more outputs;
// positions are consumed in order, as the serial generator would. Every lane
// holds the same copy of this struct (warp-uniform calls only).
struct MtWarp {
  unsigned long long *cur, *nxt;  // raw words of the current and the following block
  unsigned idx;                   // next unread position in cur (0..311)
};
// dst = the block after src (the serial in-place twist, split into its two
// dependency-free halves: words 0-155 read only src, words 156-311 read dst 0-155).
__device__ __forceinline__ void MtTwistWarp(const unsigned long long *src, unsigned long long *dst, int lane) {
  constexpr unsigned long long kUpper = 0xFFFFFFFF80000000ULL, kLower = 0x7FFFFFFFULL;
  constexpr unsigned long long kA = 0xB5026F5AA96619E9ULL;
  for (int k = lane; k < 156; k += 32) {
    const unsigned long long x = (src[k] & kUpper) | (src[k + 1] & kLower);
    dst[k] = src[k + 156] ^ (x >> 1) ^ ((x & 1ULL) ? kA : 0ULL);
  }
  __syncwarp();
  for (int k = 156 + lane; k < 312; k += 32) {
    const unsigned long long x = (src[k] & kUpper) | ((k + 1 < 312 ? src[k + 1] : dst[0]) & kLower);
    dst[k] = dst[k - 156] ^ (x >> 1) ^ ((x & 1ULL) ? kA : 0ULL);
  }
  __syncwarp();
}
__device__ __forceinline__ unsigned long long MtWarpOut(const MtWarp &w, unsigned p) {
  const unsigned q = w.idx + p;  // p < 312
  return MtTemperOut(q < 312 ? w.cur[q] : w.nxt[q - 312]);
}
__device__ __forceinline__ void MtWarpAdvance(MtWarp &w, unsigned count, int lane) {
  w.idx += count;  // count <= 312
  if (w.idx >= 312) {
    unsigned long long *tmp = w.cur;
    w.cur = w.nxt;
    w.nxt = tmp;
    w.idx -= 312;
    __syncwarp();
    MtTwistWarp(w.cur, w.nxt, lane);
  }
}
// uniform_int_distribution<size_t>(0, range - 1), one draw at a time (Lemire's rejection).
__device__ __forceinline__ unsigned long long MtWarpBelow(MtWarp &w, unsigned long long range, int lane) {
  unsigned long long x = MtWarpOut(w, 0);
  MtWarpAdvance(w, 1, lane);
  unsigned long long low = x * range;
  if (low < range) {
    const unsigned long long threshold = (0ULL - range) % range;
    while (low < threshold) {
      x = MtWarpOut(w, 0);
      MtWarpAdvance(w, 1, lane);
      low = x * range;
    }
  }
  return __umul64hi(x, range);
}
// GenerateLatticeIdJumpPair on the stream: pairs of draws until the species differ.
// The 32 lanes test the next 32 candidate pairs (64 draws) at once; the first
// different-species candidate wins and exactly its draws and those before it are
// consumed. A draw that Lemire's method would reject (probability below range / 2^64)
// shifts the pairing, so from the first such candidate on the draws are taken one by one.
// `threshold` = (2^64 - range) mod range, Lemire's rejection bound (hoisted out of the loops).
__device__ __forceinline__ bool MtWarpPair(MtWarp &w, const int8_t *species, unsigned long long range,
                                           unsigned long long threshold, int lane, long long *l1, long long *l2) {
  for (unsigned round = 0; round < (1u << 19); ++round) {
    const unsigned long long x1 = MtWarpOut(w, 2 * lane), x2 = MtWarpOut(w, 2 * lane + 1);
    const bool rej = x1 * range < threshold || x2 * range < threshold;
    const long long a = static_cast<long long>(__umul64hi(x1, range)), b = static_cast<long long>(__umul64hi(x2, range));
    const bool diff = species[a] != species[b];
    const unsigned mrej = __ballot_sync(0xffffffffu, rej);
    const int r0 = mrej ? __ffs(mrej) - 1 : 32;
    const unsigned mdiff = __ballot_sync(0xffffffffu, diff) & (r0 == 32 ? 0xffffffffu : (1u << r0) - 1u);
    if (mdiff) {
      const int g = __ffs(mdiff) - 1;
      *l1 = __shfl_sync(0xffffffffu, a, g);
      *l2 = __shfl_sync(0xffffffffu, b, g);
      MtWarpAdvance(w, 2 * (g + 1), lane);
      return true;
    }
    if (r0 < 32) {
      MtWarpAdvance(w, 2 * r0, lane);
      const long long c1 = static_cast<long long>(MtWarpBelow(w, range, lane));
      const long long c2 = static_cast<long long>(MtWarpBelow(w, range, lane));
      if (species[c1] != species[c2]) {
        *l1 = c1;
        *l2 = c2;
        return true;
      }
      continue;
    }
    MtWarpAdvance(w, 64, lane);
  }
  return false;
}

// ---------------------------------------------------------------------------
// K5a: CanonicalMcOmp (CanonicalMcOmp.cpp:40-92, CanonicalMcAbstract.cpp:43-101)
// in its exact order, one block. Warp 0 reads the mt19937_64 stream as a warp and
// builds the batch: each pair is redrawn until both sites lie outside the 1-3NN
// shells (site included) of the sites already chosen, the batch given up after 50
// tries. The shells are not marked on a lattice-sized array: on an FCC supercell
// with n >= 6 a site lies in the shell of c exactly when its minimum-image
// displacement from c has squared length <= 6 (half units: 1NN 2, 2NN 4, 3NN 6,
// 4NN 8), so the lanes test the candidates' coordinates against each other and
// against the chosen sites directly.
// The block's warps then compute the batch's dE values on the unchanged lattice,
// one pair per warp, as the reference's OpenMP threads do; warp 0 runs the
// Metropolis tests of up to 32 pairs at once (a pair's uniform is the stream's
// output after those of the earlier pairs with dE >= 0, its factor exp(-dE / kT)
// one lane's FP64 exp) and sums the energy in batch order.
// ---------------------------------------------------------------------------
constexpr int kCmcRefWarps = 16;
// Lattices up to this many sites are copied into shared memory for the launch.
constexpr long long kCmcRefSmemSites = 192 * 1024;
__device__ __forceinline__ bool CmcRefNear(H3 a, H3 b, int n) {
  const int dx = WrapDelta(a.x - b.x, n), dy = WrapDelta(a.y - b.y, n), dz = WrapDelta(a.z - b.z, n);
  return dx * dx + dy * dy + dz * dz <= 6;
}
__global__ void __launch_bounds__(kCmcRefWarps * 32, 1) cmc_ref_kernel(DevTables t, int8_t *species_global, CmcRefArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const SiteSmem s = CarveSiteSmem(t, smem);
  __shared__ unsigned long long s_mt[2][312];
  __shared__ long long s_pair[kCmcRefMaxBatch][2];
  __shared__ H3 s_h[2 * kCmcRefMaxBatch];
  __shared__ double s_de[kCmcRefMaxBatch];
  __shared__ int s_nb, s_fail, s_stop;
  // warp 0's set of candidate pairs while it builds a batch
  __shared__ long long s_c1[32], s_c2[32];
  __shared__ unsigned s_cend[32], s_cmask[32];
  __shared__ H3 s_ch[64];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int n = a.n;
  const long long nsites_ll = 4LL * n * n * n;
  const unsigned long long nsites = static_cast<unsigned long long>(nsites_ll);
  const unsigned long long threshold = (0ULL - nsites) % nsites;
  const bool local_lattice = nsites_ll <= kCmcRefSmemSites;
  int8_t *species = species_global;
  if (local_lattice) {
    // after the site tables and the warps' 2 x 44 arrays (the layout SiteSmemBytes(t, kCmcRefWarps) sizes)
    species = reinterpret_cast<int8_t *>((reinterpret_cast<size_t>(s.arr + 88 * kCmcRefWarps) + 15) & ~size_t(15));
    for (long long k = threadIdx.x; k < nsites_ll; k += blockDim.x) species[k] = species_global[k];
  }
  StageArray(t.site_cl, s.cl, t.n_site_cl);
  StageArray(t.site_off, s.off, kSiteSites * 4);
  const unsigned long long *gmt = reinterpret_cast<const unsigned long long *>(a.rng);
  for (int k = threadIdx.x; k < 312; k += blockDim.x) s_mt[0][k] = gmt[k];
  __syncthreads();
  MtWarp mw{s_mt[0], s_mt[1], a.rng[2 * 312]};
  if (warp == 0) {
    if (mw.idx >= 312) {  // the serial generator twists on its next draw
      MtTwistWarp(mw.cur, mw.nxt, lane);
      unsigned long long *tmp = mw.cur;
      mw.cur = mw.nxt;
      mw.nxt = tmp;
      mw.idx = 0;
    }
    MtTwistWarp(mw.cur, mw.nxt, lane);
  }
  int8_t *sa = s.arr + warp * 88, *sb = sa + 44;
  double energy = *a.energy;  // kept by warp 0, every lane the same copy
  unsigned long long done = 0, accepted = 0;
  bool stop = a.attempts == 0;
  while (!stop) {
    if (warp == 0) {
      // The batch: pair slot after pair slot, the stream's different-species pairs in order, each
      // kept when neither site lies in the shells of the pairs kept before, the batch given up at
      // a slot's 50th pair. The different-species pairs are found a set at a time (the 32 lanes
      // test 32 consecutive draw pairs per ballot, up to 32 pairs within the draws readable
      // before the stream advances), tested against each other and the pairs kept before as bit
      // masks, then taken in order; only the draws up to the pair that completes the batch are
      // consumed.
      int nb = 0, ct = 0, empty_sets = 0;
      bool failed = false, ended = false;
      while (nb < a.batch && !failed && !ended) {
        int m = 0;          // pairs found in this set (s_c1 / s_c2 / s_cend [0, m))
        unsigned off = 0;   // draws examined
        bool rejected = false;
        const unsigned window = 624 - mw.idx;  // draws readable before the stream advances
        while (m < 32 && off + 64 <= window) {
          const unsigned long long x1 = MtWarpOut(mw, off + 2 * lane), x2 = MtWarpOut(mw, off + 2 * lane + 1);
          const bool rej = x1 * nsites < threshold || x2 * nsites < threshold;
          const long long pa = static_cast<long long>(__umul64hi(x1, nsites));
          const long long pb = static_cast<long long>(__umul64hi(x2, nsites));
          const bool diff = species[pa] != species[pb];
          const unsigned mrej = __ballot_sync(0xffffffffu, rej);
          const int r0 = mrej ? __ffs(mrej) - 1 : 32;
          const unsigned below = r0 == 32 ? 0xffffffffu : (1u << r0) - 1u;
          const unsigned mdiff = __ballot_sync(0xffffffffu, diff) & below;
          const int rank = m + __popc(mdiff & ((1u << lane) - 1u));
          const bool take = ((mdiff >> lane) & 1u) && rank < 32;
          if (take) {
            s_c1[rank] = pa;
            s_c2[rank] = pb;
            s_cend[rank] = off + 2 * static_cast<unsigned>(lane + 1);
          }
          if (m + __popc(mdiff) >= 32) {  // the set ends at its 32nd pair
            off += 2 * static_cast<unsigned>(__ffs(__ballot_sync(0xffffffffu, take && rank == 31)));
            m = 32;
            break;
          }
          m += __popc(mdiff);
          if (r0 < 32) {  // a draw Lemire's method rejects: the pairing shifts from there
            off += 2 * static_cast<unsigned>(r0);
            rejected = true;
            break;
          }
          off += 64;
        }
        empty_sets = m == 0 ? empty_sets + 1 : 0;
        if (empty_sets > (1 << 15)) {  // no different-species pair in millions of draws
          failed = true;
          break;
        }
        __syncwarp();
        // the set's first mm pairs (enough to fill the batch with 8 rejections to spare): lane j
        // forms pair j's coordinates and whether it lies in the shells of a pair chosen before
        // this set (bit 31); then the lanes test the set's pairs against each other (bit k of
        // word j: pair k < j conflicts with pair j)
        const int mm = min(m, a.batch - nb + 8);
        if (lane < mm) {
          const H3 e1 = SiteCoord(s_c1[lane], n), e2 = SiteCoord(s_c2[lane], n);
          s_ch[2 * lane] = e1;
          s_ch[2 * lane + 1] = e2;
          bool prev = false;
          for (int q = 0; q < 2 * nb; ++q) prev |= CmcRefNear(e1, s_h[q], n) | CmcRefNear(e2, s_h[q], n);
          s_cmask[lane] = prev ? 0x80000000u : 0u;
        }
        __syncwarp();
        const int npairs = mm * (mm - 1) / 2;
        for (int p = lane; p < npairs; p += 32) {
          int j = static_cast<int>((1.0f + sqrtf(1.0f + 8.0f * static_cast<float>(p))) * 0.5f);
          while (j * (j - 1) / 2 > p) --j;
          while ((j + 1) * j / 2 <= p) ++j;
          const int kk = p - j * (j - 1) / 2;
          const H3 a1 = s_ch[2 * j], a2 = s_ch[2 * j + 1], b1 = s_ch[2 * kk], b2 = s_ch[2 * kk + 1];
          if (CmcRefNear(a1, b1, n) | CmcRefNear(a1, b2, n) | CmcRefNear(a2, b1, n) | CmcRefNear(a2, b2, n))
            atomicOr(&s_cmask[j], 1u << kk);
        }
        __syncwarp();
        // the pairs in order (lane 0): a slot's 50th pair ends the batch, a pair clear of the
        // shells of the chosen ones fills the slot
        unsigned chosen = 0;
        int add = 0, jend = -1, ended_i = 0;
        if (lane == 0) {
          for (int j = 0; j < mm; ++j) {
            if (++ct == 50) {
              jend = j;
              ended_i = 1;
              break;
            }
            const unsigned cm = s_cmask[j];
            if (!(cm & 0x80000000u) && !(cm & chosen)) {
              chosen |= 1u << j;
              ct = 0;
              if (nb + ++add == a.batch) {
                jend = j;
                break;
              }
            }
          }
        }
        chosen = __shfl_sync(0xffffffffu, chosen, 0);
        add = __shfl_sync(0xffffffffu, add, 0);
        jend = __shfl_sync(0xffffffffu, jend, 0);
        ct = __shfl_sync(0xffffffffu, ct, 0);
        ended = __shfl_sync(0xffffffffu, ended_i, 0) != 0;
        if (lane < mm && ((chosen >> lane) & 1u)) {
          const int idx = nb + __popc(chosen & ((1u << lane) - 1u));
          s_pair[idx][0] = s_c1[lane];
          s_pair[idx][1] = s_c2[lane];
          s_h[2 * idx] = s_ch[2 * lane];
          s_h[2 * idx + 1] = s_ch[2 * lane + 1];
        }
        nb += add;
        // draws this set consumes: through the pair that ended or completed the batch, else through
        // the last pair examined (all examined slots when every pair of the set was examined)
        const unsigned used = jend >= 0 ? s_cend[jend] : (mm < m ? s_cend[mm - 1] : off);
        __syncwarp();
        MtWarpAdvance(mw, used > 312 ? 312 : used, lane);
        if (used > 312) MtWarpAdvance(mw, used - 312, lane);
        if (rejected && used == off && nb < a.batch && !ended) {
          // the pair at the rejected draw and its successors, one at a time
          long long l1 = 0, l2 = 0;
          if (!MtWarpPair(mw, species, nsites, threshold, lane, &l1, &l2)) {
            failed = true;
            break;
          }
          if (++ct == 50) {
            ended = true;
            break;
          }
          const H3 q1 = SiteCoord(l1, n), q2 = SiteCoord(l2, n);
          bool hit = false;
          for (int q = lane; q < 2 * nb; q += 32) hit |= CmcRefNear(q1, s_h[q], n) || CmcRefNear(q2, s_h[q], n);
          if (!__any_sync(0xffffffffu, hit)) {
            if (lane == 0) {
              s_pair[nb][0] = l1;
              s_pair[nb][1] = l2;
              s_h[2 * nb] = q1;
              s_h[2 * nb + 1] = q2;
            }
            __syncwarp();
            ++nb;
            ct = 0;
          }
        }
      }
      if (lane == 0) {
        s_nb = nb;
        s_fail = failed;
        if (failed) atomicOr(a.status, kStatusNumeric);
      }
    }
    __syncthreads();
    if (s_fail) break;
    const int nb = s_nb;
    for (int i = warp; i < nb; i += kCmcRefWarps) {
      int pa, pb;
      GatherSwap(s.off, species, n, s_h[2 * i], s_h[2 * i + 1], sa, sb, &pa, &pb, lane);
      const long long acc = WarpSum(SwapDePartial(t, s.cl, sa, sb, pa, pb, lane));
      if (lane == 0) s_de[i] = static_cast<double>(acc) * t.de_scale;
    }
    __syncthreads();
    if (warp == 0) {
      // The Metropolis tests of the batch, 32 pairs at a time in parallel: pair i draws a uniform
      // only when dE_i >= 0, so its draw is the stream's next output after those of the earlier
      // pairs with dE >= 0, and its acceptance does not depend on theirs (the dE values are
      // those of the unchanged lattice; the pairs' sites are disjoint). The energy is summed in
      // batch order, as the serial loop does.
      for (int c0 = 0; c0 < nb; c0 += 32) {
        const int i = c0 + lane, m = min(32, nb - c0);
        const bool in = lane < m;
        const double dE = in ? s_de[i] : 0.0;
        const bool need = in && !(dE < 0);
        const unsigned mneed = __ballot_sync(0xffffffffu, need);
        bool acc = in && dE < 0;
        if (need) {  // the Metropolis factors of the 32 pairs in one warp: one FP64 exp per lane
          const unsigned k = static_cast<unsigned>(__popc(mneed & ((1u << lane) - 1u)));
          const double u0 = __ull2double_rn(MtWarpOut(mw, k)) * 5.421010862427522170e-20;  // 2^-64
          acc = (u0 >= 1.0 ? 0.99999999999999988898 : u0) < exp(-dE * a.beta);
        }
        const unsigned macc = __ballot_sync(0xffffffffu, acc);
        if (acc) {
          const long long l1 = s_pair[i][0], l2 = s_pair[i][1];
          const int8_t v = species[l1];
          species[l1] = species[l2];
          species[l2] = v;
        }
        for (int j = 0; j < m; ++j) {
          if (a.energy_trace && lane == 0) a.energy_trace[done + j] = energy;
          if ((macc >> j) & 1u) energy += s_de[c0 + j];
        }
        done += static_cast<unsigned long long>(m);
        accepted += static_cast<unsigned long long>(__popc(macc));
        MtWarpAdvance(mw, static_cast<unsigned>(__popc(mneed)), lane);
      }
      if (nb == 0) done = a.attempts;  // no pair could be placed: stop rather than spin
      if (lane == 0) s_stop = done >= a.attempts;
    }
    __syncthreads();
    stop = s_stop;
  }
  if (threadIdx.x == 0) {
    *a.energy = energy;
    *a.done = done;
    *a.accepted = accepted;
  }
  __syncthreads();
  if (local_lattice)
    for (long long k = threadIdx.x; k < nsites_ll; k += blockDim.x) species_global[k] = species[k];
  if (warp == 0) {
    unsigned long long *gw = reinterpret_cast<unsigned long long *>(a.rng);
    for (int k = lane; k < 312; k += 32) gw[k] = mw.cur[k];
    if (lane == 0) a.rng[2 * 312] = mw.idx;
  }
}

// ---------------------------------------------------------------------------
// K5c: simulated annealing (SimulatedAnnealing.cpp:99-185), one warp. Per step:
// Dump's lowest-energy bookkeeping on the state before the step (:83-97), a
// trial pair redrawn until the species differ (:138-146), its PairSite dE (warp
// cluster sums), Metropolis (:148-167), then UpdateTemperature (:99-137):
// windowed acceptance cool-down, bounded reheats, the baseline exponential decay.
// The same FP64 operations as the reference, with the ones whose result a step may
// not use deferred: 1 / kT is formed when a step draws a uniform (and at the end),
// the acceptance estimate only when the reheat's integer conditions hold, the decay
// factor once per launch (it is the same every step).
// ---------------------------------------------------------------------------
constexpr double kSaEpsilon = 1e-4;  // kEpsilon, lmc/cfg/include/VectorMatrix.hpp:65
// Lattices up to this many sites are copied into shared memory for the launch:
// the trial-pair redraws (one per same-species draw) then read species at
// shared-memory latency instead of L2 latency.
constexpr long long kSaSmemSites = 200 * 1024;
__global__ void sa_kernel(DevTables t, int8_t *species_global, SaArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  const SiteSmem s = CarveSiteSmem(t, smem);
  const long long nsites_ll = 4LL * a.n * a.n * a.n;
  const bool local_lattice = nsites_ll <= kSaSmemSites;
  int8_t *species = species_global;
  if (local_lattice) {
    // after the site tables and one warp's 2 x 44 arrays (the layout SiteSmemBytes(t, 1) sizes)
    species = reinterpret_cast<int8_t *>((reinterpret_cast<size_t>(s.arr + 88) + 15) & ~size_t(15));
    for (long long i = threadIdx.x; i < nsites_ll; i += blockDim.x) species[i] = species_global[i];
  }
  __shared__ unsigned long long s_mt[2][312];
  StageArray(t.site_cl, s.cl, t.n_site_cl);
  StageArray(t.site_off, s.off, kSiteSites * 4);
  const unsigned long long *gmt = reinterpret_cast<const unsigned long long *>(a.rng);
  for (int i = threadIdx.x; i < 312; i += blockDim.x) s_mt[0][i] = gmt[i];
  __syncthreads();
  const int lane = threadIdx.x;
  MtWarp mw{s_mt[0], s_mt[1], a.rng[2 * 312]};
  if (mw.idx >= 312) {  // the serial generator twists on its next draw
    MtTwistWarp(mw.cur, mw.nxt, lane);
    unsigned long long *tmp = mw.cur;
    mw.cur = mw.nxt;
    mw.nxt = tmp;
    mw.idx = 0;
  }
  MtTwistWarp(mw.cur, mw.nxt, lane);  // the following block, ready for reads past the current one
  const int n = a.n;
  const unsigned long long nsites = 4ULL * n * n * n;
  const unsigned long long threshold = (0ULL - nsites) % nsites;
  int8_t *sa = s.arr, *sb = sa + 44;
  SaState st = *a.state;  // every lane keeps the same copy; lane 0 writes memory
  // the baseline decay factor of every step (UpdateTemperature's exp(-3 / maximum_steps))
  const double decay = exp(-3.0 / static_cast<double>(st.maximum_steps > 1ULL ? st.maximum_steps : 1ULL));
  bool beta_fresh = true;  // st.beta belongs to st.temperature
  unsigned bad = 0;
  for (unsigned long long it = 0; it < a.steps; ++it) {
    int stop = 0;
    if (lane == 0) stop = (a.stop_flag && (it & 255) == 0 && *a.stop_flag) ? 1 : 0;
    if (__shfl_sync(0xffffffffu, stop, 0)) {
      bad |= kStatusStopped;
      break;
    }
    // Dump: lowest-energy bookkeeping on the state before this step
    if (st.energy < st.lowest - kSaEpsilon) st.lowest = st.energy;
    long long l1 = 0, l2 = 0;
    if (!MtWarpPair(mw, species, nsites, threshold, lane, &l1, &l2)) {  // the host rejects single-species lattices
      bad |= kStatusNumeric;
      break;
    }
    int pa, pb;
    GatherSwap(s.off, species, n, SiteCoord(l1, n), SiteCoord(l2, n), sa, sb, &pa, &pb, lane);
    const long long acc_fx = WarpSum(SwapDePartial(t, s.cl, sa, sb, pa, pb, lane));
    const double dE = static_cast<double>(acc_fx) * t.de_scale;
    const double e_before = st.energy, t_before = st.temperature;
    bool accepted = dE < 0;
    if (!accepted) {
      // generate_canonical<double, 53>: one draw scaled by 2^-64, 1 rounded down
      const double u0 = __ull2double_rn(MtWarpOut(mw, 0)) * 5.421010862427522170e-20;
      MtWarpAdvance(mw, 1, lane);
      const double u = u0 >= 1.0 ? 0.99999999999999988898 : u0;
      if (!beta_fresh) {
        st.beta = 1.0 / kBoltzmannEv / fmax(st.temperature, 1e-12);
        beta_fresh = true;
      }
      accepted = u < exp(-dE * st.beta);
    }
    __syncwarp();
    if (accepted) {
      if (lane == 0) {
        const int8_t v = species[l1];
        species[l1] = species[l2];
        species[l2] = v;
      }
      st.energy += dE;
    }
    // UpdateTemperature(accepted)
    ++st.window_trials;
    if (accepted) {
      ++st.window_accepts;
      if (st.energy < st.recent_best - kSaEpsilon) {
        st.recent_best = st.energy;
        st.last_improvement = st.steps;
      }
    }
    if (st.window_trials >= st.window_size) {
      const double accr = static_cast<double>(st.window_accepts) / static_cast<double>(st.window_trials);
      if (accr > 0.50) st.temperature *= 0.99;
      st.window_trials = 0;
      st.window_accepts = 0;
    }
    // (the acceptance estimate, an FP64 division, only when the integer conditions hold)
    if (st.reheats_done < 5 && st.steps - st.last_improvement >= st.reheat_trigger &&
        st.steps - st.last_reheat >= st.reheat_cooldown) {
      const double acc_est = st.window_trials > 0u
                                 ? static_cast<double>(st.window_accepts) / static_cast<double>(st.window_trials)
                                 : 1.0;
      if (acc_est < 0.05) {
        st.temperature *= 1.10;
        st.last_improvement = st.steps;
        st.last_reheat = st.steps;
        st.recent_best = st.energy;
        ++st.reheats_done;
      }
    }
    st.temperature *= decay;
    beta_fresh = false;  // 1 / kT is formed when a step needs it (and at the end)
    if (a.trace && lane == 0) {
      SaStepRec rec;
      rec.site1 = l1;
      rec.site2 = l2;
      rec.accepted = accepted ? 1 : 0;
      rec.pad = 0;
      rec.de = dE;
      rec.energy = e_before;
      rec.temperature = t_before;
      a.trace[it] = rec;
    }
    ++st.steps;
    __syncwarp();
  }
  if (!beta_fresh) st.beta = 1.0 / kBoltzmannEv / fmax(st.temperature, 1e-12);
  if (lane == 0) {
    *a.state = st;
    if (bad) atomicOr(a.status, static_cast<int>(bad));
  }
  __syncwarp();
  if (local_lattice)
    for (long long i = lane; i < nsites_ll; i += 32) species_global[i] = species[i];
  unsigned long long *gw = reinterpret_cast<unsigned long long *>(a.rng);
  for (int i = lane; i < 312; i += 32) gw[i] = mw.cur[i];
  if (lane == 0) a.rng[2 * 312] = mw.idx;
}

// ---------------------------------------------------------------------------
// K5b: throughput CMC. Each round draws `candidates` different-species pairs
// (Philox), resolves overlaps by random priority (a pair survives only if its
// priority is the largest on every site within 3NN of both its sites, so two
// survivors are never within 3NN of each other and their dE terms are
// independent), evaluates dE on the unchanged lattice and applies Metropolis to
// each survivor independently (FP32 factor exp(-dE / kT) and 24-bit uniform; the
// energy change summed exactly in the dE fixed point). Survivors are the
// Metropolis attempts.
// ---------------------------------------------------------------------------
constexpr int kCmcTpThreads = 256;
__global__ void __launch_bounds__(kCmcTpThreads) cmc_tp_kernel(DevTables t, int8_t *species, CmcTpArgs a) {
  cg::grid_group grid = cg::this_grid();
  extern __shared__ __align__(16) unsigned char smem[];
  const SiteSmem s = CarveSiteSmem(t, smem);
  __shared__ unsigned long long s_energy_fix;  // the block's accepted dE sum in the dE fixed point
  __shared__ unsigned long long s_done, s_acc;
  StageArray(t.site_cl, s.cl, t.n_site_cl);
  StageArray(t.site_off, s.off, kSiteSites * 4);
  if (threadIdx.x == 0) {
    s_energy_fix = 0;
    s_done = 0;
    s_acc = 0;
  }
  __syncthreads();
  const int n = a.n;
  const unsigned long long nsites = 4ULL * n * n * n;
  const int warps = blockDim.x >> 5, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int8_t *sa = s.arr + warp * 88, *sb = sa + 44;
  const long long gtid = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
  const uint32_t k0 = static_cast<uint32_t>(a.seed), k1 = static_cast<uint32_t>(a.seed >> 32);
  const float de_beta = static_cast<float>(t.de_scale * a.beta);  // dE / kT per fixed-point unit
  unsigned long long prev_done = 0;
  int empty_rounds = 0;
  for (unsigned long long round = 1;; ++round) {
    // Termination is decided from words written before the last grid barrier,
    // so every thread reads the same values and leaves in the same round.
    const unsigned long long now = *reinterpret_cast<volatile unsigned long long *>(a.done);
    if (now >= a.attempts || *reinterpret_cast<volatile int *>(a.quit)) break;
    empty_rounds = now == prev_done ? empty_rounds + 1 : 0;
    prev_done = now;
    if (empty_rounds > 4096) {  // no swappable pair found for thousands of rounds
      if (gtid == 0) atomicOr(a.status, kStatusNumeric);
      break;
    }
    // phase A: one warp per candidate (candidates spread over the blocks). The
    // lanes make 32 draws at once; the first different-species draw in try
    // order wins, exactly as a sequential search would. Then the lanes claim
    // the 2 x 43 sites within 3NN of the pair. The warp keeps its first
    // candidate (and the two species) in registers for phase B.
    const long long c_first = static_cast<long long>(blockIdx.x) * warps + warp;
    const long long c_stride = static_cast<long long>(gridDim.x) * warps;
    long long r_l1 = -1, r_l2 = -1;
    int r_s1 = 0, r_s2 = 0;
    for (long long c = c_first; c < a.candidates; c += c_stride) {
      long long l1 = -1, l2 = -1;
      int s1 = 0, s2 = 0;
      uint32_t prio = 0;
      for (uint32_t tr0 = 0; tr0 < 64; tr0 += 32) {
        const uint4 x = PhiloxRound10(static_cast<uint32_t>(round), static_cast<uint32_t>(round >> 32),
                                      static_cast<uint32_t>(c), tr0 + lane, k0, k1);
        const long long c1 = static_cast<long long>(__umul64hi((static_cast<unsigned long long>(x.x) << 32) | x.y, nsites));
        const long long c2 = static_cast<long long>(__umul64hi((static_cast<unsigned long long>(x.z) << 32) | x.w, nsites));
        const int sp1 = species[c1], sp2 = species[c2];
        const bool ok = c1 != c2 && sp1 != sp2;
        const unsigned m = __ballot_sync(0xffffffffu, ok);
        if (m) {
          const int src = __ffs(m) - 1;
          l1 = __shfl_sync(0xffffffffu, c1, src);
          l2 = __shfl_sync(0xffffffffu, c2, src);
          s1 = __shfl_sync(0xffffffffu, sp1, src);
          s2 = __shfl_sync(0xffffffffu, sp2, src);
          prio = __shfl_sync(0xffffffffu, (x.x ^ x.w) & 0xFFFF0000u, src);
          break;
        }
      }
      if (c == c_first) {
        r_l1 = l1;
        r_l2 = l2;
        r_s1 = s1;
        r_s2 = s2;
      } else if (lane == 0) {
        a.cand[2 * c] = l1;
        a.cand[2 * c + 1] = l2;
      }
      if (l1 < 0) continue;  // warp-uniform
      const unsigned long long key = (round << 32) | prio | static_cast<uint32_t>(c & 0xFFFF);
      const H3 h1 = SiteCoord(l1, n), h2 = SiteCoord(l2, n);
      for (int q = lane; q < 2 * kSiteSites; q += 32) {
        const int k = q < kSiteSites ? q : q - kSiteSites;
        const int8_t *o = s.off + k * 4;
        atomicMax(&a.claim[NeighborId(q < kSiteSites ? h1 : h2, o[0], o[1], o[2], n)], key);
      }
    }
    grid.sync();
    // phase B: survivors -> dE -> Metropolis (FP32 factor and uniform; the energy as an exact
    // fixed-point sum). The claim words and the pair's neighbourhood are read together; a pair
    // that lost a claim drops its gathered copy.
    for (long long c = c_first; c < a.candidates; c += c_stride) {
      long long l1, l2;
      int s1, s2;
      if (c == c_first) {
        l1 = r_l1;
        l2 = r_l2;
        s1 = r_s1;
        s2 = r_s2;
      } else {
        l1 = a.cand[2 * c];
        l2 = a.cand[2 * c + 1];
        s1 = l1 >= 0 ? species[l1] : 0;  // survivors' sites are written only by themselves
        s2 = l1 >= 0 ? species[l2] : 0;
      }
      if (l1 < 0) continue;
      const unsigned long long c1 = a.claim[l1], c2 = a.claim[l2];
      int pa, pb;
      GatherSwap(s.off, species, n, SiteCoord(l1, n), SiteCoord(l2, n), sa, sb, &pa, &pb, lane);
      const uint32_t lowbits = static_cast<uint32_t>(c1);
      // our key: round in the high word and candidate index in the low 16 bits
      if (c1 != c2 || (c1 >> 32) != round || (lowbits & 0xFFFF) != static_cast<uint32_t>(c & 0xFFFF)) continue;
      const long long acc = WarpSum(SwapDePartial(t, s.cl, sa, sb, pa, pb, lane));
      if (lane == 0) {
        bool ok = acc < 0;  // dE = acc x de_scale, de_scale > 0
        if (!ok) {
          const uint4 x = PhiloxRound10(static_cast<uint32_t>(round), static_cast<uint32_t>(round >> 32),
                                        static_cast<uint32_t>(c), 0xACCE97u, k0, k1);
          ok = static_cast<float>(x.x >> 8) * 5.9604644775390625e-8f < expf(-(I64ToFloat(acc) * de_beta));
        }
        if (ok) {
          species[l1] = static_cast<int8_t>(s2);
          species[l2] = static_cast<int8_t>(s1);
          atomicAdd(&s_energy_fix, static_cast<unsigned long long>(acc));
          atomicAdd(&s_acc, 1ULL);
        }
        atomicAdd(&s_done, 1ULL);
      }
      __syncwarp();
    }
    __syncthreads();
    if (threadIdx.x == 0 && s_done) {
      atomicAdd(a.done, s_done);
      atomicAdd(a.accepted, s_acc);
      s_done = 0;
      s_acc = 0;
    }
    // only one thread reads the host-written stop flag; the decision travels
    // through the quit word and the grid barrier
    if (gtid == 0 && a.stop_flag && *a.stop_flag) {
      atomicOr(a.status, kStatusStopped);
      atomicExch(a.quit, 1);
    }
    if (gtid == 0 && a.rounds) ++*a.rounds;
    grid.sync();
  }
  __syncthreads();
  if (threadIdx.x == 0)
    a.energy_acc[blockIdx.x] = static_cast<double>(static_cast<long long>(s_energy_fix)) * t.de_scale;
}

// Lowest-id vacancy (Config::GetVacancyLatticeId, Config.cpp:298-310) and a
// species histogram per replica.
__global__ void replica_scan_kernel(const int8_t *__restrict__ species, const long long *lat_off, const int *lat_n,
                                    int num_replicas, int x_code, int num_species, long long *first_x,
                                    unsigned long long *hist) {
  const int r = blockIdx.y;
  if (r >= num_replicas) return;
  const int n = lat_n[r];
  const long long nsites = 4LL * n * n * n;
  const int8_t *lat = species + lat_off[r];
  long long best = 0x7fffffffffffffffLL;
  unsigned long long local[kMaxSpecies] = {0, 0, 0, 0, 0, 0};
  unsigned long long invalid = 0;
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < nsites;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int c = lat[i];
    if (c == x_code && i < best) best = i;
    if (c >= 0 && c < num_species) local[c] += 1;
    else invalid += 1;
  }
  // warp totals first: one atomic per warp instead of one per thread
  const int lane = threadIdx.x & 31;
  if (first_x) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const long long v = __shfl_xor_sync(0xffffffffu, best, o);
      best = v < best ? v : best;
    }
    if (lane == 0 && best != 0x7fffffffffffffffLL) atomicMin(&first_x[r], best);
  }
  for (int c = 0; c < num_species; ++c) {
    const unsigned long long v = WarpSumU(local[c]);
    if (lane == 0 && v) atomicAdd(&hist[r * (kMaxSpecies + 1) + c], v);
  }
  const unsigned long long bad = WarpSumU(invalid);
  if (lane == 0 && bad) atomicAdd(&hist[r * (kMaxSpecies + 1) + kMaxSpecies], bad);
}

}  // namespace

cudaError_t LaunchReplicaScan(const int8_t *species, const long long *lat_off, const int *lat_n, int num_replicas,
                              int x_code, int num_species, long long *first_x, unsigned long long *hist,
                              cudaStream_t stream) {
  dim3 grid(num_replicas > 256 ? 8 : 64, num_replicas);
  replica_scan_kernel<<<grid, 256, 0, stream>>>(species, lat_off, lat_n, num_replicas, x_code, num_species, first_x,
                                                hist);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------
namespace {
constexpr int kJumpWarps = 8;
int Blocks(long long work, int per_block) {
  long long b = (work + per_block - 1) / per_block;
  if (b < 1) b = 1;
  if (b > 65535LL * 8) b = 65535LL * 8;
  return static_cast<int>(b);
}
}  // namespace

cudaError_t LaunchBarrierBatch(const DevTables &t, const int8_t *species, int n, const long long *pairs, int m,
                               int kind, double *ea, double *de, double *d_or_e0, double *ks, int *status,
                               cudaStream_t stream) {
  if (m <= 0) return cudaSuccess;
  const size_t sm = JumpSmemBytes(t, kJumpWarps);
  barrier_batch_kernel<<<Blocks(m, kJumpWarps), kJumpWarps * 32, sm, stream>>>(t, species, n, pairs, m, nullptr, kind,
                                                                              ea, de, d_or_e0, ks, status);
  return cudaGetLastError();
}

cudaError_t LaunchBarrierBatchCounted(const DevTables &t, const int8_t *species, int n, const long long *pairs,
                                      int m_max, const int *m_dev, int kind, double *ea, double *de, int *status,
                                      cudaStream_t stream) {
  if (m_max <= 0) return cudaSuccess;
  const size_t sm = JumpSmemBytes(t, kJumpWarps);
  // a grid for a few percent of the pairs: the warps stride over whatever the device count holds
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = std::max(1, std::min(Blocks(m_max, kJumpWarps), sms * 2));
  barrier_batch_kernel<<<blocks, kJumpWarps * 32, sm, stream>>>(t, species, n, pairs, m_max, m_dev, kind, ea, de,
                                                                nullptr, nullptr, status);
  return cudaGetLastError();
}

cudaError_t LaunchSurrogateDataset(const DevTables &t, const SurrogateGen &g, cudaStream_t stream) {
  if (g.count <= 0) return cudaSuccess;
  if (g.enc.width < 1 || g.in_pad < (kEnvSites + 1) * g.enc.width) return cudaErrorInvalidValue;
  const size_t sm = JumpSmemBytes(t, kJumpWarps) + kJumpWarps * 144;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long need = (g.count + kJumpWarps - 1) / kJumpWarps;
  const int blocks = static_cast<int>(need < sms * 8LL ? need : sms * 8LL);
  cudaError_t err = cudaFuncSetAttribute(surrogate_dataset_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(sm));
  if (err != cudaSuccess) return err;
  surrogate_dataset_kernel<<<blocks, kJumpWarps * 32, sm, stream>>>(t, g);
  return cudaGetLastError();
}

cudaError_t LaunchSurrogateFeatures(const DevTables &t, const int8_t *species, int n, const long long *pairs, int m,
                                    int in_pad, const FeatEnc &enc, __nv_bfloat16 *features, int *status,
                                    cudaStream_t stream) {
  if (m <= 0) return cudaSuccess;
  if (enc.width < 1 || in_pad < (kEnvSites + 1) * enc.width) return cudaErrorInvalidValue;
  if (in_pad % 8 == 0 && (reinterpret_cast<uintptr_t>(features) & 15) == 0) {
    const int blocks = static_cast<int>((m + 255) / 256);
    switch (enc.width) {
      case 1: surrogate_features_thread_kernel<1><<<blocks, 256, 0, stream>>>(t, species, n, pairs, m, in_pad, enc, features, status); return cudaGetLastError();
      case 2: surrogate_features_thread_kernel<2><<<blocks, 256, 0, stream>>>(t, species, n, pairs, m, in_pad, enc, features, status); return cudaGetLastError();
      case 3: surrogate_features_thread_kernel<3><<<blocks, 256, 0, stream>>>(t, species, n, pairs, m, in_pad, enc, features, status); return cudaGetLastError();
      case 4: surrogate_features_thread_kernel<4><<<blocks, 256, 0, stream>>>(t, species, n, pairs, m, in_pad, enc, features, status); return cudaGetLastError();
      case 5: surrogate_features_thread_kernel<5><<<blocks, 256, 0, stream>>>(t, species, n, pairs, m, in_pad, enc, features, status); return cudaGetLastError();
      default: break;
    }
  }
  const size_t sm = kJumpWarps * 64;
  surrogate_features_kernel<<<Blocks(m, kJumpWarps), kJumpWarps * 32, sm, stream>>>(t, species, n, pairs, m, in_pad, enc,
                                                                                  features, status);
  return cudaGetLastError();
}

namespace {
// Pairs whose ensemble spread exceeds the threshold (or whose mean is not finite) go to the plain predictor.
__global__ void fallback_compact_kernel(const long long *pairs, const float *mean, const float *spread, int m,
                                        float threshold, long long *fb_pairs, int *fb_index, int *count,
                                        uint8_t *flag) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  const bool fb = !(spread[i] <= threshold) || !isfinite(mean[i]);
  if (flag) flag[i] = fb ? 1 : 0;
  if (!fb) return;
  const int k = atomicAdd(count, 1);
  fb_pairs[2 * k] = pairs[2 * i];
  fb_pairs[2 * k + 1] = pairs[2 * i + 1];
  fb_index[k] = i;
}
// Surrogate means first; the plain barriers of the fallback pairs are scattered over them afterwards.
__global__ void fallback_merge_kernel(const float *mean, int m, double *ea) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < m) ea[i] = static_cast<double>(mean[i]);
}
__global__ void fallback_scatter_kernel(const double *fb_ea, const int *fb_index, const int *count, double *ea) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < *count) ea[fb_index[k]] = fb_ea[k];
}
}  // namespace

cudaError_t LaunchFallbackCompact(const long long *pairs, const float *mean, const float *spread, int m,
                                  float threshold, long long *fb_pairs, int *fb_index, int *count, uint8_t *flag,
                                  cudaStream_t stream) {
  if (m <= 0) return cudaSuccess;
  fallback_compact_kernel<<<(m + 255) / 256, 256, 0, stream>>>(pairs, mean, spread, m, threshold, fb_pairs, fb_index,
                                                               count, flag);
  return cudaGetLastError();
}

cudaError_t LaunchFallbackMerge(const float *mean, int m, const double *fb_ea, const int *fb_index, const int *count,
                                double *ea, cudaStream_t stream) {
  if (m <= 0) return cudaSuccess;
  fallback_merge_kernel<<<(m + 255) / 256, 256, 0, stream>>>(mean, m, ea);
  fallback_scatter_kernel<<<(m + 255) / 256, 256, 0, stream>>>(fb_ea, fb_index, count, ea);
  return cudaGetLastError();
}

cudaError_t LaunchEncodeBatch(const DevTables &t, const int8_t *species, int n, const long long *pairs, int m,
                              int *state_start, int *state_end, int *mmm, int *mm2f, int *mm2b, int *status,
                              cudaStream_t stream) {
  if (m <= 0) return cudaSuccess;
  const size_t sm = JumpSmemBytes(t, kJumpWarps);
  encode_batch_kernel<<<Blocks(m, kJumpWarps), kJumpWarps * 32, sm, stream>>>(t, species, n, pairs, m, state_start,
                                                                             state_end, mmm, mm2f, mm2b, status);
  return cudaGetLastError();
}

cudaError_t LaunchSiteDe(const DevTables &t, const int8_t *species, int n, const long long *sites, const int8_t *from,
                         const int8_t *to, long long m, long long fill_site, int fill_code, double *de,
                         cudaStream_t stream) {
  if (m <= 0) return cudaSuccess;
  const size_t sm = SiteSmemBytes(t, kJumpWarps);
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long want = (m + kJumpWarps - 1) / kJumpWarps;
  const int blocks = static_cast<int>(std::min<long long>(want, 32LL * sms));
  site_de_kernel<<<blocks, kJumpWarps * 32, sm, stream>>>(t, species, n, sites, from, to, m, fill_site, fill_code, de);
  return cudaGetLastError();
}

cudaError_t LaunchExitEnergies(const DevTables &t, const int8_t *species, int n, long long vac, int solvent,
                               const double *mu, double *binding, double *profile, cudaStream_t stream) {
  if (t.num_species - 1 > kExitMaxElements || t.x_code < 0) return cudaErrorInvalidValue;
  const long long nsites = 4LL * n * n * n;
  const size_t sm = SiteSmemBytes(t, kJumpWarps);
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = static_cast<int>(std::min<long long>((nsites + kJumpWarps - 1) / kJumpWarps, 32LL * sms));
  exit_energy_kernel<<<blocks, kJumpWarps * 32, sm, stream>>>(t, species, n, vac, solvent, mu, binding, profile);
  return cudaGetLastError();
}

cudaError_t LaunchDePairs(const DevTables &t, const int8_t *species, int n, const long long *pairs, int m, double *de,
                          int *status, cudaStream_t stream) {
  if (m <= 0) return cudaSuccess;
  const size_t sm = SiteSmemBytes(t, kJumpWarps);
  de_pairs_kernel<<<Blocks(m, kJumpWarps), kJumpWarps * 32, sm, stream>>>(t, species, n, pairs, m, de, status);
  return cudaGetLastError();
}

cudaError_t LaunchCensus(const DevTables &t, const int8_t *species, int n, int base_code,
                         unsigned long long *counts, double *energy, cudaStream_t stream) {
  cudaError_t err = cudaMemsetAsync(counts, 0, sizeof(unsigned long long) * t.num_theta, stream);
  if (err != cudaSuccess) return err;
  const long long nsites = 4LL * n * n * n;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  long long blocks = (nsites + kCensusThreads - 1) / kCensusThreads;
  const long long cap = static_cast<long long>(sms) * 8;
  if (blocks > cap) blocks = cap;
  census_kernel<false><<<static_cast<int>(blocks), kCensusThreads, 0, stream>>>(t, species, n, base_code, counts,
                                                                                nullptr);
  err = cudaGetLastError();
  if (err != cudaSuccess) return err;
  census_energy_kernel<<<1, 32, 0, stream>>>(t, counts, energy, nullptr);
  return cudaGetLastError();
}

cudaError_t LaunchCensusCheckedNoAlloc(const DevTables &t, const int8_t *species, int n, int base_code,
                                       unsigned long long *scratch, double *energy, cudaStream_t stream) {
  if (t.num_theta > kNoAllocMaxTheta) return cudaErrorInvalidValue;
  // every call starts from zero: the counters and the bad-code word after them
  cudaError_t err = cudaMemsetAsync(scratch, 0, sizeof(unsigned long long) * kNoAllocScratchWords, stream);
  if (err != cudaSuccess) return err;
  unsigned long long *bad = scratch + kNoAllocMaxTheta;
  const long long nsites = 4LL * n * n * n;
  int dev = 0, sms = 0;
  err = cudaGetDevice(&dev);
  if (err != cudaSuccess) return err;
  err = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (err != cudaSuccess) return err;
  long long blocks = (nsites + kCensusThreads - 1) / kCensusThreads;
  const long long cap = static_cast<long long>(sms) * 8;
  if (blocks > cap) blocks = cap;
  census_kernel<true><<<static_cast<int>(blocks), kCensusThreads, 0, stream>>>(t, species, n, base_code, scratch,
                                                                               bad);
  err = cudaGetLastError();
  if (err != cudaSuccess) return err;
  census_energy_kernel<<<1, 32, 0, stream>>>(t, scratch, energy, bad);
  return cudaGetLastError();
}

size_t KmcSharedBytes(const DevTables &t, const KmcLaunch &l) {
  size_t b = 4u * (t.n_de_cl + t.n_mmm_cl + t.n_mm2_cl) + sizeof(SmallTables) + 12 * kStateSites +
             3 * 12 * kEnvSites + kLocalSites * 4;
  b = (b + 15) & ~size_t(15);
  b += sizeof(double) * kExpTableSize;
  b += sizeof(KmcShared) * l.replicas_per_block;
  b += static_cast<size_t>(kArr) * l.warps_per_replica * l.replicas_per_block;
  if (l.sparse) b += 4 * 12 * 136 + 4 * 2 * (kTriEnv + 1) + 4 * kLocalSites * kInterWords + 2 * (kTriState + 1);
  return (b + 15) & ~size_t(15);
}

template <typename K>
static cudaError_t PrepareKmc(K kern, size_t sm) {
  return cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(sm));
}

// Kernel instance for the launch shape of `l`.
using KmcKernelFn = void (*)(DevTables, int8_t *, KmcDevState, KmcLaunch);
static KmcKernelFn KmcKernelFor(const KmcLaunch &l) {
  const int threads = l.warps_per_replica * l.replicas_per_block * 32;
  const int shape = threads <= kShapeThreads[0] ? 0 : (threads <= kShapeThreads[1] ? 1 : 2);
  // the RNG kind and the epilogue precision are template parameters so the Philox instances carry
  // no mt19937_64 code (and back) and the FP32 instances no FP64 epilogue
  if (l.mt) {
    if (l.sparse)
      return shape == 0 ? kmc_kernel<true, 0, true, false>
                        : (shape == 1 ? kmc_kernel<true, 1, true, false> : kmc_kernel<true, 2, true, false>);
    return shape == 0 ? kmc_kernel<false, 0, true, false>
                      : (shape == 1 ? kmc_kernel<false, 1, true, false> : kmc_kernel<false, 2, true, false>);
  }
  if (l.f32) {
    if (l.sparse)
      return shape == 0 ? kmc_kernel<true, 0, false, true>
                        : (shape == 1 ? kmc_kernel<true, 1, false, true> : kmc_kernel<true, 2, false, true>);
    return shape == 0 ? kmc_kernel<false, 0, false, true>
                      : (shape == 1 ? kmc_kernel<false, 1, false, true> : kmc_kernel<false, 2, false, true>);
  }
  if (l.sparse)
    return shape == 0 ? kmc_kernel<true, 0, false, false>
                      : (shape == 1 ? kmc_kernel<true, 1, false, false> : kmc_kernel<true, 2, false, false>);
  return shape == 0 ? kmc_kernel<false, 0, false, false>
                    : (shape == 1 ? kmc_kernel<false, 1, false, false> : kmc_kernel<false, 2, false, false>);
}

cudaError_t KmcOccupancy(const DevTables &t, const KmcLaunch &l, int *blocks_per_sm, size_t *shared_bytes) {
  const int threads = l.warps_per_replica * l.replicas_per_block * 32;
  if (threads > kShapeThreads[2] || (threads > kShapeThreads[1] && l.warps_per_replica != 1))
    return cudaErrorInvalidConfiguration;
  const size_t sm = KmcSharedBytes(t, l);
  const KmcKernelFn kern = KmcKernelFor(l);
  cudaError_t err = PrepareKmc(kern, sm);
  if (err != cudaSuccess) return err;
  *shared_bytes = sm;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, kern, threads, sm);
}

cudaError_t LaunchKmc(const DevTables &t, int8_t *species, const KmcDevState &s, const KmcLaunch &l,
                      cudaStream_t stream, bool prepare) {
  const int threads = l.warps_per_replica * l.replicas_per_block * 32;
  if (threads > kShapeThreads[2] || (threads > kShapeThreads[1] && l.warps_per_replica != 1))
    return cudaErrorInvalidConfiguration;
  const int blocks = (s.num_replicas + l.replicas_per_block - 1) / l.replicas_per_block;
  const size_t sm = KmcSharedBytes(t, l);
  const KmcKernelFn kern = KmcKernelFor(l);
  if (prepare) {
    cudaError_t err = PrepareKmc(kern, sm);
    if (err != cudaSuccess) return err;
  }
  kern<<<blocks, threads, sm, stream>>>(t, species, s, l);
  return cudaGetLastError();
}

cudaError_t LaunchSoluteLabels(const DevTables &t, const int8_t *species, int n, int solvent, uint32_t *parent,
                               int *status, cudaStream_t stream) {
  const long long nsites = 4LL * n * n * n;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = static_cast<int>(std::min<long long>((nsites + 255) / 256, 8LL * sms));
  solute_label_init_kernel<<<blocks, 256, 0, stream>>>(species, nsites, solvent, parent);
  solute_hook_kernel<<<blocks, 256, 0, stream>>>(t, species, n, solvent, parent, status);
  solute_flatten_kernel<<<blocks, 256, 0, stream>>>(nsites, parent);
  return cudaGetLastError();
}

cudaError_t LaunchClusterCensus(const DevTables &t, const int8_t *species, int n, int solvent, long long clusters,
                                const long long *s_off, const long long *s_ids, const long long *l_off,
                                const long long *l_ids, double *energies, cudaStream_t stream) {
  if (clusters <= 0) return cudaSuccess;
  if (clusters > 0x7FFFFFFFLL || t.num_theta > 512 || t.n_census_tri > 160 || t.num_species > 6)
    return cudaErrorInvalidValue;
  cluster_census_kernel<<<static_cast<int>(clusters), kClusterThreads, 0, stream>>>(t, species, n, solvent, s_off,
                                                                                    s_ids, l_off, l_ids, energies);
  return cudaGetLastError();
}

cudaError_t LaunchSiteJumps(const DevTables &t, const int8_t *species, const SiteJumpArgs &a, cudaStream_t stream) {
  if (a.m <= 0) return cudaSuccess;
  KmcLaunch l{};
  l.warps_per_replica = 1;
  l.replicas_per_block = kSiteJumpWarps;
  l.sparse = 1;  // the carve always holds the sparse tables
  const size_t sm = KmcSharedBytes(t, l);
  auto kern = a.sparse ? site_jumps_kernel<true> : site_jumps_kernel<false>;
  cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(sm));
  if (err != cudaSuccess) return err;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long need = (a.m + kSiteJumpWarps - 1) / kSiteJumpWarps;
  const int blocks = static_cast<int>(std::min<long long>(need, static_cast<long long>(sms) * 8));
  kern<<<blocks, kSiteJumpWarps * 32, sm, stream>>>(t, species, a);
  return cudaGetLastError();
}

cudaError_t LaunchBarrierGroup(const DevTables &t, const int8_t *species, const BarrierGroupArgs &a,
                               cudaStream_t stream) {
  if (a.m <= 0) return cudaSuccess;
  KmcLaunch l{};
  l.warps_per_replica = 1;
  l.replicas_per_block = kSiteJumpWarps;
  l.sparse = 1;
  const size_t sm = KmcSharedBytes(t, l);
  cudaError_t err =
      cudaFuncSetAttribute(barrier_group_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(sm));
  if (err != cudaSuccess) return err;
  int dev = 0, sms = 0;
  err = cudaGetDevice(&dev);
  if (err != cudaSuccess) return err;
  err = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (err != cudaSuccess) return err;
  // one warp per 12 pairs, at most one wave of resident blocks (each block stages the tables once
  // and strides over the runs); a device-side count (m_dev) only shrinks the work
  int resident = 0;
  err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, barrier_group_kernel, kSiteJumpWarps * 32, sm);
  if (err != cudaSuccess) return err;
  const long long need = (a.m + 12LL * kSiteJumpWarps - 1) / (12LL * kSiteJumpWarps);
  const long long wave = static_cast<long long>(sms) * std::max(1, resident);
  const int blocks = static_cast<int>(std::max<long long>(1, std::min<long long>(need, wave)));
  barrier_group_kernel<<<blocks, kSiteJumpWarps * 32, sm, stream>>>(t, species, a);
  return cudaGetLastError();
}

size_t KmcChainSharedBytes(const DevTables &t, bool sparse) { return ChainSharedBytes(t, sparse); }

cudaError_t LaunchKmcChain(const DevTables &t, int8_t *species, const KmcDevState &s, const KmcLaunch &l,
                           cudaStream_t stream) {
  const size_t sm = ChainSharedBytes(t, l.sparse != 0);
  auto kern = l.sparse ? kmc_chain_kernel<true> : kmc_chain_kernel<false>;
  cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(sm));
  if (err != cudaSuccess) return err;
  kern<<<s.num_replicas, kChainWarps * 32, sm, stream>>>(t, species, s, l);
  return cudaGetLastError();
}

size_t KmcMultiSharedBytes(const DevTables &t, bool sparse) { return MultiSharedBytes(t, sparse); }

cudaError_t LaunchKmcMulti(const DevTables &t, int8_t *species, const KmcMultiArgs &a, bool sparse,
                           cudaStream_t stream) {
  const size_t sm = MultiSharedBytes(t, sparse);
  auto kern = sparse ? (a.f32 ? kmc_multi_kernel<true, true> : kmc_multi_kernel<true, false>)
                     : (a.f32 ? kmc_multi_kernel<false, true> : kmc_multi_kernel<false, false>);
  cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(sm));
  if (err != cudaSuccess) return err;
  kern<<<a.num_replicas, kMultiWarps * 32, sm, stream>>>(t, species, a);
  return cudaGetLastError();
}

template <int kC>
static cudaError_t LaunchSurrogateKmcC(const DevTables &t, int8_t *species, const KmcSurrogateArgs &a, const MlpDev &d,
                                       const FusedJumps &j, cudaStream_t stream) {
  constexpr size_t sm = SurrogateSmemBytes<kC>();
  const cudaError_t err = cudaFuncSetAttribute(kmc_surrogate_kernel<kC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               static_cast<int>(sm));
  if (err != cudaSuccess) return err;
  kmc_surrogate_kernel<kC><<<1, kSurWarps * 32, sm, stream>>>(t, species, a, d, j);
  return cudaGetLastError();
}

cudaError_t LaunchKmcSurrogate(const DevTables &t, int8_t *species, const KmcSurrogateArgs &a, const MlpDev &d,
                               const FusedJumps &j, cudaStream_t stream) {
  if (a.nv < 1 || a.nv > kMaxMultiVac || a.nsteps == 0) return cudaErrorInvalidValue;
  const int kc = MlpFusedChannels(d);
  if (kc != j.channels) return cudaErrorInvalidValue;
  return kc == 2 ? LaunchSurrogateKmcC<2>(t, species, a, d, j, stream)
                 : LaunchSurrogateKmcC<3>(t, species, a, d, j, stream);
}

cudaError_t LaunchCmcReference(const DevTables &t, int8_t *species, const CmcRefArgs &a, cudaStream_t stream) {
  if (a.batch < 1 || a.batch > kCmcRefMaxBatch || a.n < 6) return cudaErrorInvalidValue;
  const long long nsites = 4LL * a.n * a.n * a.n;
  const size_t sm = SiteSmemBytes(t, kCmcRefWarps) + (nsites <= kCmcRefSmemSites ? static_cast<size_t>(nsites) : 0);
  cudaError_t err = cudaFuncSetAttribute(cmc_ref_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(sm));
  if (err != cudaSuccess) return err;
  cmc_ref_kernel<<<1, kCmcRefWarps * 32, sm, stream>>>(t, species, a);
  return cudaGetLastError();
}

cudaError_t LaunchSa(const DevTables &t, int8_t *species, const SaArgs &a, cudaStream_t stream) {
  const long long nsites = 4LL * a.n * a.n * a.n;
  const size_t sm = SiteSmemBytes(t, 1) + (nsites <= kSaSmemSites ? static_cast<size_t>(nsites) : 0);
  cudaError_t err = cudaFuncSetAttribute(sa_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(sm));
  if (err != cudaSuccess) return err;
  sa_kernel<<<1, 32, sm, stream>>>(t, species, a);
  return cudaGetLastError();
}

int CmcThroughputResidentWarps(const DevTables &t, int device) {
  const size_t sm = SiteSmemBytes(t, kCmcTpThreads / 32);
  int per_sm = 0, sms = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, cmc_tp_kernel, kCmcTpThreads, sm) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  return sms * per_sm * (kCmcTpThreads / 32);
}

cudaError_t LaunchCmcThroughput(const DevTables &t, int8_t *species, const CmcTpArgs &a, int device,
                                cudaStream_t stream) {
  const size_t sm = SiteSmemBytes(t, kCmcTpThreads / 32);
  int per_sm = 0, sms = 0;
  cudaError_t err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, cmc_tp_kernel, kCmcTpThreads, sm);
  if (err != cudaSuccess) return err;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  if (per_sm < 1) return cudaErrorCooperativeLaunchTooLarge;
  int blocks = sms * per_sm;
  const int needed = (a.candidates + (kCmcTpThreads / 32) - 1) / (kCmcTpThreads / 32);
  if (blocks > needed) blocks = needed < 1 ? 1 : needed;
  DevTables tt = t;
  CmcTpArgs aa = a;
  int8_t *sp = species;
  void *args[] = {&tt, &sp, &aa};
  return cudaLaunchCooperativeKernel(reinterpret_cast<void *>(cmc_tp_kernel), blocks, kCmcTpThreads, args, sm,
                                     stream);
}

// Self-check of the FP64 helpers: fn 0 ExpFast / exp, fn 1 RcpFast / 1.0 / x.
__global__ void fastmath_check_kernel(DevTables t, int fn, const double *x, long long n, double *fast, double *ref) {
  const ExpConsts ec{t.exp_tab, t.exp_l1, t.exp_l2};
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    const double v = x[i];
    fast[i] = fn == 0 ? ExpFast(v, ec) : RcpFast(v);
    ref[i] = fn == 0 ? exp(v) : 1.0 / v;
  }
}

cudaError_t LaunchFastmathCheck(const DevTables &t, int fn, const double *x, long long n, double *fast, double *ref,
                                cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  const long long blocks = (n + 255) / 256;
  fastmath_check_kernel<<<static_cast<int>(blocks < 4096 ? blocks : 4096), 256, 0, stream>>>(t, fn, x, n, fast, ref);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Allocation-free census: the cluster histogram lives in a file-scope device
// array shared by every call on a device (see lmc_energy_noalloc).
// ---------------------------------------------------------------------------
namespace {
static __device__ __align__(256) unsigned long long g_noalloc_census_counts[kNoAllocScratchWords];
}  // namespace

cudaError_t NoAllocCensusScratch(int device, unsigned long long **ptr) {
  // The array's host-side name is only a stand-in; the device address is
  // looked up once per device, with that device current.
  static std::mutex mu;
  static unsigned long long *addr[kNoAllocMaxDevices] = {};
  if (device < 0 || device >= kNoAllocMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(mu);
  if (addr[device] == nullptr) {
    int current = -1;
    cudaError_t err = cudaGetDevice(&current);
    if (err != cudaSuccess) return err;
    if (current != device) return cudaErrorInvalidDevice;
    void *p = nullptr;
    err = cudaGetSymbolAddress(&p, g_noalloc_census_counts);
    if (err != cudaSuccess) return err;
    addr[device] = static_cast<unsigned long long *>(p);
  }
  *ptr = addr[device];
  return cudaSuccess;
}

void MtSeed(uint64_t seed, uint32_t *words) {
  // std::mt19937_64 seeding (the C++ standard, [rand.eng.mers]):
  // x0 = seed, x_i = 6364136223846793005 * (x_{i-1} ^ (x_{i-1} >> 62)) + i.
  unsigned long long *mt = reinterpret_cast<unsigned long long *>(words);
  mt[0] = seed;
  for (int i = 1; i < 312; ++i) mt[i] = 6364136223846793005ULL * (mt[i - 1] ^ (mt[i - 1] >> 62)) + i;
  words[2 * 312] = 312;  // next draw twists
  words[2 * 312 + 1] = 0;
}

}  // namespace lmc
