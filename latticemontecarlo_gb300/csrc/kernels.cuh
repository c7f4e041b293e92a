// Launch interface of the sm_103a kernels (implemented in kernels.cu).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "device_tables.hpp"
#include "model.hpp"
#include "mlp.cuh"

namespace lmc {

// Per-replica KMC state (structure of arrays, device memory).
struct KmcDevState {
  long long *vacancy;
  unsigned long long *steps;
  double *time;
  double *energy;
  double *temperature;        // base temperature (used when no T(t) table)
  double *corr_cvac;          // rate-corrector inputs; negative = disabled
  double *corr_csol;
  uint32_t *rng;              // per replica: kRngWords words
  const long long *lat_off;   // site offset of each replica in the species arena
  const int *lat_n;           // cube edge of each replica
  int num_replicas;
  int rng_kind;               // 0 = MT19937-64, 1 = Philox
  int barrier_kind;           // 0 = Quartic, 1 = E0
  const double *tt_time;      // optional T(t) table
  const double *tt_temp;
  int tt_len;
  int early_stop;             // IsEscaped: stop a replica whose vacancy is surrounded by solvent
  const int8_t *solvent;      // per replica: most frequent species code
  uint8_t *escaped;           // per replica: 1 once the early stop ended the trajectory
  long long *prev;            // per replica: previous vacancy site (second-order chain KMC)
};

constexpr int kRngWords = 2 * 312 + 2;  // MT19937-64 state (312 x u64) + index; Philox uses 4 words

struct KmcTraceRec {
  long long vacancy, target;
  int selected, slot;  // slot: the vacancy that moved (multi-vacancy kernel; 0 otherwise)
  double ea, de, total_rate, time, energy;
};

// Tables of the sparse jump evaluation, built for one dominant "base" species b.
// With all non-pair sites at b a jump's sums are per-migrant constants. Any
// cluster holds at most two sites other than the pair sites, so by
// inclusion-exclusion the exact sums are
//   constant + sum over non-base sites p of S[list][p][species(p)]
//            + sum over non-base pairs (p, q) sharing a cluster of a pair term,
// all in the same int64 fixed point as the dense evaluation (bit-identical,
// since wrapping integer sums do not depend on their order).
// Lists: 0 state (energy change), 1 MMM, 2 MM2 forward, 3 MM2 backward.
constexpr int kMaxSparseSites = 32;  // more non-base neighbourhood sites: dense evaluation for that step
constexpr int kMaxSparsePairs = 96;  // more interacting non-base pairs: dense evaluation for that step
constexpr int kInterWords = 5;       // 135-bit rows of the local pair-interaction table
constexpr int kTriState = 60 * 59 / 2, kTriEnv = 58 * 57 / 2;
__host__ __device__ __forceinline__ int Tri(int p, int q) {
  const int hi = p > q ? p : q, lo = p > q ? q : p;
  return hi * (hi - 1) / 2 + lo;
}
struct KmcSparse {
  const uint8_t *pos;      // [4][12][136]: local index -> position in list of jump c, 255 none (column 135: none)
  const uint32_t *inter;   // [135][5]: bit b of row a set when local sites a, b share a cluster in some jump
  const long long *s_de;   // [E migrant][61][E species]: single-site energy-change terms, row 60 zero
  const long long *s_env;  // [slot][3 forms: D, Ks, e0][59][8 ranks]: single-site feature terms, row 58 zero
  // site-pair lookups, strict lower triangles: entry (p, q), p != q, at
  // Tri(max, min) = max * (max - 1) / 2 + min, one extra "none" entry at the end
  const uint16_t *px_st;   // [kTriState + 1]: up to two triplets holding both sites, (label | side << 3) per
                           // byte, 0 none (label 0 rows of p_de are zero)
  const uint32_t *px_env;  // [2: MMM, MM2][kTriEnv + 1]: feature base | mode << 20 | (lower site is the
                           // cluster's first) << 22 of the pair cluster; none points at the zero block
  const long long *p_de;   // [8][E][E][E]: pair term of a triplet, F(c1, c2) - F(c1, b) - F(b, c2); label 0 zero
  const long long *base_de;    // [E] all-base energy change per migrant code
  const long long *dw_d;       // [slot][dw_stride_mmm] W - W(block entry of the base pair type), then 64 zeros
  const long long *dw_ks;      // [slot][dw_stride_mm2]
  const long long *dw_e0;      // [slot][dw_stride_mmm]
  const long long *base_form;  // [slot][3] all-base sums of D, Ks (forward + backward), e0
  int dw_stride_mmm, dw_stride_mm2;
  int base_code;
  int center;  // local index of the vacancy site
  int x_code;  // species code of the vacancy
};

struct KmcLaunch {
  int warps_per_replica;
  int replicas_per_block;
  unsigned long long steps;
  int trace_replica;             // -1 = none
  KmcTraceRec *trace;            // device, steps records
  double *events12;              // device, steps * 36 doubles, may be null
  volatile int *stop_flag;       // host-mapped, may be null
  int *status;                   // device status word (bit flags)
  int sparse;                    // 1: sparse solute corrections, 0: dense cluster sums
  int mt;                        // 1: mt19937_64 stream (KmcDevState::rng_kind 0), 0: Philox
  int f32;                       // 1 (Philox only): FP32 barriers and rates, FP64 rate sum and clock
  KmcSparse sp;
};

// Status bits written by kernels.
constexpr int kStatusNotNeighbor = 1;     // a queried pair is not 1NN
constexpr int kStatusNoCoefficients = 2;  // migrating element without coefficients
constexpr int kStatusBadCluster = 4;      // ElementCluster outside the indexer (e.g. two vacancies)
constexpr int kStatusXInEnv = 8;          // vacancy inside an MMM/MM2 environment
constexpr int kStatusNumeric = 16;        // NaN / inf / non-positive total rate
constexpr int kStatusStopped = 32;        // stop flag observed
constexpr int kStatusBadSite = 64;        // site id out of range

cudaError_t LaunchBarrierBatch(const DevTables &t, const int8_t *species, int n, const long long *pairs, int m,
                               int kind, double *ea, double *de, double *d_or_e0, double *ks, int *status,
                               cudaStream_t stream);
cudaError_t LaunchEncodeBatch(const DevTables &t, const int8_t *species, int n, const long long *pairs, int m,
                              int *state_start, int *state_end, int *mmm, int *mm2f, int *mm2b, int *status,
                              cudaStream_t stream);
cudaError_t LaunchDePairs(const DevTables &t, const int8_t *species, int n, const long long *pairs, int m, double *de,
                          int *status, cudaStream_t stream);
// GetDeFromLatticeIdSite for m queries: species at sites[q] (from[q], or the lattice's own when from
// is null) replaced by to[q], the lattice read with fill_site (>= 0) holding fill_code.
cudaError_t LaunchSiteDe(const DevTables &t, const int8_t *species, int n, const long long *sites, const int8_t *from,
                         const int8_t *to, long long m, long long fill_site, int fill_code, double *de,
                         cudaStream_t stream);
// ExitTime's binding energies binding[k][i] (k = rank of the element among the non-X codes) and
// profile energies profile[i] of every site, the vacancy `vac` (>= 0) read as the solvent.
cudaError_t LaunchExitEnergies(const DevTables &t, const int8_t *species, int n, long long vac, int solvent,
                               const double *mu, double *binding, double *profile, cudaStream_t stream);
cudaError_t LaunchCensus(const DevTables &t, const int8_t *species, int n, int base_code,
                         unsigned long long *counts, double *energy, cudaStream_t stream);
// Multi-vacancy KMC: every vacancy of a lattice is tracked and one event is
// chosen per step among all of them (residence-time selection over V x 12
// events); one block per lattice. Vacancies are slots 0..V-1 (ascending site
// id at initialisation), kept when they move.
constexpr int kMaxMultiVac = 256;
constexpr int kMultiWarps = 8;
constexpr int kMultiItemSubs = 8;                         // threads per sparse item, one re-evaluated slot
constexpr int kMultiItemWarps = 24 * kMultiItemSubs / 32;  // the warps that share the 24 items
static_assert(kMultiItemWarps <= kMultiWarps, "items fit the block");
constexpr int kLocalSpan = 9;  // neighbourhood displacements lie in [-4, 4]^3 (half-lattice units)
constexpr int kLocalBitWords = (kLocalSpan * kLocalSpan * kLocalSpan + 31) / 32;
struct KmcMultiArgs {
  long long *vac_pos;               // [slots] lattice id of each vacancy
  const int *vac_off;               // [R + 1] first slot of each lattice
  unsigned long long *steps;        // [R]
  double *time, *energy;            // [R]
  const double *temperature;        // [R]
  const uint32_t *key;              // [R][2] Philox key
  const long long *lat_off;
  const int *lat_n;
  int num_replicas;
  int barrier_kind;
  int f32;                          // 1: FP32 barriers and rates, FP64 rate sums and clock, exact energy
  unsigned long long nsteps;        // steps per launch
  int trace_replica;                // -1 = none
  KmcTraceRec *trace;               // [nsteps] records of lattice trace_replica
  volatile int *stop_flag;          // host-mapped, may be null
  int *status;
  KmcSparse sp;
  uint32_t local_bits[kLocalBitWords];  // displacements (dx, dy, dz) + 4 of the 135-site neighbourhood
};
size_t KmcMultiSharedBytes(const DevTables &t, bool sparse);
cudaError_t LaunchKmcMulti(const DevTables &t, int8_t *species, const KmcMultiArgs &a, bool sparse,
                           cudaStream_t stream);

// Surrogate-assisted multi-vacancy KMC of one lattice (kmc_surrogate_kernel, one persistent
// CTA): the device state of a run.
struct KmcSurrogateArgs {
  long long *vac_pos;             // [nv] vacancy site of each slot
  int nv;
  unsigned long long nsteps;      // steps of this launch
  unsigned long long *steps;      // [1] steps taken (the Philox counter of the next draw)
  double *time, *energy;          // [1]
  double temperature;
  uint32_t key0, key1;            // Philox key of the lattice
  int replica;                    // the lattice's index (Philox counter word)
  long long lat_off;
  int n;
  int barrier_kind;
  float threshold;                // ensemble spread (eV) above which a jump takes the plain predictor
  float *mean, *spread;           // [nv * 12] network outputs of the listed jumps
  long long *pairs;               // [nv * 12][2] listed jumps, 12 per listed slot in direction order
  int *dirty;                     // [nv] listed slots
  double *cum, *ea;               // [nv * 12] per slot in id order: inclusive rate scan, barrier used
  long long *tgt;                 // [nv * 12]
  uint32_t *kmask;                // [nv] bit e: event e of the slot has a positive rate
  double *pair_ea;                // [nv * 12] plain barriers of the rows that fell back
  unsigned long long *fallbacks;  // [1] jumps sent to the plain predictor
  int *halt;                      // [1] set by a stop or an error
  int *net_status;                // [1] set when a tensor-core wait expired
  KmcTraceRec *trace;             // nullable: step s at trace[s - trace_base], s - trace_base < trace_len
  double *plain_ea;               // nullable: the plain barrier of the selected event, same index
  unsigned long long trace_base, trace_len;
  volatile int *stop_flag;
  int *status;
  uint32_t local_bits[kLocalBitWords];
};
// j: the lattice and encoding of the fused jump gather (species, n, offsets, channels; its pairs,
// counts and outputs are unused), with the network's label scale in mean_label / std_label.
cudaError_t LaunchKmcSurrogate(const DevTables &t, int8_t *species, const KmcSurrogateArgs &a, const MlpDev &d,
                               const FusedJumps &j, cudaStream_t stream);

// Second-order chain KMC (KineticMcChainOmpi semantics): one block of 12 warps
// per replica, warp d evaluating the 12 jumps after the jump along direction d.
constexpr int kChainWarps = 12;
size_t KmcChainSharedBytes(const DevTables &t, bool sparse);
cudaError_t LaunchKmcChain(const DevTables &t, int8_t *species, const KmcDevState &s, const KmcLaunch &l,
                           cudaStream_t stream);

// prepare = false skips the shared-memory attribute call (already made by
// KmcOccupancy), so the launch can be recorded into a CUDA graph.
cudaError_t LaunchKmc(const DevTables &t, int8_t *species, const KmcDevState &s, const KmcLaunch &l,
                      cudaStream_t stream, bool prepare = true);
size_t KmcSharedBytes(const DevTables &t, const KmcLaunch &l);

// Surrogate training data (see surrogate_dataset_kernel).
// Feature encoding of the surrogate: each site's species becomes `width` channels, one of
// them 1. One-hot: the channel is the one-hot rank (width E'). Solute channels: the base
// species has no channel (its site is all zero) and the other ranks keep their order
// (width E' - 1); a network's first-layer bias absorbs the base, so both encodings give
// the same function class with E' - 1 / E' of the inputs.
struct FeatEnc {
  unsigned long long rank_ch;  // byte r: channel of one-hot rank r, 0xFF none
  int width;                   // channels per site
};
__host__ __device__ __forceinline__ int FeatChannel(const FeatEnc &f, int rank) {
  return static_cast<int>(static_cast<signed char>((f.rank_ch >> (8 * (rank & 7))) & 0xFFu));
}

struct SurrogateGen {
  unsigned long long seed;
  long long count;
  float solute_lo, solute_hi;  // per-sample solute fraction range
  int base_code;               // species filling the non-solute sites
  int kind;                    // 0 Quartic, 1 E0
  int in_pad;                  // feature row length (>= 59 x enc.width)
  FeatEnc enc;
  __nv_bfloat16 *features;     // [count][in_pad]
  float *ea;                   // [count]
  double *ea64, *de64;         // optional [count]
  int *status;
};
cudaError_t LaunchSurrogateDataset(const DevTables &t, const SurrogateGen &g, cudaStream_t stream);
// lmc_barrier_batch with the pair count on the device (at most m_max pairs).
cudaError_t LaunchBarrierBatchCounted(const DevTables &t, const int8_t *species, int n, const long long *pairs,
                                      int m_max, const int *m_dev, int kind, double *ea, double *de, int *status,
                                      cudaStream_t stream);
// Surrogate fallback: compact the pairs whose ensemble spread exceeds `threshold`
// (flag per pair, optional), then merge the plain barriers of those pairs into ea.
cudaError_t LaunchFallbackCompact(const long long *pairs, const float *mean, const float *spread, int m,
                                  float threshold, long long *fb_pairs, int *fb_index, int *count, uint8_t *flag,
                                  cudaStream_t stream);
cudaError_t LaunchFallbackMerge(const float *mean, int m, const double *fb_ea, const int *fb_index, const int *count,
                                double *ea, cudaStream_t stream);
cudaError_t LaunchSurrogateFeatures(const DevTables &t, const int8_t *species, int n, const long long *pairs, int m,
                                    int in_pad, const FeatEnc &enc, __nv_bfloat16 *features, int *status,
                                    cudaStream_t stream);
// fn 0: ExpFast and exp; fn 1: RcpFast and 1 / x, over n device doubles.
cudaError_t LaunchFastmathCheck(const DevTables &t, int fn, const double *x, long long n, double *fast, double *ref,
                                cudaStream_t stream);
// Resident blocks per SM and dynamic shared memory of the KMC launch `l`.
cudaError_t KmcOccupancy(const DevTables &t, const KmcLaunch &l, int *blocks_per_sm, size_t *shared_bytes);

// Reference-batch CMC (one block, mt19937_64 stream, batch = `batch` pairs, n >= 6).
struct CmcRefArgs {
  int n;
  double beta;
  unsigned long long attempts;
  int batch;
  uint32_t *rng;             // MT state
  double *energy;            // in/out
  double *energy_trace;      // optional: energy before every test (attempts + batch entries)
  unsigned long long *done;  // attempts done
  unsigned long long *accepted;
  int *status;
};
cudaError_t LaunchCmcReference(const DevTables &t, int8_t *species, const CmcRefArgs &a, cudaStream_t stream);

// Solute clusters (ansys::SoluteCluster): parent[i] = root site of i's 1NN-connected component
// of non-solvent sites (0xFFFFFFFF for solvent sites); n <= 1000 keeps ids below 2^32 - 1.
cudaError_t LaunchSoluteLabels(const DevTables &t, const int8_t *species, int n, int solvent, uint32_t *parent,
                               int *status, cudaStream_t stream);
// GetEnergyOfCluster of every cluster k on its sorted site set s_ids[s_off[k]..s_off[k+1]) (members
// and their 1-3NN shells) with the sorted members l_ids[l_off[k]..): energies[2k] with the members'
// species on a solvent background, energies[2k+1] with the solvent everywhere.
cudaError_t LaunchClusterCensus(const DevTables &t, const int8_t *species, int n, int solvent, long long clusters,
                                const long long *s_off, const long long *s_ids, const long long *l_off,
                                const long long *l_ids, double *energies, cudaStream_t stream);

// Jump energetics with the vacancy placed on each of a list of sites
// (ansys::ExitTime::GetJumpEnergetics / GetBarrierListAndExitTime).
struct SiteJumpArgs {
  int n;
  const long long *sites;   // [m] or null: every site (m = 4 n^3)
  long long m;
  long long vacancy;        // the lattice's own vacancy (replaced by `solvent`), -1 none
  int solvent;              // species code put on the own vacancy
  int barrier_kind;
  double beta_escape;       // 1 / kT of the exit-time rates
  double *ea12, *de12;      // [m][12] in id order of the neighbours, nullable
  long long *nb12;          // [m][12], nullable
  double *average, *exit_time;  // [m], nullable
  int *status;
  KmcSparse sp;
  int sparse;
};
cudaError_t LaunchSiteJumps(const DevTables &t, const int8_t *species, const SiteJumpArgs &a, cudaStream_t stream);

// Batched barriers with the sparse evaluation for runs of pairs that share a vacancy as first
// site (identical results to LaunchBarrierBatch; `sp` built for the lattice's dominant species).
struct BarrierGroupArgs {
  int n;
  const long long *pairs;  // [m][2] (device)
  long long m;
  const int *m_dev;        // device count that caps m, or null
  int kind;
  double *ea, *de;         // [m]
  double *d_or_e0, *ks;    // [m], nullable
  int *status;
  KmcSparse sp;
};
cudaError_t LaunchBarrierGroup(const DevTables &t, const int8_t *species, const BarrierGroupArgs &a,
                               cudaStream_t stream);

// Simulated annealing (SimulatedAnnealing.cpp:99-185): one warp, the reference's
// mt19937_64 stream, one trial pair per step and its adaptive temperature schedule.
struct SaState {
  unsigned long long steps, maximum_steps, last_improvement, last_reheat;
  unsigned long long reheat_trigger, reheat_cooldown, window_size;
  double temperature, beta, energy, lowest, recent_best;
  unsigned int window_trials, window_accepts, reheats_done, pad;
};
struct SaStepRec {
  long long site1, site2;
  int accepted, pad;
  double de, energy, temperature;  // dE of the trial; energy and temperature before the step
};
struct SaArgs {
  int n;
  unsigned long long steps;  // steps of this launch
  uint32_t *rng;             // MT state
  SaState *state;
  SaStepRec *trace;          // nullable, `steps` records
  volatile int *stop_flag;
  int *status;
};
cudaError_t LaunchSa(const DevTables &t, int8_t *species, const SaArgs &a, cudaStream_t stream);

// Throughput CMC (cooperative persistent grid, Philox, priority-resolved rounds).
struct CmcTpArgs {
  int n;
  double beta;
  unsigned long long attempts;
  int candidates;            // candidate pairs per round
  unsigned long long seed;
  unsigned long long *claim; // N words scratch (round-stamped priorities)
  long long *cand;           // 2 * candidates scratch
  double *energy_acc;        // per-block energy change accumulators (gridDim)
  unsigned long long *done;
  unsigned long long *accepted;
  int *quit;                 // device word, zero on entry
  int *status;
  volatile int *stop_flag;
  unsigned long long *rounds;  // nullable: rounds run (zero on entry)
};
// Warps of the throughput CMC grid that fit on the device at once (0 on error).
int CmcThroughputResidentWarps(const DevTables &t, int device);
cudaError_t LaunchCmcThroughput(const DevTables &t, int8_t *species, const CmcTpArgs &a, int device,
                                cudaStream_t stream);

// first_x (may be null) must be preset to INT64_MAX and hist (num_replicas x (kMaxSpecies + 1),
// the last column counting codes outside the alphabet) to 0.
cudaError_t LaunchReplicaScan(const int8_t *species, const long long *lat_off, const int *lat_n, int num_replicas,
                              int x_code, int num_species, long long *first_x, unsigned long long *hist,
                              cudaStream_t stream);

// Scratch of the allocation-free census: a file-scope device array of
// kNoAllocMaxTheta counters followed by one word that counts sites skipped for
// species codes outside the alphabet. Returns its device address for `device`,
// which must be the current device; the lookup happens on the first call per
// device.
constexpr int kNoAllocMaxTheta = 512;
constexpr int kNoAllocScratchWords = kNoAllocMaxTheta + 1;
constexpr int kNoAllocMaxDevices = 64;
cudaError_t NoAllocCensusScratch(int device, unsigned long long **ptr);
// The census of LaunchCensus on a caller-owned species array whose codes are not
// trusted: clears the kNoAllocScratchWords words of `scratch` (from
// NoAllocCensusScratch), skips sites whose neighbourhood holds a code outside
// [0, num_species) and writes NaN to *energy when any site was skipped.
cudaError_t LaunchCensusCheckedNoAlloc(const DevTables &t, const int8_t *species, int n, int base_code,
                                       unsigned long long *scratch, double *energy, cudaStream_t stream);

// Host-side reference seeding of std::mt19937_64 (state words for the device).
void MtSeed(uint64_t seed, uint32_t *words);

}  // namespace lmc
