/*
 * lmc_gb300.h - C ABI of the GB300-native lattice Monte Carlo hot path.
 *
 * Plain C types only (pointers, sizes, int status codes); no C++ or PyTorch
 * types cross this boundary. Every call returns LMC_OK (0) or an lmc_status
 * code; lmc_last_error() gives the message of the calling thread's last
 * failure. Nothing throws across the ABI.
 *
 * Lattices are perfect cubic FCC supercells of n x n x n conventional cells
 * (4 n^3 sites) addressed by the lattice ids the reference assigns after
 * Config::ReassignLatticeVector (lmc/cfg/src/Config.cpp:466-552), i.e.
 * id = hx * 2n^2 + hy * n + hz / 2 in half-lattice coordinates. Species are
 * int8 codes: the rank of the element's name in the string order of the
 * model's alphabet, which is the barrier element set plus "X" (vacancy), the
 * same order as the reference's std::set<Element> (lmc/cfg/include/Element.hpp:44-49).
 *
 * Threading: a context owns one CUDA stream on one device; calls on one
 * context must be serialised by the caller, distinct contexts are independent.
 */
#ifndef LMC_GB300_H_
#define LMC_GB300_H_
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum lmc_status {
  LMC_OK = 0,
  LMC_ERR_INVALID_ARGUMENT = 1, /* std::invalid_argument / std::runtime_error in the reference */
  LMC_ERR_OUT_OF_RANGE = 2,     /* std::out_of_range (.at(), ClusterIndexer::GetIndex, GetPairFlatIndex) */
  LMC_ERR_IO = 3,               /* "Cannot open <file>" */
  LMC_ERR_CUDA = 4,             /* CUDA runtime failure */
  LMC_ERR_NO_DEVICE = 5,        /* no CUDA device / extension unusable */
  LMC_ERR_NUMERIC = 6,          /* NaN / inf / non-positive total rate detected on the device */
  LMC_ERR_STOPPED = 7,          /* run stopped by lmc_request_stop or a device wait limit */
  LMC_ERR_UNSUPPORTED = 8       /* input outside the supported domain (e.g. n < 6) */
} lmc_status;

const char *lmc_strerror(int status);
const char *lmc_last_error(void);
const char *lmc_version(void);

/* ------------------------------------------------------------------------- */
/* Model: element alphabet + coefficient file contents                        */
/* ------------------------------------------------------------------------- */
typedef struct lmc_model lmc_model;

/* Quartic barrier parameters of one migrating element
 * (ParametersQuartic, lmc/pred/include/EnergyUtility.h:73-86). */
typedef struct lmc_quartic_params {
  int k_mmm, k_mm2;                   /* rows of U_mmm / U_mm2 */
  const double *mu_x_mmm, *sigma_x_mmm; /* f_mmm each */
  const double *mu_x_mm2, *sigma_x_mm2; /* f_mm2 each */
  const double *u_mmm;                /* k_mmm x f_mmm, row-major */
  const double *u_mm2;                /* k_mm2 x f_mm2, row-major */
  const double *theta_d;              /* k_mmm */
  const double *theta_ks;             /* k_mm2 */
  double mu_d, sigma_d, mu_ks, sigma_ks;
} lmc_quartic_params;

/* E0 barrier parameters (ParametersE0, EnergyUtility.h:88-95). */
typedef struct lmc_e0_params {
  int k_mmm;
  const double *mu_x_mmm, *sigma_x_mmm; /* f_mmm each */
  const double *u_mmm;                  /* k_mmm x f_mmm, row-major */
  const double *theta_e0;               /* k_mmm */
  double mu_e0, sigma_e0;
} lmc_e0_params;

/* Creates a model for the barrier element set `element_names` (the reference's
 * `element_set` parameter-file key, e.g. {"Al","Mg","Zn"}); "X" is added to the
 * species alphabet automatically. Replaces the element-set handling of the
 * predictor constructors (VacancyMigrationPredictorQuartic.cpp:16-37). */
int lmc_model_create(const char *const *element_names, int num_elements, lmc_model **out);
/* Parses a reference coefficient JSON ("Base".theta plus per-element Quartic
 * and, when present, E0 blocks) into a new model: the constructors'
 * JSON handling (VacancyMigrationPredictorQuartic.cpp:38-63,
 * VacancyMigrationPredictorE0.cpp:22-40, EnergyPredictor.cpp:24-33). */
int lmc_model_load_json(const char *path, const char *const *element_names, int num_elements, lmc_model **out);
void lmc_model_destroy(lmc_model *model);
/* Species alphabet size (element set + X) and the code of a name (-1 if absent). */
int lmc_model_num_species(const lmc_model *model);
int lmc_model_species_code(const lmc_model *model, const char *name);
/* Writes the alphabet as a space-separated string. */
int lmc_model_alphabet(const lmc_model *model, char *buf, int buflen);
/* Layout: length of "Base".theta, MMM and MM2 feature counts. */
int lmc_model_layout(const lmc_model *model, int *num_theta, int *f_mmm, int *f_mm2);
/* Orbit size of every MMM (which=0) or MM2 (which=1) feature: feature value =
 * one-hot numerator / orbit size (GetOneHotParametersFromMap, EnergyUtility.cpp:790-792). */
int lmc_model_feature_orbit_sizes(const lmc_model *model, int which, int32_t *sizes);
int lmc_model_set_base_theta(lmc_model *model, const double *theta, int n);
int lmc_model_set_quartic(lmc_model *model, const char *migrant, const lmc_quartic_params *p);
int lmc_model_set_e0(lmc_model *model, const char *migrant, const lmc_e0_params *p);

/* ------------------------------------------------------------------------- */
/* Host-only queries (no GPU needed): geometry and encodings                  */
/* ------------------------------------------------------------------------- */
/* Sorted 1/2/3NN ids of `site` in an n^3 supercell (Config.cpp:955-1045): 42 ids. */
int lmc_geom_neighbors(int n, int64_t site, int64_t *out42);
/* Sorted id lists of a 1NN pair (GetSortedLatticeVectorStateOfPair and
 * GetSymmetricallySortedLatticeVector{MMM,MM2}, EnergyUtility.cpp:45-104,261-287). */
int lmc_geom_pair_lists(int n, int64_t first, int64_t second, int64_t *state60, int64_t *mmm58, int64_t *mm258);
/* Sorted 1-3NN id list of a site (GetSortedLatticeVectorStateOfSite): 43 ids. */
int lmc_geom_site_list(int n, int64_t site, int64_t *out43);
/* Cluster-mapping sizes: counts[0..7] state-pair clusters per label,
 * counts[8..15] site clusters per label, counts[16] MMM orbits, counts[17] MM2
 * orbits, counts[18] MMM clusters, counts[19] MM2 clusters. */
int lmc_geom_mapping_sizes(int *counts20);
/* Flattened MMM (which=0) / MM2 (which=1) mapping: per cluster (orbit, a, b),
 * b = -1 for singlets; `cap` clusters at most. Returns the cluster count in *n. */
int lmc_geom_env_mapping(int which, int32_t *orbit_a_b, int cap, int *n);

/* Integer encodings of a 1NN jump pair on a host lattice (species codes):
 * the ElementCluster start/end counts behind GetDe (num_theta each,
 * VacancyMigrationPredictorQuartic.cpp:112-166) and the MMM / MM2-forward /
 * MM2-backward one-hot numerators (feature value = numerator / orbit size,
 * EnergyUtility.cpp:743-796). Any pointer may be NULL. */
int lmc_host_encode_pair(const lmc_model *model, int n, const int8_t *species, int64_t first, int64_t second,
                         int32_t *state_start, int32_t *state_end, int32_t *mmm, int32_t *mm2_fwd,
                         int32_t *mm2_bwd);

/* ------------------------------------------------------------------------- */
/* Device context                                                            */
/* ------------------------------------------------------------------------- */
typedef struct lmc_ctx lmc_ctx;

/* Uploads the model's folded coefficient tables to `device` and creates the
 * context's stream. Fails with LMC_ERR_NO_DEVICE when no GPU is usable. */
int lmc_ctx_create(const lmc_model *model, int device, lmc_ctx **out);
void lmc_ctx_destroy(lmc_ctx *ctx);
int lmc_ctx_synchronize(lmc_ctx *ctx);

/* Lattices ("replicas"): R cubic supercells with edges n[r] (6 <= n <= 1000),
 * species concatenated in replica order (host pointer). Replaces the Config
 * species storage read by Config::GetElementAtLatticeId (Config.cpp:132-135). */
int lmc_ctx_set_lattices(lmc_ctx *ctx, int num_replicas, const int32_t *n, const int8_t *species);
int lmc_ctx_get_lattices(lmc_ctx *ctx, int8_t *species);
/* Total sites over all replicas and the site offset of replica r. */
int64_t lmc_ctx_total_sites(const lmc_ctx *ctx);
int64_t lmc_ctx_replica_offset(const lmc_ctx *ctx, int replica);
/* Device address of the species arena (for device-resident callers). */
void *lmc_ctx_species_device_ptr(lmc_ctx *ctx);

/* Barrier predictors over a batch of 1NN pairs (first = vacancy site,
 * second = migrating atom) of one replica; host arrays of length m.
 * kind 0 = Quartic (VacancyMigrationPredictorQuartic::GetBarrierAndDiffFromLatticeIdPair,
 * VacancyMigrationPredictorQuartic.cpp:247-276), kind 1 = E0
 * (VacancyMigrationPredictorE0.cpp:153-159). d / ks (Quartic) or e0 (E0) may be NULL. */
#define LMC_BARRIER_QUARTIC 0
#define LMC_BARRIER_E0 1
int lmc_barrier_batch(lmc_ctx *ctx, int replica, int kind, const int64_t *pairs, int m, double *ea, double *de,
                      double *d_or_e0, double *ks);
/* Device-resident variant: pairs/outputs are device pointers, asynchronous on the context stream. */
int lmc_barrier_batch_device(lmc_ctx *ctx, int replica, int kind, const int64_t *pairs_dev, int m, double *ea_dev,
                             double *de_dev);
/* Evaluation used by the barrier batch entry points (and the surrogate's fallback), identical
 * results either way: LMC_EVAL_SPARSE (default) evaluates each run of consecutive pairs that
 * share a vacancy as first site once, with the solvent-relative sparse sums (the way
 * KineticMcFirstOmp::BuildEventList asks for a vacancy's 12 jumps, KineticMcFirstOmp.cpp:57-64);
 * LMC_EVAL_DENSE sums every cluster of every pair. No reference counterpart (a GPU choice). */
int lmc_ctx_set_barrier_evaluation(lmc_ctx *ctx, int evaluation);

/* Integer encodings of a batch of 1NN jump pairs computed on the device (same
 * layout as lmc_host_encode_pair, m consecutive records per array). */
int lmc_encode_batch(lmc_ctx *ctx, int replica, const int64_t *pairs, int m, int32_t *state_start,
                     int32_t *state_end, int32_t *mmm, int32_t *mm2_fwd, int32_t *mm2_bwd);

/* Pair-swap energy change (EnergyChangePredictorPairSite::GetDeFromLatticeIdPair,
 * EnergyChangePredictorPairSite.cpp:69-192) for a batch of arbitrary site pairs. */
int lmc_de_pairs(lmc_ctx *ctx, int replica, const int64_t *pairs, int m, double *de);

/* Total energy (EnergyPredictor::GetEnergy, EnergyPredictor.cpp:40-96,173-177)
 * of one replica; counts (num_theta int64, may be NULL) receives the integer
 * cluster census behind it. */
int lmc_energy(lmc_ctx *ctx, int replica, double *energy, int64_t *counts);

/* Allocation-free variant of lmc_energy. It has no counterpart in the
 * reference. It serves callers that cannot allocate device memory at the call
 * site: a host application whose own pool allocator already owns the GPU's
 * memory and forbids other cudaMalloc calls, a plugin run under a fixed memory
 * budget, or a stepping loop where cudaMalloc / cudaFree would synchronise the
 * device and stall its other streams.
 * species_dev: the caller's device array of 4 n^3 species codes (lattice ids
 * as above); energy_dev: the caller's device double that receives the energy.
 * The call allocates nothing: the cluster counters live in one static device
 * array of 512 counters plus one status word per GPU (about 4 KiB, held by
 * every GPU that loads the library until the process exits); models with more
 * cluster types are rejected with LMC_ERR_UNSUPPORTED, edges outside [6, 1000]
 * likewise. The first call on a device looks the array up
 * (cudaGetSymbolAddress) with that device current and keeps the address for
 * the life of the process: make that first call before any stream capture,
 * and do not call it again on a device after cudaDeviceReset. The species
 * codes are checked on the device: if any code lies outside [0, number of
 * species), energy_dev receives NaN (no status is returned, because the call
 * does not wait for the GPU). The work is queued on the context's stream and
 * the call returns without waiting (lmc_ctx_synchronize before reading
 * energy_dev). Every call shares the array and clears it first, so calls that
 * overlap on the GPU (other streams, other contexts on the same device) race
 * and must be serialised by the caller. */
int lmc_energy_noalloc(lmc_ctx *ctx, const int8_t *species_dev, int n, double *energy_dev);

/* Self-check of the device FP64 helpers the barrier epilogue, the rates and the
 * clock use (GB300 runs FP64 at 1/64 of the FP32 rate): fn 0 evaluates the
 * table-driven exponential and CUDA's exp, fn 1 the Newton reciprocal and
 * 1.0 / x, on n host doubles. No reference counterpart (numerics test hook). */
int lmc_fastmath_check(lmc_ctx *ctx, int fn, const double *x, int64_t n, double *fast, double *ref);

/* ------------------------------------------------------------------------- */
/* Learned barrier surrogate (no reference counterpart: the plain predictor    */
/* above is its fallback and the yardstick of its error)                      */
/* ------------------------------------------------------------------------- */
/* Ensemble of `members` MLPs in -> hidden -> hidden -> 1 (GELU), BF16 weights and
 * activations on the tensor cores, FP32 accumulation, FP32 master weights, Adam.
 * Features (bf16 rows, passed as uint16_t): channels of the 58 MMM-ordered
 * environment sites of a jump (VacancyMigrationPredictorQuartic's MMM list), then of
 * the migrant, zero padded to in_features (a multiple of 64); the context's encoding
 * (lmc_surrogate_set_encoding) sets the channels. */
typedef struct lmc_mlp lmc_mlp;
int lmc_mlp_create(int device, int in_features, int hidden, int members, uint64_t seed, lmc_mlp **out);
void lmc_mlp_destroy(lmc_mlp *mlp);
int lmc_mlp_layout(const lmc_mlp *mlp, int *in_features, int *hidden, int *members, int64_t *num_params);
/* Flat FP32 parameters in the order W1 [M*H][in], b1 [M*H], W2 [M][H][H], b2 [M*H], w3 [M*H], b3 [M]. */
int lmc_mlp_get_params(lmc_mlp *mlp, float *params);
int lmc_mlp_set_params(lmc_mlp *mlp, const float *params);
/* Labels are standardised as (ea - mean) / std inside; predictions come back in eV. */
int lmc_mlp_set_label_scale(lmc_mlp *mlp, float mean, float std_dev);
/* Gradients (flat, parameter order) of every member's mean squared error on one batch
 * (host arrays; batch a multiple of 64), and the per-member loss. Nothing is updated. */
int lmc_mlp_gradients(lmc_mlp *mlp, const uint16_t *features, const float *labels, int batch, float *grad,
                      float *loss);
/* Trains every member on the same shuffled batches (device arrays, n samples); loss
 * (nullable, per member) is the mean loss of the last epoch in standardised units. */
int lmc_mlp_train(lmc_mlp *mlp, const uint16_t *features_dev, const float *labels_dev, int64_t n, int batch,
                  int epochs, float lr, uint64_t seed, float *loss);
/* Training GEMM kernels: 0 (default) the tcgen05 kernel (BF16 operands, FP32 accumulators in
 * TMEM) for every GEMM whose rows are a multiple of 128 (batch and hidden widths), the mma.sync
 * kernel otherwise; 1 the mma.sync kernel for all. Same arithmetic (BF16 products, FP32 sums). */
int lmc_mlp_set_train_path(lmc_mlp *mlp, int path);
/* Inference kernels: 0 automatic (tcgen05 where a kernel serves the network: feature rows
 * for hidden = 256 and in_features <= 256; lattice jumps, features gathered inside the
 * kernel, for 2 members of 128 -> 128 -> 128 with solute-channel features of a
 * three-species alphabet), 1 tcgen05, 2 the mma.sync GEMMs of training. */
int lmc_mlp_set_inference_path(lmc_mlp *mlp, int path);
/* Ensemble mean and spread (max - min over members), eV, for n feature rows (device arrays). */
int lmc_mlp_predict(lmc_mlp *mlp, const uint16_t *features_dev, int64_t n, float *mean_dev, float *spread_dev);

/* Feature encodings of the surrogate (per site, one channel set to 1):
 * ONEHOT  the one-hot rank of the species (E' channels, E' = one-hot alphabet size);
 * SOLUTE  one channel per species other than the base (the solvent, Al when present):
 *         E' - 1 channels, a base site is all zero. A network's first-layer bias absorbs
 *         the base, so both encodings describe the same function class. */
#define LMC_FEATURES_ONEHOT 0
#define LMC_FEATURES_SOLUTE 1
/* Encoding of the context's surrogate features, datasets and lattice-jump inference
 * (default ONEHOT). A network must be used with the encoding it was trained on. */
int lmc_surrogate_set_encoding(lmc_ctx *ctx, int encoding);
/* Feature row length of a context's model and encoding: at least 59 x the channels per
 * site, padded to 64. */
int lmc_surrogate_feature_count(const lmc_ctx *ctx, int *min_features, int *padded_features);
/* Training data: `count` seeded random neighbourhoods (solute fraction ~ U(solute_lo, solute_hi),
 * solutes equally likely, the rest the base element), their features and the plain
 * predictor's barrier (ea_dev float; ea64_dev / de64_dev optional double). Device arrays. */
int lmc_surrogate_dataset(lmc_ctx *ctx, uint64_t seed, int64_t count, double solute_lo, double solute_hi, int kind,
                          int in_features, uint16_t *features_dev, float *ea_dev, double *ea64_dev, double *de64_dev);
/* Features of lattice jumps (pairs first -> second, device arrays). */
int lmc_surrogate_features(lmc_ctx *ctx, int replica, const int64_t *pairs_dev, int m, int in_features,
                           uint16_t *features_dev);
/* The network alone on m lattice jumps (device arrays): ensemble mean and spread (max - min
 * over members), eV. Rows that the network cannot describe (a pair that is not a 1NN jump,
 * an environment with a second vacancy) get spread +inf in the fused kernel. */
int lmc_surrogate_predict_device(lmc_ctx *ctx, lmc_mlp *mlp, int replica, const int64_t *pairs_dev, int m,
                                 float *mean_dev, float *spread_dev);
/* Surrogate barriers of m jumps (device arrays): the ensemble mean, or the plain predictor
 * (lmc_barrier_batch) where the ensemble spread exceeds threshold_ev; fallback_dev (nullable)
 * flags those pairs and num_fallback (nullable) counts them. */
int lmc_surrogate_barrier_batch_device(lmc_ctx *ctx, lmc_mlp *mlp, int replica, int kind, const int64_t *pairs_dev,
                                       int m, float threshold_ev, double *ea_dev, uint8_t *fallback_dev,
                                       int *num_fallback);

/* ------------------------------------------------------------------------- */
/* Kinetic MC (KineticMcFirstOmp semantics, KineticMcAbstract.cpp:140-190)    */
/* ------------------------------------------------------------------------- */
#define LMC_RNG_MT19937_64 0 /* std::mt19937_64 + libstdc++ distributions: same stream as the reference */
#define LMC_RNG_PHILOX 1     /* Philox4x32-10 counter-based, one stream per replica */

typedef struct lmc_kmc_options {
  int rng;                 /* LMC_RNG_* */
  uint64_t seed;           /* replica r uses seed + r */
  int barrier_kind;        /* LMC_BARRIER_QUARTIC or LMC_BARRIER_E0 */
  int rate_corrector;      /* RateCorrector time factor (RateCorrector.hpp:17-24) */
  const double *tt_time;   /* optional T(t) table (TimeTemperatureInterpolator), NULL if unused */
  const double *tt_temp;
  int tt_len;
  int warps_per_replica;   /* 0 = autotuned */
  int replicas_per_block;  /* 0 = autotuned */
  int evaluation;          /* LMC_EVAL_SPARSE (default) or LMC_EVAL_DENSE; identical results */
  int early_stop;          /* IsEscaped (KineticMcAbstract.cpp:192-223): a replica whose vacancy has only
                              solvent (its most frequent element) in the 1-3NN shells completes that step
                              and takes no further steps */
  int chain;               /* 1: second-order residence-time KMC of KineticMcChainOmpi
                              (KineticMcChainOmpi.cpp:56-152): per step the 12 x 12 jumps after each
                              first jump, deterministic second-order time, one uniform draw for the
                              selection; one block of 12 warps per replica. Not combined with early_stop,
                              lmc_kmc_run_graph or lmc_kmc_autotune; no events12 output. */
  int rates;               /* LMC_RATES_FP32 (default) or LMC_RATES_FP64, for the first-order KMC on
                              LMC_RNG_PHILOX streams: FP32 barriers and rates (within 1e-6 relative of the
                              FP64 ones), FP64 rate sum and clock, exact energy sums. The reference's
                              mt19937_64 stream and the chain KMC always use FP64; the multi-vacancy
                              KMC takes lmc_kmc_multi_set_rates. */
} lmc_kmc_options;

#define LMC_RATES_FP32 0
#define LMC_RATES_FP64 1

/* Jump evaluation inside the KMC kernel: both give bit-identical barriers.
 * Sparse: constant all-solvent sums plus corrections for the clusters that touch
 * a non-solvent site (fast for dilute alloys). Dense: every cluster term. */
#define LMC_EVAL_SPARSE 0
#define LMC_EVAL_DENSE 1

/* Per-step record of replica `trace_replica` (for parity checks and logs). */
typedef struct lmc_kmc_step {
  int64_t vacancy;     /* vacancy site before the step */
  int64_t target;      /* selected neighbour (lattice id) */
  int32_t selected;    /* index in the id-sorted 1NN list */
  int32_t slot;        /* vacancy slot that moved (multi-vacancy runs; 0 otherwise) */
  double ea, de;       /* barrier and energy change of the selected event */
  double total_rate;   /* sum of exp(-Ea beta) over the 12 events (no prefactor) */
  double time;         /* simulated time after the step */
  double energy;       /* energy after the step */
} lmc_kmc_step;

/* Initialises KMC state for every replica (the KineticMcFirstAbstract constructor,
 * KineticMcAbstract.cpp:5-50): temperature[r] (K), vacancy = the lowest-id X site, time = 0,
 * energy = 0. */
int lmc_kmc_init(lmc_ctx *ctx, const double *temperature, const lmc_kmc_options *opt);
/* KineticMcFirstAbstract::Simulate's step loop (KineticMcAbstract.cpp:140-190,
 * KineticMcFirstOmp.cpp:52-82): runs `steps` steps on every replica in one persistent launch. If trace is
 * non-NULL it receives `steps` records of replica trace_replica; events12
 * (NULL or 12 * 3 * steps doubles: target id, Ea, dE per id-sorted event)
 * receives the full event lists of that replica. */
int lmc_kmc_run(lmc_ctx *ctx, uint64_t steps, int trace_replica, lmc_kmc_step *trace, double *events12);
/* Per-replica state (any pointer may be NULL). */
int lmc_kmc_get_state(lmc_ctx *ctx, int64_t *vacancy, uint64_t *steps, double *time, double *energy);
/* Per replica 1 when its trajectory ended by the early stop (KineticMcAbstract.cpp:213-220), else 0. */
int lmc_kmc_get_escaped(lmc_ctx *ctx, uint8_t *escaped);
/* Device time (ms) of the last lmc_kmc_run / lmc_cmc_run launch (CUDA events on the context stream). */
int lmc_last_run_ms(lmc_ctx *ctx, double *ms);
/* Launch shape of lmc_kmc_run under the current options: warps per replica,
 * replicas per block, resident blocks per SM and dynamic shared memory per
 * block. No reference counterpart (GPU launch introspection, used by the
 * autotuner and the benchmark record). Any output may be NULL. */
int lmc_kmc_launch_info(lmc_ctx *ctx, int *warps_per_replica, int *replicas_per_block, int *blocks_per_sm,
                        int64_t *shared_bytes);
/* Runs `launches` x `steps_per_launch` steps on every replica as one CUDA graph
 * (status clear, the persistent KMC launches, status copy to pinned host memory),
 * recorded on the first call and replayed while the launch arguments are
 * unchanged. Same results as `launches` calls of lmc_kmc_run(steps_per_launch)
 * without a trace. Replaces the per-step driver loop of
 * KineticMcFirstAbstract::Simulate (KineticMcAbstract.cpp:182-190). */
int lmc_kmc_run_graph(lmc_ctx *ctx, uint64_t steps_per_launch, int launches);
/* Picks the KMC launch shape (warps per replica, replicas per block, sparse or
 * dense evaluation) by timing every shape the kernel accepts for `probe_steps`
 * steps on a copy of this context's state (the state is restored), and stores
 * the choice in the context's options. With a non-empty cache_path the choice is
 * read from / written to that JSON file, keyed by the GPU, its SM count, the
 * replica count and the histogram of supercell sizes (plus the options that
 * change the kernel's work). All shapes give identical results. No reference
 * counterpart (GPU launch tuning). Any output may be NULL. */
int lmc_kmc_autotune(lmc_ctx *ctx, uint64_t probe_steps, const char *cache_path, int *warps_per_replica,
                     int *replicas_per_block, int *evaluation, int *from_cache);

/* Multi-vacancy KMC (no reference counterpart: KineticMcFirstOmp tracks the
 * first vacancy only, Config.cpp:298-310, and its encodings throw when a second
 * vacancy enters a jump environment, EnergyUtility.cpp:784). Every X site of a
 * lattice is a tracked vacancy ("slot", ascending site id at init, 1 to 256 per
 * lattice); each step chooses one event among all slots x 12 jumps by residence
 * time (rates and clock as KineticMcFirstOmp, Philox stream per lattice) and
 * moves that vacancy. A second vacancy inside a jump's neighbourhood
 * contributes nothing to its encodings (clusters with two vacancies have no
 * coefficients, a vacancy has no one-hot slot); a jump onto a vacancy has rate
 * 0. One block per lattice; replaces KineticMcAbstract.cpp:140-190 for this case. */
int lmc_kmc_multi_init(lmc_ctx *ctx, const double *temperature, uint64_t seed, int barrier_kind, int evaluation);
/* Runs `steps` steps on every lattice; trace (NULL or `steps` records) receives
 * lattice trace_replica's events, `slot` naming the vacancy that moved. */
int lmc_kmc_multi_run(lmc_ctx *ctx, uint64_t steps, int trace_replica, lmc_kmc_step *trace);
/* Arithmetic of the following lmc_kmc_multi_run calls: LMC_RATES_FP64 (the default; the oracle's
 * operations exactly) or LMC_RATES_FP32 (barriers and rates in FP32, within 1e-6 relative of the
 * FP64 ones; rate sums and the clock in FP64; energy sums exact in fixed point). The trajectories
 * agree except where a draw falls within the rates' rounding of an event boundary. */
int lmc_kmc_multi_set_rates(lmc_ctx *ctx, int rates);
/* First slot of every lattice, R + 1 entries (the last is the slot count). */
int lmc_kmc_multi_slots(lmc_ctx *ctx, int32_t *slot_offsets);
/* Vacancy site of every slot and per-lattice steps, time, energy (any may be NULL). */
int lmc_kmc_multi_get_state(lmc_ctx *ctx, int64_t *vacancies, uint64_t *steps, double *time, double *energy);
/* Surrogate-assisted multi-vacancy KMC: `steps` steps of lmc_kmc_multi_run on a context holding
 * one lattice (lmc_kmc_multi_init with the Quartic barrier), with the barriers of the jumps whose
 * environment changed taken from the ensemble `mlp` (the fused jump kernel: the context's
 * solute-channel encoding, 2 members of hidden 128), and from the plain predictor where the
 * ensemble spread exceeds threshold_ev or the network does not describe the jump. The energy
 * change of each selected jump is the plain predictor's, so the energy sums stay exact; with
 * threshold_ev = 0 the trajectory is lmc_kmc_multi_run's. trace (nullable, `steps` records)
 * receives the events with the barrier used; plain_barrier (nullable, `steps` values) the plain
 * predictor's barrier of each selected event; num_fallback (nullable) the jumps that took the
 * plain predictor. No reference counterpart for the network (KineticMcAbstract.cpp:140-190 for
 * the step loop). */
int lmc_kmc_multi_surrogate_run(lmc_ctx *ctx, lmc_mlp *mlp, uint64_t steps, float threshold_ev,
                                lmc_kmc_step *trace, double *plain_barrier, uint64_t *num_fallback);

/* ------------------------------------------------------------------------- */
/* Vacancy placed on every site: ExitTime's barrier queries (ansys)          */
/* ------------------------------------------------------------------------- */
/* ansys::ExitTime::GetJumpEnergetics (ExitTime.cpp:257-310) and GetBarrierListAndExitTime
 * (:217-255) in one pass: the lattice's own vacancy (its first X) gets `solvent_code`, then for
 * each listed site (sites NULL = every site, m ignored) the vacancy is put there and its 12 jumps
 * are evaluated (Quartic or E0). Outputs, host pointers, any may be NULL: ea12 / de12 / nb12
 * [m][12] in the id order of the neighbours (the adjacency-list order), average [m] = mean
 * barrier, exit_time [m] = 1 / sum exp(-Ea / (kB T_escape)) / 1e13, both over the barriers in
 * ascending order. No reference counterpart as one call; one warp per site. */
int lmc_site_jump_energetics(lmc_ctx *ctx, int replica, int kind, int solvent_code, double escape_temperature,
                             const int64_t *sites, int64_t m, double *ea12, double *de12, int64_t *nb12,
                             double *average, double *exit_time);

/* EnergyChangePredictorPairSite::GetDeFromAtomIdSite / GetDeFromLatticeIdSite
 * (EnergyChangePredictorPairSite.cpp:148-192) for m queries on lattice `replica`: the energy change
 * of replacing the species at sites[q] (taken as from_codes[q], or the lattice's own when
 * from_codes is NULL) by to_codes[q], the lattice read as if fill_site (when >= 0) held fill_code.
 * Host arrays; one GPU warp per query. The building block of ExitTime::GetBindingEnergy and
 * GetProfileEnergy (ExitTime.cpp:401-511): fill_site = the vacancy, fill_code = the solvent. */
int lmc_site_de_batch(lmc_ctx *ctx, int replica, const int64_t *sites, const int8_t *from_codes,
                      const int8_t *to_codes, int64_t m, int64_t fill_site, int fill_code, double *de);

/* ExitTime::GetBindingEnergy and GetProfileEnergy (ExitTime.cpp:401-511) for every site of lattice
 * `replica`, the lattice's vacancy (its first X) read as `solvent_code`: binding [E - 1][N] (rows in
 * ascending order of the non-X species codes) = dE(site: e -> X) - (mu_X - mu_e); profile [N] =
 * dE(site: own -> X) + mu_own - mu_X, at the vacancy the largest dE(e -> X) + mu_e - mu_X.
 * chemical_potential per species code (EnergyPredictor::GetChemicalPotential); host outputs, either
 * may be NULL. One GPU warp per site, every element's sum from one pass over the site's clusters;
 * at most 5 elements besides X. */
int lmc_exit_time_energies(lmc_ctx *ctx, int replica, int solvent_code, const double *chemical_potential,
                           double *binding, double *profile);

/* ExitTime::GetExitTimeInfo's per-cluster quantities (ExitTime.cpp:53-128) for `num_clusters`
 * clusters of lattice `replica` given as CSR lattice-id lists (offsets [num_clusters + 1],
 * members; e.g. from lmc_solute_cluster_get). For each cluster S and its first-neighbour shell T:
 * markov_escape_time = ExitTime::BuildMarkovChain (ExitTime.cpp:165-216) over the states S u T
 * (start probabilities ~ exp(-profile_energy beta_escape), rates 1e13 exp(-Ea beta_escape), jumps
 * out of S u T absorbing), neighbor_size = |T|, barriers [num_clusters][8] = the mean and the
 * population standard deviation of Ea - dE / 2 over the jumps in / to / on / off the cluster
 * (GetAverageBarriers, ExitTime.cpp:311-399; NaN when a category is empty) and
 * effective_binding_energy = -ln(escape_time 1e13) / beta_escape + mean_off (ExitTime.cpp:121).
 * profile_energy: the lattice's per-site profile energies (lmc_exit_time_energies). The barriers
 * are the Quartic ones of lmc_site_jump_energetics (the lattice's vacancy read as solvent_code) on
 * the GPU; each chain's linear system is solved on the host (at most 4096 states). Any output may
 * be NULL. */
int lmc_exit_time_clusters(lmc_ctx *ctx, int replica, int solvent_code, double escape_temperature,
                           const int64_t *offsets, const int64_t *members, int64_t num_clusters,
                           const double *profile_energy, double *markov_escape_time, int64_t *neighbor_size,
                           double *barriers, double *effective_binding_energy);

/* ------------------------------------------------------------------------- */
/* Solute clusters (ansys::SoluteCluster)                                     */
/* ------------------------------------------------------------------------- */
/* ansys::SoluteCluster::FindAtomListOfClusters (SoluteCluster.cpp:277-373) on lattice `replica`:
 * the 1NN-connected components of the sites whose species is not `solvent_code` (vacancies
 * included), those with fewer than `smallest` sites dropped; a component of more than
 * `solvent_bond` sites gains every site of its 1NN shell that has more than `solvent_bond` 1NN
 * bonds to its non-solvent sites (such a solvent site may join several clusters). Clusters are
 * ordered by size, larger first, equal sizes by their smallest site id (the reference leaves
 * that order to std::sort over hash-set order); members are sorted by id. With
 * `chemical_potential` (per species code, as EnergyPredictor::GetChemicalPotential; NULL skips
 * it) each cluster also gets SoluteCluster::GetFormationEnergy (:395-410): GetEnergyOfCluster
 * (EnergyPredictor.cpp:97-184) with the members' species on a solvent background minus that of
 * the pure solvent, minus the members' chemical potentials (a cluster of the census holding two
 * vacancies counts nothing, where the reference's ClusterIndexer throws). The results are kept in the context:
 * num_clusters and num_members size the buffers of lmc_solute_cluster_get. Components are found
 * by union-find on the GPU, the energies by one GPU block per cluster. */
int lmc_solute_clusters(lmc_ctx *ctx, int replica, int solvent_code, int64_t smallest, int64_t solvent_bond,
                        const double *chemical_potential, int64_t *num_clusters, int64_t *num_members);
/* Copies the last lmc_solute_clusters result (host pointers, any may be NULL): offsets
 * [num_clusters + 1], members [num_members], formation_energy [num_clusters] (NaN without
 * chemical potentials). */
int lmc_solute_cluster_get(lmc_ctx *ctx, int64_t *offsets, int64_t *members, double *formation_energy);

/* ------------------------------------------------------------------------- */
/* Simulated annealing (SimulatedAnnealing.cpp:99-185, a next row of the path) */
/* ------------------------------------------------------------------------- */
/* Per-step record: the trial pair, whether it was accepted, its dE, and the
 * energy and temperature before the step (what Dump logs, SimulatedAnnealing.cpp:78-97). */
typedef struct lmc_sa_step {
  int64_t site1, site2;
  int32_t accepted;
  int32_t pad;
  double de, energy, temperature;
} lmc_sa_step;
/* Starts an annealing run on lattice `replica`: mt19937_64 seeded with `seed` (the reference seeds
 * from the clock, McAbstract.cpp:32), schedule lengths from maximum_steps (window 0.1 %, reheat
 * trigger 5 %, cooldown 10 %), T = initial_temperature, energy = initial_energy (the reference's
 * cluster energy relative to the dilute solution, SimulatedAnnealing.cpp:59-70, is the caller's). */
int lmc_sa_init(lmc_ctx *ctx, int replica, uint64_t seed, uint64_t maximum_steps, double initial_temperature,
                double initial_energy);
/* Runs `steps` trial moves (one warp: pair redrawn until the species differ, PairSite dE, Metropolis,
 * UpdateTemperature); trace (NULL or `steps` records). */
int lmc_sa_run(lmc_ctx *ctx, uint64_t steps, lmc_sa_step *trace);
/* Steps done, current temperature and energy, lowest energy seen by Dump's bookkeeping. */
int lmc_sa_get_state(lmc_ctx *ctx, uint64_t *steps, double *temperature, double *energy, double *lowest_energy);

/* ------------------------------------------------------------------------- */
/* Canonical MC (CanonicalMcOmp semantics, CanonicalMcOmp.cpp:40-92)          */
/* ------------------------------------------------------------------------- */
#define LMC_CMC_REFERENCE_BATCH 0 /* mt19937_64 stream, batch of `batch` pairs as the reference draws them */
#define LMC_CMC_THROUGHPUT 1      /* Philox, many pairs per round, kept when more than 3NN apart */

typedef struct lmc_cmc_options {
  int mode;          /* LMC_CMC_* */
  uint64_t seed;
  int batch;         /* reference-batch mode: pairs per batch (the OpenMP thread count) */
  int candidates;    /* throughput mode: candidate pairs per round, 0 = automatic */
  double *energy_trace; /* reference-batch mode, optional host array of attempts + batch doubles: the
                           energy before every Metropolis test (what CanonicalMcOmp::Simulate hands to
                           ThermodynamicAveraging::AddEnergy and Dump, CanonicalMcOmp.cpp:82-90) */
} lmc_cmc_options;

/* CanonicalMcOmp::Simulate (CanonicalMcOmp.cpp:40-92, CanonicalMcAbstract.cpp:43-101): runs CMC
 * on one replica until at least `attempts` Metropolis tests were made.
 * energy_io: in = current energy, out = energy after the run.
 * attempts_done / accepted: totals of this call. */
int lmc_cmc_run(lmc_ctx *ctx, int replica, double temperature, uint64_t attempts, const lmc_cmc_options *opt,
                double *energy_io, uint64_t *attempts_done, uint64_t *accepted);

/* Rounds of the last throughput-mode lmc_cmc_run (each round: draw, claim, grid barrier, dE and
 * Metropolis tests of the survivors, grid barrier); 0 after a reference-batch run. Diagnostic, no
 * reference counterpart. */
int lmc_cmc_rounds(const lmc_ctx *ctx, uint64_t *rounds);

/* Host-writable stop flag polled by persistent kernels; also clears it when value = 0. */
int lmc_request_stop(lmc_ctx *ctx, int value);

#ifdef __cplusplus
}
#endif
#endif /* LMC_GB300_H_ */
