/*
 * lmc_oracle.h - TEST ORACLE: a plain-C restatement of the reference's
 * lattice-MC hot path (zhucongx/LatticeMonteCarlo, lmc/cfg, lmc/pred, lmc/mc).
 *
 * Test infrastructure only. It is used by tests/, __graft_entry__.smoke() and
 * the CPU-baseline leg of bench.py as the checker; it is never part of the
 * product path. Every function cites the reference code it restates. The
 * restatement is pinned against vectors produced by the reference's own
 * sources (oracle/build_ref.sh, tests/golden/).
 *
 * Species are int8 codes = rank of the element name in the string-sorted
 * alphabet (barrier element set + "X").
 */
#ifndef LMC_ORACLE_H_
#define LMC_ORACLE_H_
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_lattice orc_lattice;
typedef struct orc_model orc_model;

/* GenerateFCC({n,n,n}) + ReassignLatticeVector (Config.cpp:466-552,1060-1095)
 * with neighbour lists from the cell-list search (Config.cpp:955-1045). */
orc_lattice *orc_lattice_create(int n);
void orc_lattice_destroy(orc_lattice *lat);
int64_t orc_lattice_num_sites(const orc_lattice *lat);
/* 12 + 6 + 24 sorted neighbour ids and the fractional position of a site. */
void orc_lattice_neighbors(const orc_lattice *lat, int64_t id, int64_t *out42);
void orc_lattice_position(const orc_lattice *lat, int64_t id, double *xyz);
/* Sorted id lists of a pair / site (EnergyUtility.cpp:45-104,261-313).
 * Returns 0, or -1 if the lists do not have the expected sizes. */
int orc_pair_lists(const orc_lattice *lat, int64_t first, int64_t second, int64_t *state60, int64_t *mmm58,
                   int64_t *mm258);
int orc_site_list(const orc_lattice *lat, int64_t site, int64_t *out43);
/* Distance label 1/2/3 or -1 (Config.cpp:354-371). */
int orc_distance_label(const orc_lattice *lat, int64_t a, int64_t b);

/* Cluster mappings built from the reference pair (0, NN1[0][0]) / site 0
 * (EnergyUtility.cpp:169-259,393-581). Flattened as records of
 * (group, size, symmetric, i0, i1, i2); group = label for the state/site
 * mappings, orbit index for MMM/MM2. Returns the record count; out may be NULL. */
int orc_mapping(const orc_lattice *lat, int which /*0 state,1 site,2 mmm,3 mm2*/, int32_t *out6, int cap);

/* Model: element names (barrier set), theta, per-migrant Quartic / E0 blocks. */
orc_model *orc_model_create(const char *const *names, int num_names);
void orc_model_destroy(orc_model *m);
int orc_model_num_species(const orc_model *m);
int orc_model_num_theta(const orc_model *m);
/* Species code of a name, -1 if absent. */
int orc_model_code(const orc_model *m, const char *name);
/* Dense index of ElementCluster(label, codes...) or -1 (InitializeClusterHashMap +
 * std::map order, EnergyUtility.cpp:314-343, ElementCluster.hpp:40-50). */
int orc_model_cluster_index(const orc_model *m, int label, int size, const int *codes);
/* MMM / MM2 feature counts for the mappings of `lat`. */
int orc_model_features(const orc_model *m, const orc_lattice *lat, int which /*2 mmm, 3 mm2*/);
void orc_model_set_theta(orc_model *m, const double *theta, int n);
/* Coefficient blocks (copied): U matrices are k x F row-major. */
void orc_model_set_quartic(orc_model *m, int code, int k_mmm, int f_mmm, int k_mm2, int f_mm2,
                           const double *mu_x_mmm, const double *sigma_x_mmm, const double *mu_x_mm2,
                           const double *sigma_x_mm2, const double *u_mmm, const double *u_mm2, const double *theta_d,
                           const double *theta_ks, double mu_d, double sigma_d, double mu_ks, double sigma_ks);
void orc_model_set_e0(orc_model *m, int code, int k_mmm, int f_mmm, const double *mu_x_mmm,
                      const double *sigma_x_mmm, const double *u_mmm, const double *theta_e0, double mu_e0,
                      double sigma_e0);

/* Predictors on a species array. Return 0 or a negative error code
 * (-1 missing neighbour / not 1NN, -2 cluster not indexable, -3 X in an
 * environment, -4 no coefficients for the migrating element). */
/* Quartic: out = {Ea, dE, D, Ks} (VacancyMigrationPredictorQuartic.cpp:112-276). */
int orc_quartic(const orc_model *m, const orc_lattice *lat, const int8_t *sp, int64_t first, int64_t second,
                double *out4);
/* Integer encodings (same layout as lmc_host_encode_pair); NULL pointers skipped. */
int orc_encode(const orc_model *m, const orc_lattice *lat, const int8_t *sp, int64_t first, int64_t second,
               int32_t *state_start, int32_t *state_end, int32_t *mmm, int32_t *mm2f, int32_t *mm2b);
/* E0: out = {Ea, dE, e0} (VacancyMigrationPredictorE0.cpp:77-159). */
int orc_e0(const orc_model *m, const orc_lattice *lat, const int8_t *sp, int64_t first, int64_t second,
           double *out3);
/* PairSite swap dE (EnergyChangePredictorPairSite.cpp:69-192). */
int orc_pair_site_de(const orc_model *m, const orc_lattice *lat, const int8_t *sp, int64_t a, int64_t b,
                     double *de);
/* Single-site substitution dE (EnergyChangePredictorPairSite.cpp:154-192): species at `site` -> new_code. */
int orc_site_de(const orc_model *m, const orc_lattice *lat, const int8_t *sp, int64_t site, int new_code, double *de);
/* EnergyPredictor census counts (num_theta) and energy (EnergyPredictor.cpp:40-96,173-177). */
int orc_energy(const orc_model *m, const orc_lattice *lat, const int8_t *sp, int64_t *counts, double *energy);

/* std::mt19937_64 and the libstdc++ distributions the reference draws from. */
typedef struct orc_mt {
  uint64_t mt[312];
  int idx;
} orc_mt;
void orc_mt_seed(orc_mt *g, uint64_t seed);
uint64_t orc_mt_next(orc_mt *g);
double orc_mt_uniform(orc_mt *g);                  /* uniform_real_distribution<double>(0,1) */
uint64_t orc_mt_below(orc_mt *g, uint64_t range);  /* uniform_int_distribution<size_t>(0,range-1) */

/* KineticMcFirstOmp trajectory (KineticMcAbstract.cpp:140-182, KineticMcFirstOmp.cpp:52-82,
 * JumpEvent.cpp:6-13) on species `sp` (modified in place), temperature T,
 * generator seeded with `seed`. Per step writes trace rows of 8 doubles
 * {vacancy, target, selected, Ea, dE, total_rate, time, energy}; events (NULL or
 * 36 doubles per step) receives the id-sorted {target, Ea, dE} of every event.
 * kind 0 Quartic, 1 E0. memo != 0 memoises barriers by the exact species
 * signature of the jump (the role of VacancyMigrationPredictorQuarticLru). */
int orc_kmc(const orc_model *m, const orc_lattice *lat, int8_t *sp, double T, uint64_t seed, int64_t steps, int kind,
            int memo, double *trace8, double *events36);
/* orc_kmc with a time-temperature schedule (tt_len > 0: T(t) interpolated as
 * TimeTemperatureInterpolator does, at the start of every step), the
 * RateCorrector time factor (rate_corrector != 0) and the IsEscaped early stop
 * (early_stop != 0); steps_done (nullable) receives the steps executed. */
int orc_kmc_ex(const orc_model *m, const orc_lattice *lat, int8_t *sp, double T, uint64_t seed, int64_t steps,
               int kind, int memo, double *trace8, double *events36, const double *tt_time, const double *tt_temp,
               int tt_len, int rate_corrector, int early_stop, int64_t *steps_done);

/* KineticMcFirstOmp with the 12 barriers of a step on `threads` OpenMP threads
 * (KineticMcFirstOmp.cpp:52-82), the id lists of every (site, jump) built first; the
 * trajectory is orc_kmc's without memo, rate corrector, schedule or early stop. *loop_s
 * receives the wall time of the step loop. Returns 0, or -1. */
int orc_kmc_threads(const orc_model *m, const orc_lattice *lat, int8_t *sp, double T, uint64_t seed, int64_t steps,
                    int kind, int threads, double *trace8, double *loop_s);
/* CanonicalMcOmp with batch size `batch` (CanonicalMcOmp.cpp:40-92,
 * CanonicalMcAbstract.cpp:43-101): runs until `attempts` Metropolis tests were
 * made (whole batches). energy_trace (NULL or capacity `cap`) receives energy_
 * before every test, as cmc_log.txt does. Returns the number of tests. */
int64_t orc_cmc(const orc_model *m, const orc_lattice *lat, int8_t *sp, double T, uint64_t seed, int64_t attempts,
                int batch, double *energy_io, double *energy_trace, int64_t cap, int64_t *accepted);

/* Multi-vacancy extension switch: with on != 0 a cluster whose element multiset
 * has no index (two or more vacancies) counts nothing and a vacancy inside a
 * one-hot environment contributes a zero vector, instead of the reference's
 * exceptions (ClusterIndexer::GetIndex, one_hot_encode_hashmap.at()). */
void orc_model_set_vacancy_zero(orc_model *m, int on);

/* Philox4x32-10 block (Salmon et al., SC'11): out = bijection(ctr) under key. */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

/* Multi-vacancy KMC as the GPU defines it (lmc_kmc_multi_run): the nv slots
 * vac[] (site ids, updated in place) of lattice `replica`, steps step0 ..
 * step0 + steps - 1 of its Philox stream. Every step re-evaluates all slots
 * (a vacancy inside another's neighbourhood contributes nothing to the
 * encodings), scans the rates as the kernel does, selects and moves one vacancy.
 * trace9 (NULL or 9 doubles per step): slot, vacancy, target, selected, Ea, dE,
 * total rate, time, energy. time_io / energy_io carry the clock and energy. */
int orc_kmc_multi(orc_model *m, const orc_lattice *lat, int8_t *sp, double T, uint64_t seed, uint32_t replica,
                  uint64_t step0, int64_t steps, int kind, int64_t *vac, int nv, double *time_io, double *energy_io,
                  double *trace9);

/* KineticMcChainOmpi (second-order residence time, KineticMcChainOmpi.cpp:56-152) on one
 * lattice: per step the 12 x 12 barriers i -> l after each jump k -> i, the reverse events'
 * rates and the second-order probabilities and time, sums in rank (id) order, one uniform
 * draw per step for the selection (rng 0: mt19937_64 seeded with `seed`; rng 1: the Philox
 * production stream of lattice `replica`). trace8 as orc_kmc, Ea = the chain event's barrier. */
int orc_kmc_chain(const orc_model *m, const orc_lattice *lat, int8_t *sp, double T, uint64_t seed, int64_t steps,
                  int kind, int rng, uint32_t replica, double *trace8);

/* SimulatedAnnealing's loop (SimulatedAnnealing.cpp:78-185) on lattice `sp` (modified in place):
 * mt19937_64 seeded with `seed`, `steps` trial moves of a run planned for maximum_steps, energy
 * starting at energy0. trace7 (NULL or 7 doubles per step): site1, site2, accepted, dE, energy and
 * temperature before the step, lowest energy after Dump's bookkeeping. state4 (NULL or 4
 * doubles): steps, temperature, energy, lowest energy at the end. */
int orc_sa(const orc_model *m, const orc_lattice *lat, int8_t *sp, double T0, uint64_t seed, uint64_t maximum_steps,
           int64_t steps, double energy0, double *trace7, double *state4);

/* EnergyPredictor::GetEnergyOfCluster (EnergyPredictor.cpp:97-184) over the listed sites and their
 * 1-3NN shells; mode 0: species sp, 1: solvent except at the listed sites, 2: solvent everywhere. */
int orc_cluster_energy(const orc_model *m, const orc_lattice *lat, const int8_t *sp, int solvent, int mode,
                       const int64_t *sites, int64_t count, double *energy);
/* SoluteCluster::FindAtomListOfClusters (SoluteCluster.cpp:277-373): CSR cluster lists (members sorted,
 * clusters by size, larger first, ties by first id). Returns the cluster count, -1 if `cap` is short. */
int64_t orc_solute_clusters(const orc_lattice *lat, const int8_t *sp, int solvent, int64_t smallest, int64_t bond,
                            int64_t *offsets, int64_t *members, int64_t cap);

#ifdef __cplusplus
}
#endif
#endif
