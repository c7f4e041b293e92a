// Host-side model: species alphabet, ElementCluster indexing and the folding
// of the reference's coefficient blocks into per-feature fixed-point weights.
//
// Folding. The reference evaluates, per migrating element M,
//   logD  = sigma_D  * theta_D  . (U_mmm ((x_mmm - mu) / sigma)) + mu_D
//   logKs = sigma_Ks * theta_Ks . (U_mm2 ((x_fwd + x_bwd - mu) / sigma)) + mu_Ks
// (lmc/pred/src/VacancyMigrationPredictorQuartic.cpp:167-246). With
// b = (U^T theta) / sigma this is sigma * (b . x - b . mu) + mu, and since each
// feature x_f is an orbit average of one-hot codes, b . x is a sum over the
// orbit's clusters of b_f / |orbit|. The weights b_f / |orbit| are stored as
// int64 fixed point with a per-table power-of-two scale chosen so the largest
// possible sum stays below 2^61; sums are then exact and order independent.
// The energy-change tables hold theta_idx / cluster_counter[label] per
// (label, species...) tuple in the same fixed point
// (VacancyMigrationPredictorQuartic.cpp:156-165, EnergyChangePredictorPairSite.cpp:83-94).
#pragma once
#include <cstdint>
#include <map>
#include <string>
#include <vector>

#include "geometry.hpp"

namespace lmc {

constexpr int kMaxSpecies = 6;   // X, Al, Mg, Zn, Cu, Sn
constexpr int kMaxLabel = 8;     // cluster labels 0..7

// Cluster counters of the energy-change predictors (labels 0..10) and of the
// full-lattice EnergyPredictor (lmc/pred/src/EnergyPredictor.cpp:8).
extern const double kDeClusterCounter[11];
extern const double kCensusClusterCounter[11];

struct QuarticBlock {
  int k_mmm{0}, k_mm2{0};
  std::vector<double> mu_x_mmm, sigma_x_mmm, mu_x_mm2, sigma_x_mm2, u_mmm, u_mm2, theta_d, theta_ks;
  double mu_d{0}, sigma_d{0}, mu_ks{0}, sigma_ks{0};
};
struct E0Block {
  int k_mmm{0};
  std::vector<double> mu_x_mmm, sigma_x_mmm, u_mmm, theta_e0;
  double mu_e0{0}, sigma_e0{0};
};

// Folded fixed-point weights of one linear form sigma * (b . x - c) + mu.
struct FoldedForm {
  std::vector<int64_t> w;   // per feature
  int shift{0};             // w = round(value * 2^shift)
  double c{0}, sigma{0}, mu{0};
};

struct Model {
  std::vector<std::string> onehot;     // barrier element set, string order
  std::vector<std::string> alphabet;   // onehot + "X", string order; species code = index
  int x_code{-1};
  std::vector<int> onehot_rank;        // per species code: rank in `onehot`, -1 if none
  int num_theta{0};
  std::vector<int> cluster_index;      // [label][c1][c2][c3] -> theta index or -1 (codes in any order)
  std::vector<int> theta_label;        // label of each theta index
  std::vector<double> base_theta;
  std::map<int, QuarticBlock> quartic; // by species code of the migrating element
  std::map<int, E0Block> e0;

  int NumSpecies() const { return static_cast<int>(alphabet.size()); }
  int NumOnehot() const { return static_cast<int>(onehot.size()); }
  int Code(const std::string &name) const;
  int FeaturesMmm() const;
  int FeaturesMm2() const;
  int ClusterIdx(int label, int c1, int c2, int c3) const;
};

// Builds the alphabet for an element set (names as in the reference's
// Element(std::string) constructor; unknown names map to "X" as it does).
Model MakeModel(const std::vector<std::string> &element_names);
// Reads "Base".theta and every per-element block of a coefficient JSON.
void LoadJson(Model &m, const std::string &path);

// Dense index of an ordered/symmetric pair type or singlet within an orbit block
// (GetOneHotEncodeHashmap, lmc/pred/src/EnergyUtility.cpp:7-43): mode 0 singlet
// (ra), 1 ordered pair (ra * e + rb), 2 symmetric pair (upper triangle).
int PairType(int mode, int ra, int rb, int e);

// Folded tables of a model, ready for upload.
struct FoldedModel {
  int num_species{0}, num_onehot{0}, x_code{-1}, num_theta{0};
  int f_mmm{0}, f_mm2{0};
  std::vector<int8_t> onehot_rank;         // per code
  std::vector<int16_t> cluster_index;      // [8][E][E][E]
  std::vector<int64_t> w_de;               // [8][E][E][E] theta/kDeClusterCounter, fixed point
  int de_shift{0};
  std::vector<double> census_weight;       // per theta index: theta / kCensusClusterCounter
  std::vector<double> theta;               // base theta
  std::vector<double> census_bonds;        // per theta index
  std::vector<double> de_bonds;            // per theta index
  // Per migrating species code: slot or -1; forms per slot.
  std::vector<int8_t> migrant_slot;        // per code
  std::vector<int> slot_code;
  std::vector<FoldedForm> quartic_d, quartic_ks, e0;  // per slot (empty w if absent)
  std::vector<uint8_t> has_quartic, has_e0;          // per slot
};
FoldedModel Fold(const Model &m);

// Integer encodings of a jump pair on a host lattice (see lmc_host_encode_pair).
void HostEncodePair(const Model &m, int n, const int8_t *species, int64_t first, int64_t second,
                    int32_t *state_start, int32_t *state_end, int32_t *mmm, int32_t *mm2_fwd, int32_t *mm2_bwd);

}  // namespace lmc
