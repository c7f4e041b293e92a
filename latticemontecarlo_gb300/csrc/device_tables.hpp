// Layout of the read-only tables the kernels consume, shared by the host
// packer (context.cpp) and the kernels (kernels.cu). Plain C++ so both g++ and
// nvcc compile it.
#pragma once
#include <cstdint>

namespace lmc {

constexpr int kLocalSites = 135;  // union of the 12 jump-pair neighbourhoods of a vacancy
constexpr int kMaxOnehot = 8;
constexpr int kMaxSlots = 6;

// Packed cluster descriptors (bit fields):
//  jump-dE cluster (state clusters containing exactly one pair site):
//    [0,3) label  [3] side (0 = first/vacancy site, 1 = second/migrant site)
//    [4,10) other site 1 (state index)  [10,16) other site 2 (63 = none)
//  MMM/MM2 cluster: [0,6) a  [6,12) b (63 = singlet)  [12,14) mode  [14,28) feature base
//  site cluster (43-site list): [0,3) label  [3,9) other 1 (63 = none)  [9,15) other 2 (63 = none)
//  census triplet: [0,3) label  [3,9) k2  [9,15) k3 (site-list indices)
//  full state cluster (integer export): [0,3) label [3,5) size [5,11) i1 [11,17) i2 [17,23) i3
struct DevTables {
  // geometry
  const int8_t *dir;         // [12][4] 1NN offsets (half units)
  const int8_t *dir_of;      // [27] (dx+1)*9+(dy+1)*3+(dz+1) -> direction index or -1
  const int8_t *state_off;   // [12][60][4]
  const int8_t *mmm_off;     // [12][58][4]
  const int8_t *mm2_off;     // [12][58][4]
  const int8_t *site_off;    // [43][4]
  const int8_t *local_off;   // [135][4] KMC neighbourhood of a vacancy
  const uint8_t *shell_local;  // [42] local indices of the vacancy's 1NN, 2NN, 3NN shells
  const int8_t *id_order;    // [27][12] direction of id rank q, per boundary case (context.cpp)
  const uint8_t *local_st;   // [12][60] state list of jump c as indices into the local list
  const uint8_t *local_mmm;  // [12][58]
  const uint8_t *local_mm2f; // [12][58]
  const uint8_t *local_mm2b; // [12][58] backward (second -> first) MM2 list of jump c
  const uint32_t *de_cl;
  // state clusters holding both pair sites, and the two singlets:
  // [0,3) label [3,5) kind (0 first singlet, 1 second singlet, 2 both) [5,11) other site (63 = none)
  const uint32_t *de_both;
  int n_de_both;
  const uint32_t *mmm_cl;
  const uint32_t *mm2_cl;
  const uint32_t *site_cl;
  const uint32_t *census_tri;
  const uint32_t *state_all;
  int n_de_cl, n_mmm_cl, n_mm2_cl, n_site_cl, n_census_tri, n_state_all;
  int pos_first, pos_second, site_center;
  // model
  int num_species, num_onehot, x_code, num_theta, f_mmm, f_mm2, num_slots;
  // Small tables (device memory; kernels stage them in shared memory):
  const int8_t *onehot_rank;     // [8] per species code; kMaxOnehot - 1 marks "no one-hot slot"
  const int8_t *migrant_slot;    // [8] per species code, -1 if no coefficients
  const int8_t *pairtype;        // [3][8][8] (mode, ra, rb) -> index within the orbit block, -1 if invalid
  const uint8_t *has_quartic;    // [kMaxSlots]
  const uint8_t *has_e0;         // [kMaxSlots]
  const int16_t *cluster_index;  // [8][E][E][E]
  const long long *w_de;         // [8][E][E][E]
  double de_scale;               // 2^-shift
  const long long *w_d;          // [slot][f_mmm]
  const long long *w_ks;         // [slot][f_mm2]
  const long long *w_e0;         // [slot][f_mmm]
  const double *form;            // [kMaxSlots][12]: {d: scale, c, sigma, mu}, {ks: ...}, {e0: ...}
  // FP32 epilogue (production KMC streams): per slot the integer centres of the three sums and
  //   [0] 2 sigma_D scale_D, [1] sigma_Ks scale_Ks, [2] P0 = Ks D^2 at the centres,
  //   [3] sigma_e0 scale_e0, [4] e0 at the centre, [7] the energy-change scale
  // so that P = P0 exp([0] (S_D - C_D) + [1] (S_Ks - C_Ks)) and e0 = [4] exp([3] (S_e0 - C_e0)).
  const long long *form32_c;     // [kMaxSlots][3]
  const float *form32;           // [kMaxSlots][8]
  const double *exp_tab;         // [256] 2^(j/256) for ExpFast
  double exp_l1, exp_l2;         // ln2/256 split for ExpFast
  const double *theta;           // [num_theta]
  const double *census_bonds;    // [num_theta]
};

}  // namespace lmc
