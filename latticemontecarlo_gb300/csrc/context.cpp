// C ABI of the GB300 lattice-MC hot path (include/lmc_gb300.h): models,
// host-only geometry queries, device contexts, table packing and launches.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cstdio>
#include <sstream>
#include <fstream>
#include <cmath>
#include <cstring>
#include <ios>
#include <tuple>
#include <limits>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/lmc_gb300.h"
#include "geometry.hpp"
#include "json.hpp"
#include "kernels.cuh"
#include "model.hpp"
#include "abi_common.hpp"
#include "mlp.cuh"

namespace {
using lmc::abi::CudaCheck;
using lmc::abi::g_error;
using lmc::abi::Guard;
using lmc::abi::LmcError;
using lmc::abi::Require;

int8_t Pack4(int v) { return static_cast<int8_t>(v); }

uint32_t PackEnv(const lmc::EnvCluster &c, int base) {
  const uint32_t b = c.b < 0 ? 63u : static_cast<uint32_t>(c.b);
  return static_cast<uint32_t>(c.a) | (b << 6) | (static_cast<uint32_t>(c.mode) << 12) | (static_cast<uint32_t>(base) << 14);
}

// Device buffer owned by a context.
struct DevBuf {
  void *p{nullptr};
  size_t bytes{0};
  void Alloc(size_t b) {
    Free();
    if (b == 0) b = 16;
    CudaCheck(cudaMalloc(&p, b), "cudaMalloc");
    bytes = b;
  }
  void Ensure(size_t b) {
    if (b > bytes) Alloc(b);
  }
  void Free() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  template <typename T>
  T *as() const {
    return static_cast<T *>(p);
  }
};

}  // namespace

struct lmc_model {
  lmc::Model m;
};

struct lmc_ctx {
  int device{0};
  cudaStream_t stream{nullptr};
  cudaEvent_t ev0{nullptr}, ev1{nullptr};
  lmc::Model model;
  lmc::FoldedModel fm;
  lmc::DevTables t{};
  std::vector<DevBuf> tables;
  // lattices
  int num_replicas{0};
  std::vector<int> n;
  std::vector<long long> offsets;
  long long total_sites{0};
  DevBuf species, lat_off, lat_n, scan;
  std::vector<unsigned long long> scan_host;  // per replica species histogram + invalid count
  std::vector<long long> first_host;          // per replica lowest X site (LLONG_MAX: none)
  bool scan_fresh{false};                     // scan_host / first_host describe the current lattices
  int barrier_eval{LMC_EVAL_SPARSE};          // evaluation of the barrier batch entry points
  int feat_encoding{LMC_FEATURES_ONEHOT};     // surrogate feature rows (lmc_surrogate_set_encoding)
  DevBuf scan_first;
  // batch scratch
  DevBuf pairs, out0, out1, out2, out3, status, counts, energy, enc;
  // KMC
  bool kmc_ready{false};
  lmc_kmc_options kmc_opt{};
  DevBuf k_vac, k_steps, k_time, k_energy, k_temp, k_cvac, k_csol, k_rng, k_trace, k_events, k_tt_time, k_tt_temp;
  DevBuf k_solvent, k_escaped, k_prev, c_trace;
  DevBuf s_feat, s_mean, s_spread, s_fb_pairs, s_fb_index, s_fb_ea, s_fb_de;
  int tt_len{0};
  // sparse KMC tables (built for the dominant species at lmc_kmc_init)
  std::vector<DevBuf> sparse_bufs;
  int sparse_base{-1};  // base species the sparse tables were built for (-1: none)
  lmc::KmcSparse sparse{};
  // CMC
  DevBuf c_claim, c_cand, c_eacc, c_stats;
  unsigned long long cmc_rounds{0};  // rounds of the last throughput-mode run
  std::map<int, std::pair<uint64_t, DevBuf>> c_mt;  // per replica: seed and MT state
  // host-mapped stop flag
  int *h_stop{nullptr};
  int *d_stop{nullptr};
  double last_ms{0};
  // graph-captured KMC launches (lmc_kmc_run_graph): the executable graph and the
  // kernel argument bytes it was recorded with; pinned word the graph copies the status into
  cudaGraphExec_t kmc_graph{nullptr};
  std::vector<unsigned char> kmc_graph_key;
  int *h_status{nullptr};
  // solute clusters of the last lmc_solute_clusters call (CSR lists, formation energies)
  std::vector<int64_t> cl_offsets, cl_members;
  std::vector<double> cl_energy;
  // simulated annealing on one lattice
  bool sa_ready{false};
  int sa_replica{0};
  DevBuf sa_state, sa_rng, sa_trace;
  // multi-vacancy KMC (every vacancy of a lattice tracked; slots per lattice)
  bool multi_ready{false};
  int multi_kind{0}, multi_eval{0};
  int multi_rates{LMC_RATES_FP64};  // lmc_kmc_multi_set_rates
  std::vector<int> m_off_host;
  DevBuf m_pos, m_off, m_steps, m_time, m_energy, m_temp, m_key, m_trace;
  std::array<uint32_t, lmc::kLocalBitWords> local_bits{};
  // surrogate-assisted multi-vacancy KMC (lmc_kmc_multi_surrogate_run)
  DevBuf su_pairs, su_dirty, su_mean, su_spread, su_cum, su_ea, su_tgt, su_kmask, su_pair_ea, su_fb, su_halt,
      su_trace, su_plain;

  ~lmc_ctx() {
    for (auto &b : tables) b.Free();
    for (DevBuf *b : {&species, &lat_off, &lat_n, &scan, &scan_first, &pairs, &out0, &out1, &out2, &out3, &status, &counts, &energy, &enc,
                      &k_vac, &k_steps, &k_time, &k_energy, &k_temp, &k_cvac, &k_csol, &k_rng, &k_trace, &k_events,
                      &k_tt_time, &k_tt_temp, &k_solvent, &k_escaped, &k_prev, &c_trace, &s_feat, &s_mean, &s_spread,
                      &s_fb_pairs, &s_fb_index, &s_fb_ea, &s_fb_de, &c_claim, &c_cand, &c_eacc, &c_stats})
      b->Free();
    for (DevBuf *b : {&m_pos, &m_off, &m_steps, &m_time, &m_energy, &m_temp, &m_key, &m_trace, &sa_state, &sa_rng,
                      &sa_trace, &su_pairs, &su_dirty, &su_mean, &su_spread, &su_cum, &su_ea, &su_tgt,
                      &su_kmask, &su_pair_ea, &su_fb, &su_halt, &su_trace, &su_plain})
      b->Free();
    for (auto &kv : c_mt) kv.second.second.Free();
    for (auto &b : sparse_bufs) b.Free();
    if (h_stop) cudaFreeHost(h_stop);
    if (kmc_graph) cudaGraphExecDestroy(kmc_graph);
    if (h_status) cudaFreeHost(h_status);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (stream) cudaStreamDestroy(stream);
  }

  template <typename T>
  const T *Upload(const std::vector<T> &v, std::vector<DevBuf> *into = nullptr) {
    DevBuf b;
    b.Alloc(std::max<size_t>(v.size() * sizeof(T), 16));
    if (!v.empty()) CudaCheck(cudaMemcpy(b.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice), "upload");
    (into ? into : &tables)->push_back(b);
    return b.as<T>();
  }
  void Sync() { CudaCheck(cudaStreamSynchronize(stream), "cudaStreamSynchronize"); }
  int ReadStatus() {
    int st = 0;
    CudaCheck(cudaMemcpyAsync(&st, status.p, sizeof(int), cudaMemcpyDeviceToHost, stream), "status copy");
    Sync();
    return st;
  }
  void ClearStatus() { CudaCheck(cudaMemsetAsync(status.p, 0, sizeof(int), stream), "status clear"); }
  // Four pinned host words for status / count copies that stay asynchronous.
  int *Pinned() {
    if (!h_status) CudaCheck(cudaMallocHost(&h_status, 4 * sizeof(int)), "cudaMallocHost");
    return h_status;
  }
  void CheckReplica(int r) const {
    Require(r >= 0 && r < num_replicas, LMC_ERR_OUT_OF_RANGE, "replica index out of range");
  }
};

namespace {

void RaiseStatus(int st, const char *what) {
  if (st == 0) return;
  std::string m = std::string(what) + ": ";
  if (st & lmc::kStatusBadSite) throw LmcError(LMC_ERR_OUT_OF_RANGE, m + "lattice id out of range");
  if (st & lmc::kStatusNotNeighbor)
    throw LmcError(LMC_ERR_OUT_OF_RANGE, m + "Neighbor not found for lattice pair in GetPairFlatIndex");
  if (st & lmc::kStatusNoCoefficients)
    throw LmcError(LMC_ERR_OUT_OF_RANGE, m + "migrating element has no coefficients");
  if (st & lmc::kStatusBadCluster) throw LmcError(LMC_ERR_OUT_OF_RANGE, m + "Cluster not found in ClusterIndexer");
  if (st & lmc::kStatusXInEnv)
    throw LmcError(LMC_ERR_OUT_OF_RANGE, m + "vacancy inside a jump environment has no one-hot slot");
  if (st & lmc::kStatusNumeric) throw LmcError(LMC_ERR_NUMERIC, m + "non-finite barrier or non-positive total rate");
  if (st & lmc::kStatusStopped) throw LmcError(LMC_ERR_STOPPED, m + "stopped");
}

// Builds and uploads every read-only table of a context.
void BuildTables(lmc_ctx *c) {
  const auto &pt = lmc::GetPairTables();
  const auto &fm = c->fm;
  lmc::DevTables &t = c->t;
  std::vector<int8_t> dir, st_off, mmm_off, mm2_off, site_off;
  for (int d = 0; d < lmc::kDirections; ++d) {
    for (int v : {pt.dir[d].x, pt.dir[d].y, pt.dir[d].z, 0}) dir.push_back(Pack4(v));
    for (int k = 0; k < lmc::kStateSites; ++k)
      for (int v : {pt.state_off[d][k].x, pt.state_off[d][k].y, pt.state_off[d][k].z, 0}) st_off.push_back(Pack4(v));
    for (int k = 0; k < lmc::kEnvSites; ++k) {
      for (int v : {pt.mmm_off[d][k].x, pt.mmm_off[d][k].y, pt.mmm_off[d][k].z, 0}) mmm_off.push_back(Pack4(v));
      for (int v : {pt.mm2_off[d][k].x, pt.mm2_off[d][k].y, pt.mm2_off[d][k].z, 0}) mm2_off.push_back(Pack4(v));
    }
  }
  for (int k = 0; k < lmc::kSiteSites; ++k)
    for (int v : {pt.site_off[k].x, pt.site_off[k].y, pt.site_off[k].z, 0}) site_off.push_back(Pack4(v));
  // jump dE clusters: state clusters with exactly one pair site
  std::vector<uint32_t> de_cl, de_both, state_all;
  for (const auto &cl : pt.state_clusters) {
    uint32_t w = static_cast<uint32_t>(cl.label) | (static_cast<uint32_t>(cl.size) << 3);
    for (int q = 0; q < 3; ++q) w |= static_cast<uint32_t>(q < cl.size ? cl.idx[q] : 0) << (5 + 6 * q);
    state_all.push_back(w);
    int has_first = 0, has_second = 0;
    std::vector<int> others;
    for (int q = 0; q < cl.size; ++q) {
      if (cl.idx[q] == pt.pos_first) has_first = 1;
      else if (cl.idx[q] == pt.pos_second) has_second = 1;
      else others.push_back(cl.idx[q]);
    }
    if (has_first + has_second == 2 || others.empty()) {
      const uint32_t kind = has_first + has_second == 2 ? 2u : (has_first ? 0u : 1u);
      const uint32_t o = others.empty() ? 63u : static_cast<uint32_t>(others[0]);
      Require(others.size() <= 1, LMC_ERR_UNSUPPORTED, "unexpected cluster shape");
      de_both.push_back(static_cast<uint32_t>(cl.label) | (kind << 3) | (o << 5));
      continue;
    }
    uint32_t d = static_cast<uint32_t>(cl.label) | (static_cast<uint32_t>(has_second) << 3) |
                 (static_cast<uint32_t>(others[0]) << 4) | (static_cast<uint32_t>(others.size() > 1 ? others[1] : 63) << 10);
    de_cl.push_back(d);
  }
  auto env = [&](const lmc::EnvEncoding &e) {
    std::vector<uint32_t> out;
    const auto off = e.OrbitOffsets(fm.num_onehot);
    Require(off.back() < (1 << 14), LMC_ERR_UNSUPPORTED, "feature layout too large");
    for (const auto &cl : e.clusters) out.push_back(PackEnv(cl, off[cl.orbit]));
    return out;
  };
  std::vector<uint32_t> mmm_cl = env(pt.mmm), mm2_cl = env(pt.mm2);
  std::vector<uint32_t> site_cl;
  for (const auto &cl : pt.site_clusters) {
    std::vector<int> others;
    for (int q = 0; q < cl.size; ++q)
      if (cl.idx[q] != pt.site_center) others.push_back(cl.idx[q]);
    const uint32_t o1 = others.size() > 0 ? others[0] : 63, o2 = others.size() > 1 ? others[1] : 63;
    site_cl.push_back(static_cast<uint32_t>(cl.label) | (o1 << 3) | (o2 << 9));
  }
  auto site_index = [&](lmc::I3 s) {
    for (int k = 0; k < lmc::kSiteSites; ++k)
      if (pt.site_off[k] == s) return k;
    throw std::logic_error("census offset not in the site list");
  };
  std::vector<uint32_t> census;
  for (const auto &tr : pt.census_triplets)
    census.push_back(static_cast<uint32_t>(tr.label) | (static_cast<uint32_t>(site_index(tr.s2)) << 3) |
                     (static_cast<uint32_t>(site_index(tr.s3)) << 9));
  // KMC neighbourhood of a vacancy: union of the 12 jumps' lists
  std::vector<lmc::I3> local;
  auto add = [&](lmc::I3 s) {
    if (std::find(local.begin(), local.end(), s) == local.end()) local.push_back(s);
  };
  for (int d = 0; d < lmc::kDirections; ++d) {
    const int db = lmc::DirectionIndex(lmc::I3{0, 0, 0} - pt.dir[d]);
    for (int k = 0; k < lmc::kStateSites; ++k) add(pt.state_off[d][k]);
    for (int k = 0; k < lmc::kEnvSites; ++k) {
      add(pt.mmm_off[d][k]);
      add(pt.mm2_off[d][k]);
      add(pt.dir[d] + pt.mm2_off[db][k]);
    }
  }
  std::sort(local.begin(), local.end(), [](lmc::I3 a, lmc::I3 b) {
    return std::tie(a.x, a.y, a.z) < std::tie(b.x, b.y, b.z);
  });
  Require(static_cast<int>(local.size()) == lmc::kLocalSites, LMC_ERR_UNSUPPORTED, "unexpected KMC neighbourhood size");
  auto lidx = [&](lmc::I3 s) {
    return static_cast<uint8_t>(std::find(local.begin(), local.end(), s) - local.begin());
  };
  std::vector<int8_t> local_off;
  for (const auto &s : local)
    for (int v : {s.x, s.y, s.z, 0}) local_off.push_back(Pack4(v));
  // displacement bitmap of the neighbourhood (multi-vacancy KMC: which slots a changed site affects)
  c->local_bits.fill(0);
  for (const auto &s : local) {
    Require(std::abs(s.x) <= 4 && std::abs(s.y) <= 4 && std::abs(s.z) <= 4, LMC_ERR_UNSUPPORTED,
            "KMC neighbourhood wider than 4 half-units");
    const int b = ((s.x + 4) * lmc::kLocalSpan + (s.y + 4)) * lmc::kLocalSpan + (s.z + 4);
    c->local_bits[b >> 5] |= 1u << (b & 31);
  }
  std::vector<uint8_t> l_st, l_mmm, l_mm2f, l_mm2b;
  for (int d = 0; d < lmc::kDirections; ++d) {
    const int db = lmc::DirectionIndex(lmc::I3{0, 0, 0} - pt.dir[d]);
    for (int k = 0; k < lmc::kStateSites; ++k) l_st.push_back(lidx(pt.state_off[d][k]));
    for (int k = 0; k < lmc::kEnvSites; ++k) {
      l_mmm.push_back(lidx(pt.mmm_off[d][k]));
      l_mm2f.push_back(lidx(pt.mm2_off[d][k]));
      l_mm2b.push_back(lidx(pt.dir[d] + pt.mm2_off[db][k]));
    }
  }
  // small model tables
  Require(fm.num_onehot <= lmc::kMaxOnehot - 1, LMC_ERR_UNSUPPORTED, "too many one-hot elements");
  std::vector<int8_t> rank(8, lmc::kMaxOnehot - 1), slot(8, -1), ptype(192, -1);
  for (int code = 0; code < fm.num_species; ++code) {
    rank[code] = fm.onehot_rank[code] < 0 ? lmc::kMaxOnehot - 1 : fm.onehot_rank[code];
    slot[code] = fm.migrant_slot[code];
  }
  for (int mode = 0; mode < 3; ++mode)
    for (int ra = 0; ra < fm.num_onehot; ++ra)
      for (int rb = 0; rb < fm.num_onehot; ++rb)
        ptype[(mode * 8 + ra) * 8 + rb] = static_cast<int8_t>(lmc::PairType(mode, ra, rb, fm.num_onehot));
  const int slots = static_cast<int>(fm.slot_code.size());
  Require(slots <= lmc::kMaxSlots, LMC_ERR_UNSUPPORTED, "too many migrating elements");
  std::vector<uint8_t> hq(lmc::kMaxSlots, 0), he(lmc::kMaxSlots, 0);
  std::vector<double> form(lmc::kMaxSlots * 12, 0.0);
  std::vector<long long> wd, wks, we0;
  for (int sidx = 0; sidx < slots; ++sidx) {
    hq[sidx] = fm.has_quartic[sidx];
    he[sidx] = fm.has_e0[sidx];
    const lmc::FoldedForm *forms[3] = {&fm.quartic_d[sidx], &fm.quartic_ks[sidx], &fm.e0[sidx]};
    for (int q = 0; q < 3; ++q) {
      form[sidx * 12 + q * 4 + 0] = std::ldexp(1.0, -forms[q]->shift);
      form[sidx * 12 + q * 4 + 1] = forms[q]->c;
      form[sidx * 12 + q * 4 + 2] = forms[q]->sigma;
      form[sidx * 12 + q * 4 + 3] = forms[q]->mu;
    }
    wd.insert(wd.end(), fm.quartic_d[sidx].w.begin(), fm.quartic_d[sidx].w.end());
    wks.insert(wks.end(), fm.quartic_ks[sidx].w.begin(), fm.quartic_ks[sidx].w.end());
    we0.insert(we0.end(), fm.e0[sidx].w.begin(), fm.e0[sidx].w.end());
  }
  std::vector<long long> wde(fm.w_de.begin(), fm.w_de.end());
  std::vector<int8_t> dir_of(27, -1);
  for (int d = 0; d < lmc::kDirections; ++d)
    dir_of[(pt.dir[d].x + 1) * 9 + (pt.dir[d].y + 1) * 3 + (pt.dir[d].z + 1)] = static_cast<int8_t>(d);
  t.dir = c->Upload(dir);
  {
    // Id order of a site's 12 first neighbours. Ids are lexicographic in the wrapped half-lattice
    // coordinates, and a +-1 step wraps only at coordinate 0 (-1 becomes the largest) or 2n - 1
    // (+1 becomes the smallest), so the order depends only on which axes sit on a boundary:
    // per axis 0 interior, 1 at 0, 2 at 2n - 1; case = 9 s_x + 3 s_y + s_z; entry q = the
    // direction of rank q.
    std::vector<int8_t> order(27 * lmc::kDirections);
    for (int cs = 0; cs < 27; ++cs) {
      const int st[3] = {cs / 9, (cs / 3) % 3, cs % 3};
      auto key = [&](int d) {
        const int v[3] = {pt.dir[d].x, pt.dir[d].y, pt.dir[d].z};
        std::array<int, 3> k{};
        for (int a = 0; a < 3; ++a) {
          // the step's value relative to the site on an axis of width 8, site at 4 / 0 / 7
          const int h = st[a] == 0 ? 4 : (st[a] == 1 ? 0 : 7);
          k[a] = ((h + v[a]) % 8 + 8) % 8;
        }
        return k;
      };
      std::vector<int> ds(lmc::kDirections);
      for (int d = 0; d < lmc::kDirections; ++d) ds[d] = d;
      std::sort(ds.begin(), ds.end(), [&](int a, int b) { return key(a) < key(b); });
      for (int q = 0; q < lmc::kDirections; ++q) order[cs * lmc::kDirections + q] = static_cast<int8_t>(ds[q]);
    }
    t.id_order = c->Upload(order);
  }
  t.dir_of = c->Upload(dir_of);
  t.state_off = c->Upload(st_off);
  t.mmm_off = c->Upload(mmm_off);
  t.mm2_off = c->Upload(mm2_off);
  t.site_off = c->Upload(site_off);
  t.local_off = c->Upload(local_off);
  {
    std::vector<uint8_t> shell;
    for (int sh = 1; sh <= 3; ++sh)
      for (const auto &o : lmc::ShellOffsets(sh)) shell.push_back(lidx(o));
    Require(shell.size() == 42, LMC_ERR_UNSUPPORTED, "unexpected neighbour shells");
    for (uint8_t v : shell) Require(v < lmc::kLocalSites, LMC_ERR_UNSUPPORTED, "shell site outside the neighbourhood");
    t.shell_local = c->Upload(shell);
  }
  t.local_st = c->Upload(l_st);
  t.local_mmm = c->Upload(l_mmm);
  t.local_mm2f = c->Upload(l_mm2f);
  t.local_mm2b = c->Upload(l_mm2b);
  t.de_cl = c->Upload(de_cl);
  t.de_both = c->Upload(de_both);
  t.n_de_both = static_cast<int>(de_both.size());
  t.mmm_cl = c->Upload(mmm_cl);
  t.mm2_cl = c->Upload(mm2_cl);
  t.site_cl = c->Upload(site_cl);
  t.census_tri = c->Upload(census);
  t.state_all = c->Upload(state_all);
  t.n_de_cl = static_cast<int>(de_cl.size());
  t.n_mmm_cl = static_cast<int>(mmm_cl.size());
  t.n_mm2_cl = static_cast<int>(mm2_cl.size());
  t.n_site_cl = static_cast<int>(site_cl.size());
  t.n_census_tri = static_cast<int>(census.size());
  t.n_state_all = static_cast<int>(state_all.size());
  t.pos_first = pt.pos_first;
  t.pos_second = pt.pos_second;
  t.site_center = pt.site_center;
  t.num_species = fm.num_species;
  t.num_onehot = fm.num_onehot;
  t.x_code = fm.x_code;
  t.num_theta = fm.num_theta;
  t.f_mmm = fm.f_mmm;
  t.f_mm2 = fm.f_mm2;
  t.num_slots = slots;
  t.onehot_rank = c->Upload(rank);
  t.migrant_slot = c->Upload(slot);
  t.pairtype = c->Upload(ptype);
  t.has_quartic = c->Upload(hq);
  t.has_e0 = c->Upload(he);
  t.cluster_index = c->Upload(fm.cluster_index);
  t.w_de = c->Upload(wde);
  t.de_scale = std::ldexp(1.0, -fm.de_shift);
  t.w_d = c->Upload(wd);
  t.w_ks = c->Upload(wks);
  t.w_e0 = c->Upload(we0);
  t.form = c->Upload(form);
  {
    // FP32 epilogue tables: the sums' integer centres C = round(c / scale) (exact integer
    // deviations S - C on the device) and the folded constants, from extended precision
    std::vector<long long> fc(lmc::kMaxSlots * 3, 0);
    std::vector<float> f32(lmc::kMaxSlots * 8, 0.0f);
    Require(fm.de_shift < 126, LMC_ERR_UNSUPPORTED, "energy-change scale outside the FP32 range");
    for (int sidx = 0; sidx < slots; ++sidx) {
      const lmc::FoldedForm *forms[3] = {&fm.quartic_d[sidx], &fm.quartic_ks[sidx], &fm.e0[sidx]};
      long double lc[3];  // mu - sigma * (c - C scale): the form's value at S = C
      for (int q = 0; q < 3; ++q) {
        const long double sc = std::ldexp(1.0L, -forms[q]->shift);
        const long double centre = std::nearbyint(static_cast<long double>(forms[q]->c) / sc);
        Require(std::fabs(centre) < 9.0e18L, LMC_ERR_UNSUPPORTED, "linear-form centre outside int64");
        fc[sidx * 3 + q] = static_cast<long long>(centre);
        lc[q] = forms[q]->mu - forms[q]->sigma * (forms[q]->c - centre * sc);
      }
      f32[sidx * 8 + 0] = static_cast<float>(2.0L * forms[0]->sigma * std::ldexp(1.0L, -forms[0]->shift));
      f32[sidx * 8 + 1] = static_cast<float>(forms[1]->sigma * std::ldexp(1.0L, -forms[1]->shift));
      f32[sidx * 8 + 2] = static_cast<float>(std::exp(2.0L * lc[0] + lc[1]));
      f32[sidx * 8 + 3] = static_cast<float>(forms[2]->sigma * std::ldexp(1.0L, -forms[2]->shift));
      f32[sidx * 8 + 4] = static_cast<float>(std::exp(lc[2]));
      f32[sidx * 8 + 7] = std::ldexp(1.0f, -fm.de_shift);
      for (int q = 0; q < 8; ++q)
        Require(std::isfinite(f32[sidx * 8 + q]), LMC_ERR_UNSUPPORTED, "barrier constants outside the FP32 range");
    }
    t.form32_c = c->Upload(fc);
    t.form32 = c->Upload(f32);
  }
  // ExpFast constants: 2^(j/256) rounded from extended precision; ln2/256
  // split into a 34-bit head (exact products with |n| < 2^18) and a tail
  {
    std::vector<double> tab(256);
    for (int j = 0; j < 256; ++j) tab[j] = static_cast<double>(std::exp2(static_cast<long double>(j) / 256.0L));
    const long double l = std::log(2.0L) / 256.0L;
    int ex = 0;
    const long double mant = std::frexp(l, &ex);
    const long double head = std::ldexp(std::round(std::ldexp(mant, 34)), ex - 34);
    t.exp_tab = c->Upload(tab);
    t.exp_l1 = static_cast<double>(head);
    t.exp_l2 = static_cast<double>(l - head);
  }
  t.theta = c->Upload(fm.theta);
  t.census_bonds = c->Upload(fm.census_bonds);
}

std::vector<std::string> Names(const char *const *names, int n) {
  Require(names != nullptr && n > 0, LMC_ERR_INVALID_ARGUMENT, "empty element set");
  std::vector<std::string> v;
  for (int i = 0; i < n; ++i) {
    Require(names[i] != nullptr, LMC_ERR_INVALID_ARGUMENT, "null element name");
    v.emplace_back(names[i]);
  }
  return v;
}

int CodeOf(const lmc::Model &m, const char *name) {
  Require(name != nullptr, LMC_ERR_INVALID_ARGUMENT, "null element name");
  const int c = m.Code(name);
  Require(c >= 0, LMC_ERR_OUT_OF_RANGE, std::string("element ") + name + " is not in the model alphabet");
  return c;
}

std::vector<double> Vec(const double *p, int n, const char *what) {
  Require(p != nullptr || n == 0, LMC_ERR_INVALID_ARGUMENT, std::string(what) + " is null");
  return std::vector<double>(p, p + n);
}

// Tables of the sparse KMC evaluation for dominant species `base` (see KmcSparse).
void BuildSparse(lmc_ctx *c, int base) {
  if (c->sparse_base == base) return;  // the tables depend only on the model and the base species
  const auto &pt = lmc::GetPairTables();
  const auto &fm = c->fm;
  const int e = fm.num_species, x = fm.x_code, eh = fm.num_onehot;
  const int rb0 = fm.onehot_rank[base];
  Require(rb0 >= 0 && base != x, LMC_ERR_INVALID_ARGUMENT, "dominant species has no one-hot slot");
  for (auto &b : c->sparse_bufs) b.Free();
  c->sparse_bufs.clear();
  lmc::KmcSparse sp{};
  sp.base_code = base;
  sp.x_code = fm.x_code;
  auto w = [&](int label, int c0, int c1, int c2) {
    return static_cast<long long>(fm.w_de[((label * e + c0) * e + c1) * e + c2]);
  };
  // energy-change term of one cluster whose pair site holds M (first site) and
  // whose other sites hold (c1, c2), base subtracted; symmetric in (c1, c2)
  std::vector<long long> f_de(static_cast<size_t>(8) * e * e * e, 0), p_de(f_de.size(), 0);
  auto F = [&](int label, int m, int c1, int c2) { return f_de[((label * e + m) * e + c1) * e + c2]; };
  for (int label = 1; label < 8; ++label)
    for (int m = 0; m < e; ++m)
      for (int c1 = 0; c1 < e; ++c1)
        for (int c2 = 0; c2 < e; ++c2) {
          if (label <= 3 && c2 != 0) continue;
          const int b2 = label <= 3 ? 0 : base;
          f_de[((label * e + m) * e + c1) * e + c2] =
              (w(label, m, c1, c2) - w(label, x, c1, c2)) - (w(label, m, base, b2) - w(label, x, base, b2));
        }
  for (int label = 4; label < 8; ++label)
    for (int m = 0; m < e; ++m)
      for (int c1 = 0; c1 < e; ++c1)
        for (int c2 = 0; c2 < e; ++c2)
          p_de[((label * e + m) * e + c1) * e + c2] = F(label, m, c1, c2) - F(label, m, c1, base) - F(label, m, base, c2);
  // state-list clusters with exactly one pair site
  std::vector<long long> base_de(e, 0), s_de(static_cast<size_t>(e) * (lmc::kStateSites + 1) * e, 0);
  std::vector<uint16_t> px_st(lmc::kTriState + 1, 0);
  for (const auto &cl : pt.state_clusters) {
    int has_first = 0, has_second = 0;
    std::vector<int> others;
    for (int q = 0; q < cl.size; ++q) {
      if (cl.idx[q] == pt.pos_first) has_first = 1;
      else if (cl.idx[q] == pt.pos_second) has_second = 1;
      else others.push_back(cl.idx[q]);
    }
    if (has_first + has_second != 1 || others.empty()) continue;  // cancel when the first site is the vacancy
    const long long sign = has_second ? -1 : 1;
    const int b2 = others.size() > 1 ? base : 0;
    for (int m = 0; m < e; ++m) base_de[m] += sign * (w(cl.label, m, base, b2) - w(cl.label, x, base, b2));
    for (size_t k = 0; k < others.size(); ++k) {
      const int p = others[k];
      for (int m = 0; m < e; ++m)
        for (int sp_code = 0; sp_code < e; ++sp_code)
          s_de[(static_cast<size_t>(m) * (lmc::kStateSites + 1) + p) * e + sp_code] += sign * F(cl.label, m, sp_code, b2);
    }
    if (others.size() == 2) {
      const uint16_t code = static_cast<uint16_t>(cl.label | (has_second << 3));
      Require(cl.label >= 4, LMC_ERR_UNSUPPORTED, "unexpected triplet label");
      uint16_t &slot = px_st[lmc::Tri(others[0], others[1])];
      if ((slot & 0xFF) == 0) slot = static_cast<uint16_t>((slot & 0xFF00) | code);
      else if ((slot >> 8) == 0) slot = static_cast<uint16_t>((slot & 0x00FF) | (code << 8));
      else Require(false, LMC_ERR_UNSUPPORTED, "more than two triplets share a site pair");
    }
  }
  // environment lists: W - W(base block entry) per feature, single-site terms, pair lookup
  const int slots = static_cast<int>(fm.slot_code.size());
  std::vector<long long> dwd, dwks, dwe0, base_form(3 * std::max(1, slots), 0);
  std::vector<long long> s_env(static_cast<size_t>(std::max(1, slots)) * 3 * (lmc::kEnvSites + 1) * 8, 0);
  constexpr uint32_t kNone = 0xFFFFFFFFu;
  std::vector<uint32_t> px_env(2 * (lmc::kTriEnv + 1), kNone);
  auto env_tables = [&](const lmc::EnvEncoding &enc, int which) {
    const auto ooff = enc.OrbitOffsets(eh);
    Require(ooff.back() < (1 << 20), LMC_ERR_UNSUPPORTED, "too many environment features");
    for (const auto &cl : enc.clusters) {
      if (cl.b < 0) continue;
      const uint32_t v = static_cast<uint32_t>(ooff[cl.orbit]) | (static_cast<uint32_t>(cl.mode) << 20);
      uint32_t &v_tri = px_env[which * (lmc::kTriEnv + 1) + lmc::Tri(cl.a, cl.b)];
      Require(v_tri == kNone && cl.a != cl.b, LMC_ERR_UNSUPPORTED, "two clusters share a site pair");
      v_tri = v | (cl.a < cl.b ? (1u << 22) : 0u);
    }
    // no cluster: an ordered-pair entry in the block of 64 zeros after the features
    const uint32_t none = static_cast<uint32_t>(ooff.back()) | (1u << 20);
    for (int i = 0; i <= lmc::kTriEnv; ++i) {
      uint32_t &v = px_env[which * (lmc::kTriEnv + 1) + i];
      if (v == kNone) v = none;
      else Require(i < lmc::kTriEnv, LMC_ERR_UNSUPPORTED, "pair lookup overflow");
    }
    return ooff;
  };
  const auto off_mmm = env_tables(pt.mmm, 0);
  const auto off_mm2 = env_tables(pt.mm2, 1);
  auto delta = [&](const lmc::EnvEncoding &enc, const std::vector<int> &ooff, const std::vector<int64_t> &wv,
                   std::vector<long long> &out, long long *base_sum, int mult, long long *single) {
    const size_t first = out.size();
    for (size_t o = 0; o < enc.orbits.size(); ++o) {
      const long long w0 = wv[ooff[o] + lmc::PairType(enc.orbits[o].mode, rb0, rb0, eh)];
      for (int j = ooff[o]; j < ooff[o + 1]; ++j) out.push_back(wv[j] - w0);
      *base_sum += static_cast<long long>(mult) * w0 * enc.orbits[o].size;
    }
    out.insert(out.end(), 64, 0);  // zero block addressed by "no cluster" lookups
    const long long *dw = out.data() + first;
    for (const auto &cl : enc.clusters) {
      const int fb = ooff[cl.orbit];
      for (int r = 0; r < eh; ++r) {
        if (cl.b < 0) {
          single[cl.a * 8 + r] += dw[fb + lmc::PairType(0, r, 0, eh)];
        } else {
          single[cl.a * 8 + r] += dw[fb + lmc::PairType(cl.mode, r, rb0, eh)];
          single[cl.b * 8 + r] += dw[fb + lmc::PairType(cl.mode, rb0, r, eh)];
        }
      }
    }
  };
  for (int sidx = 0; sidx < slots; ++sidx) {
    long long *sg = s_env.data() + static_cast<size_t>(sidx) * 3 * (lmc::kEnvSites + 1) * 8;
    delta(pt.mmm, off_mmm, fm.quartic_d[sidx].w, dwd, &base_form[sidx * 3 + 0], 1, sg);
    delta(pt.mm2, off_mm2, fm.quartic_ks[sidx].w, dwks, &base_form[sidx * 3 + 1], 2, sg + (lmc::kEnvSites + 1) * 8);
    delta(pt.mmm, off_mmm, fm.e0[sidx].w, dwe0, &base_form[sidx * 3 + 2], 1, sg + 2 * (lmc::kEnvSites + 1) * 8);
  }
  // local index -> list position for each jump
  std::vector<uint8_t> pos(4 * 12 * 136, 255);
  std::vector<uint8_t> l_st(12 * lmc::kStateSites), l_mmm(12 * lmc::kEnvSites), l_f(12 * lmc::kEnvSites),
      l_b(12 * lmc::kEnvSites);
  CudaCheck(cudaMemcpy(l_st.data(), c->t.local_st, l_st.size(), cudaMemcpyDeviceToHost), "D2H");
  CudaCheck(cudaMemcpy(l_mmm.data(), c->t.local_mmm, l_mmm.size(), cudaMemcpyDeviceToHost), "D2H");
  CudaCheck(cudaMemcpy(l_f.data(), c->t.local_mm2f, l_f.size(), cudaMemcpyDeviceToHost), "D2H");
  CudaCheck(cudaMemcpy(l_b.data(), c->t.local_mm2b, l_b.size(), cudaMemcpyDeviceToHost), "D2H");
  for (int d = 0; d < 12; ++d) {
    for (int k = 0; k < lmc::kStateSites; ++k)
      if (k != pt.pos_first && k != pt.pos_second) pos[(0 * 12 + d) * 136 + l_st[d * lmc::kStateSites + k]] = k;
    for (int k = 0; k < lmc::kEnvSites; ++k) {
      pos[(1 * 12 + d) * 136 + l_mmm[d * lmc::kEnvSites + k]] = static_cast<uint8_t>(k);
      pos[(2 * 12 + d) * 136 + l_f[d * lmc::kEnvSites + k]] = static_cast<uint8_t>(k);
      pos[(3 * 12 + d) * 136 + l_b[d * lmc::kEnvSites + k]] = static_cast<uint8_t>(k);
    }
  }
  // local pairs that share a cluster in some jump's list
  std::vector<uint32_t> inter(lmc::kLocalSites * lmc::kInterWords, 0u);
  auto mark = [&](int a, int b) {
    inter[a * lmc::kInterWords + (b >> 5)] |= 1u << (b & 31);
    inter[b * lmc::kInterWords + (a >> 5)] |= 1u << (a & 31);
  };
  for (int d = 0; d < 12; ++d) {
    for (int p = 0; p < lmc::kStateSites; ++p)
      for (int q = 0; q < p; ++q)
        if (px_st[lmc::Tri(p, q)] != 0) mark(l_st[d * lmc::kStateSites + p], l_st[d * lmc::kStateSites + q]);
    const uint8_t *lists[3] = {l_mmm.data(), l_f.data(), l_b.data()};
    for (int li = 0; li < 3; ++li)
      for (int p = 0; p < lmc::kEnvSites; ++p)
        for (int q = 0; q < p; ++q)
          if (px_env[(li == 0 ? 0 : 1) * (lmc::kTriEnv + 1) + lmc::Tri(p, q)] !=
              px_env[(li == 0 ? 0 : 1) * (lmc::kTriEnv + 1) + lmc::kTriEnv])
            mark(lists[li][d * lmc::kEnvSites + p], lists[li][d * lmc::kEnvSites + q]);
  }
  auto &B = c->sparse_bufs;
  sp.pos = c->Upload(pos, &B);
  sp.inter = c->Upload(inter, &B);
  sp.s_de = c->Upload(s_de, &B);
  sp.s_env = c->Upload(s_env, &B);
  sp.px_st = c->Upload(px_st, &B);
  sp.px_env = c->Upload(px_env, &B);
  sp.p_de = c->Upload(p_de, &B);
  sp.base_de = c->Upload(base_de, &B);
  sp.dw_d = c->Upload(dwd, &B);
  sp.dw_ks = c->Upload(dwks, &B);
  sp.dw_e0 = c->Upload(dwe0, &B);
  sp.base_form = c->Upload(base_form, &B);
  sp.center = l_st[pt.pos_first];
  sp.dw_stride_mmm = off_mmm.back() + 64;
  sp.dw_stride_mm2 = off_mm2.back() + 64;
  c->sparse = sp;
  c->sparse_base = base;
}

void KmcDefaults(const lmc_ctx *c, int *g, int *rpb) {
  // Enough warps to fill the GPU: one warp per replica when there are
  // thousands of replicas, up to one warp per jump for a single trajectory.
  int sms = 152;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
  const long long r = c->num_replicas;
  const long long target = static_cast<long long>(sms) * 24;
  int best = 12;
  for (int cand : {1, 2, 3, 4, 6, 12})
    if (r * cand >= target) {
      best = cand;
      break;
    }
  *g = best;
  *rpb = std::max(1, 8 / best);  // 256-thread blocks
  if (best == 1 && c->kmc_opt.evaluation != LMC_EVAL_DENSE && r <= 28LL * sms) {
    // one block per SM holding an equal share of the replicas
    *rpb = static_cast<int>((r + sms - 1) / sms);
  }
}

// Block shape and evaluation of the KMC launch from the options (0 = default).
lmc::KmcLaunch KmcShape(const lmc_ctx *ctx) {
  lmc::KmcLaunch l{};
  int g = ctx->kmc_opt.warps_per_replica, rpb = ctx->kmc_opt.replicas_per_block;
  int dg, drpb;
  KmcDefaults(ctx, &dg, &drpb);
  if (g <= 0) g = dg;
  if (rpb <= 0) rpb = drpb;
  Require(g == 1 || g == 2 || g == 3 || g == 4 || g == 6 || g == 12, LMC_ERR_INVALID_ARGUMENT,
          "warps_per_replica must divide 12");
  Require(g * rpb <= 12 || (g == 1 && rpb <= 28), LMC_ERR_INVALID_ARGUMENT,
          "at most 12 warps per block (384 threads), or 28 single-warp replicas");
  Require(g == 1 || rpb <= 15, LMC_ERR_INVALID_ARGUMENT, "at most 15 multi-warp replicas per block");
  l.warps_per_replica = g;
  l.replicas_per_block = rpb;
  l.sparse = ctx->kmc_opt.evaluation == LMC_EVAL_DENSE ? 0 : 1;
  l.mt = ctx->kmc_opt.rng == LMC_RNG_MT19937_64 ? 1 : 0;
  l.f32 = !l.mt && ctx->kmc_opt.rates == LMC_RATES_FP32 ? 1 : 0;
  l.sp = ctx->sparse;
  return l;
}


// Device state of the KMC kernel (pointers into the context's buffers).
lmc::KmcDevState KmcState(const lmc_ctx *ctx) {
  lmc::KmcDevState s{};
  s.vacancy = ctx->k_vac.as<long long>();
  s.steps = ctx->k_steps.as<unsigned long long>();
  s.time = ctx->k_time.as<double>();
  s.energy = ctx->k_energy.as<double>();
  s.temperature = ctx->k_temp.as<double>();
  s.corr_cvac = ctx->k_cvac.as<double>();
  s.corr_csol = ctx->k_csol.as<double>();
  s.early_stop = ctx->kmc_opt.early_stop ? 1 : 0;
  s.solvent = ctx->k_solvent.as<int8_t>();
  s.escaped = ctx->k_escaped.as<uint8_t>();
  s.rng = ctx->k_rng.as<uint32_t>();
  s.lat_off = ctx->lat_off.as<long long>();
  s.lat_n = ctx->lat_n.as<int>();
  s.num_replicas = ctx->num_replicas;
  s.rng_kind = ctx->kmc_opt.rng;
  s.barrier_kind = ctx->kmc_opt.barrier_kind;
  s.tt_time = ctx->tt_len ? ctx->k_tt_time.as<double>() : nullptr;
  s.tt_temp = ctx->tt_len ? ctx->k_tt_temp.as<double>() : nullptr;
  s.tt_len = ctx->tt_len;
  s.prev = ctx->k_prev.as<long long>();
  return s;
}
// ---- KMC launch-shape autotuner -------------------------------------------
// Sweeps the (warps per replica, replicas per block, evaluation) shapes the
// kernel accepts on a short probe of the context's own replicas, keeps the
// fastest, and caches it in a JSON file keyed by the GPU, its SM count and the
// histogram of supercell sizes. Every shape gives bit-identical trajectories
// (integer cluster sums, per-replica RNG streams), so the choice is pure speed;
// the probe runs on a copy of the state, which is put back afterwards.

struct KmcTuneEntry {
  int g{1}, rpb{1}, eval{LMC_EVAL_SPARSE};
  double ms{0};
  uint64_t probe_steps{0};
};

std::string KmcTuneKey(const lmc_ctx *ctx) {
  cudaDeviceProp prop{};
  CudaCheck(cudaGetDeviceProperties(&prop, ctx->device), "cudaGetDeviceProperties");
  std::map<int, int> hist;
  for (int v : ctx->n) ++hist[v];
  std::string name = prop.name;
  for (char &ch : name)
    if (ch == '"' || ch == '\\' || static_cast<unsigned char>(ch) < 32) ch = '_';
  std::string k = "kmc1|" + name + "|sm" + std::to_string(prop.major) + std::to_string(prop.minor) + "|sms=" +
                  std::to_string(prop.multiProcessorCount) + "|R=" + std::to_string(ctx->num_replicas) + "|n=";
  bool first = true;
  for (const auto &kv : hist) {
    k += (first ? "" : ",") + std::to_string(kv.first) + ":" + std::to_string(kv.second);
    first = false;
  }
  k += "|E=" + std::to_string(ctx->fm.num_species) + "|kind=" + std::to_string(ctx->kmc_opt.barrier_kind) +
       "|rng=" + std::to_string(ctx->kmc_opt.rng) + "|stop=" + std::to_string(ctx->kmc_opt.early_stop ? 1 : 0) +
       "|tt=" + std::to_string(ctx->tt_len > 0 ? 1 : 0) + "|corr=" + std::to_string(ctx->kmc_opt.rate_corrector ? 1 : 0) +
       "|rates=" + std::to_string(ctx->kmc_opt.rates);
  return k;
}

std::map<std::string, KmcTuneEntry> ReadTuneCache(const char *path) {
  std::map<std::string, KmcTuneEntry> out;
  std::ifstream f(path);
  if (!f) return out;  // no cache yet
  std::stringstream ss;
  ss << f.rdbuf();
  try {
    const lmc::JsonValue v = lmc::JsonValue::Parse(ss.str());
    if (!v.IsObject()) return out;
    for (const auto &kv : v.Object()) {
      const lmc::JsonValue &e = kv.second;
      if (!e.Has("warps_per_replica") || !e.Has("replicas_per_block") || !e.Has("evaluation")) continue;
      KmcTuneEntry t;
      t.g = static_cast<int>(e.At("warps_per_replica").Number());
      t.rpb = static_cast<int>(e.At("replicas_per_block").Number());
      t.eval = static_cast<int>(e.At("evaluation").Number());
      if (e.Has("ms")) t.ms = e.At("ms").Number();
      if (e.Has("probe_steps")) t.probe_steps = static_cast<uint64_t>(e.At("probe_steps").Number());
      out[kv.first] = t;
    }
  } catch (const std::exception &) {
    out.clear();  // an unreadable cache is ignored and rewritten
  }
  return out;
}

void WriteTuneCache(const char *path, const std::map<std::string, KmcTuneEntry> &cache) {
  const std::string tmp = std::string(path) + ".tmp";
  {
    std::ofstream f(tmp);
    Require(static_cast<bool>(f), LMC_ERR_IO, std::string("Cannot open ") + tmp);
    f << "{\n";
    size_t i = 0;
    for (const auto &kv : cache) {
      char ms[64];
      std::snprintf(ms, sizeof(ms), "%.6g", kv.second.ms);
      f << "  \"" << kv.first << "\": {\"warps_per_replica\": " << kv.second.g
        << ", \"replicas_per_block\": " << kv.second.rpb << ", \"evaluation\": " << kv.second.eval
        << ", \"ms\": " << ms << ", \"probe_steps\": " << kv.second.probe_steps << "}"
        << (++i < cache.size() ? ",\n" : "\n");
    }
    f << "}\n";
    Require(static_cast<bool>(f), LMC_ERR_IO, std::string("Cannot write ") + tmp);
  }
  Require(std::rename(tmp.c_str(), path) == 0, LMC_ERR_IO, std::string("Cannot write ") + path);
}

// The mutable KMC state of a context (lattices and per-replica records).
struct KmcSnapshot {
  std::vector<std::pair<const DevBuf *, DevBuf>> bufs;
  size_t species_bytes{0};
  void Save(lmc_ctx *ctx) {
    const size_t R = ctx->num_replicas;
    species_bytes = static_cast<size_t>(ctx->total_sites);
    const std::pair<const DevBuf *, size_t> src[] = {
        {&ctx->species, species_bytes}, {&ctx->k_vac, 8 * R},    {&ctx->k_steps, 8 * R},
        {&ctx->k_time, 8 * R},          {&ctx->k_energy, 8 * R}, {&ctx->k_temp, 8 * R},
        {&ctx->k_rng, sizeof(uint32_t) * lmc::kRngWords * R},    {&ctx->k_escaped, R}};
    for (const auto &p : src) {
      DevBuf copy;
      copy.Alloc(p.second);
      CudaCheck(cudaMemcpyAsync(copy.p, p.first->p, p.second, cudaMemcpyDeviceToDevice, ctx->stream), "D2D save");
      bufs.emplace_back(p.first, copy);
    }
  }
  void Restore(lmc_ctx *ctx) {
    for (auto &p : bufs)
      CudaCheck(cudaMemcpyAsync(p.first->p, p.second.p, p.second.bytes, cudaMemcpyDeviceToDevice, ctx->stream),
                "D2D restore");
  }
  ~KmcSnapshot() {
    for (auto &p : bufs) p.second.Free();
  }
};

KmcTuneEntry SweepKmcShapes(lmc_ctx *ctx, uint64_t probe_steps) {
  const lmc_kmc_options saved = ctx->kmc_opt;
  int sms = 152;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
  const int R = ctx->num_replicas;
  std::vector<KmcTuneEntry> cands;
  for (int eval : {LMC_EVAL_SPARSE, LMC_EVAL_DENSE}) {
    std::vector<int> rpbs = {1, 2, 4, 8, 12, 16, 20, 24, 28};
    const int wave = (R + sms - 1) / sms;  // one block per SM
    if (wave >= 1 && wave <= 28) rpbs.push_back(wave);
    std::sort(rpbs.begin(), rpbs.end());
    rpbs.erase(std::unique(rpbs.begin(), rpbs.end()), rpbs.end());
    for (int rpb : rpbs) cands.push_back({1, rpb, eval});
    for (int g : {2, 3, 4, 6, 12})
      for (int rpb = 1; g * rpb <= 12; rpb *= 2) cands.push_back({g, rpb, eval});
  }
  KmcSnapshot snap;
  snap.Save(ctx);
  const lmc::KmcDevState s = KmcState(ctx);
  KmcTuneEntry best{};
  best.ms = std::numeric_limits<double>::infinity();
  try {
    for (KmcTuneEntry c : cands) {
      ctx->kmc_opt.warps_per_replica = c.g;
      ctx->kmc_opt.replicas_per_block = c.rpb;
      ctx->kmc_opt.evaluation = c.eval;
      lmc::KmcLaunch l{};
      try {
        l = KmcShape(ctx);
      } catch (const LmcError &) {
        continue;  // shape the kernel does not accept
      }
      int per_sm = 0;
      size_t bytes = 0;
      if (lmc::KmcOccupancy(ctx->t, l, &per_sm, &bytes) != cudaSuccess || per_sm < 1) {
        cudaGetLastError();
        continue;
      }
      l.steps = probe_steps;
      l.trace_replica = -1;
      l.stop_flag = ctx->d_stop;
      l.status = ctx->status.as<int>();
      double best_c = std::numeric_limits<double>::infinity();
      for (int rep = 0; rep < 3; ++rep) {  // first repetition warms caches and the instruction stream
        ctx->ClearStatus();
        CudaCheck(cudaEventRecord(ctx->ev0, ctx->stream), "event");
        CudaCheck(lmc::LaunchKmc(ctx->t, ctx->species.as<int8_t>(), s, l, ctx->stream), "KMC kernel");
        CudaCheck(cudaEventRecord(ctx->ev1, ctx->stream), "event");
        const int st = ctx->ReadStatus();
        snap.Restore(ctx);
        RaiseStatus(st, "KMC autotune probe");
        float ms = 0;
        CudaCheck(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1), "elapsed");
        if (rep > 0) best_c = std::min(best_c, static_cast<double>(ms));
      }
      if (best_c < best.ms) {
        best = c;
        best.ms = best_c;
      }
    }
  } catch (...) {
    snap.Restore(ctx);
    ctx->Sync();
    ctx->kmc_opt = saved;
    throw;
  }
  ctx->Sync();
  ctx->kmc_opt = saved;
  Require(std::isfinite(best.ms), LMC_ERR_UNSUPPORTED, "no KMC launch shape fits this device");
  best.probe_steps = probe_steps;
  return best;
}

// Number of distinct species in a replica's lattice (device scan).
int SpeciesPresent(lmc_ctx *ctx, int replica) {
  DevBuf hist, first;
  hist.Alloc(sizeof(unsigned long long) * (lmc::kMaxSpecies + 1));
  first.Alloc(sizeof(long long));
  const long long big = std::numeric_limits<long long>::max();
  CudaCheck(cudaMemcpyAsync(first.p, &big, sizeof(big), cudaMemcpyHostToDevice, ctx->stream), "H2D");
  CudaCheck(cudaMemsetAsync(hist.p, 0, hist.bytes, ctx->stream), "memset");
  CudaCheck(lmc::LaunchReplicaScan(ctx->species.as<int8_t>(), ctx->lat_off.as<long long>() + replica,
                                   ctx->lat_n.as<int>() + replica, 1, ctx->fm.x_code, ctx->fm.num_species,
                                   first.as<long long>(), hist.as<unsigned long long>(), ctx->stream),
            "scan kernel");
  unsigned long long h[lmc::kMaxSpecies + 1];
  CudaCheck(cudaMemcpyAsync(h, hist.p, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream), "D2H");
  ctx->Sync();
  int present = 0;
  for (int c = 0; c < ctx->fm.num_species; ++c) present += h[c] > 0;
  return present;
}

}  // namespace

extern "C" {

const char *lmc_strerror(int status) {
  switch (status) {
    case LMC_OK: return "ok";
    case LMC_ERR_INVALID_ARGUMENT: return "invalid argument";
    case LMC_ERR_OUT_OF_RANGE: return "out of range";
    case LMC_ERR_IO: return "i/o error";
    case LMC_ERR_CUDA: return "CUDA error";
    case LMC_ERR_NO_DEVICE: return "no usable CUDA device";
    case LMC_ERR_NUMERIC: return "numeric error";
    case LMC_ERR_STOPPED: return "stopped";
    case LMC_ERR_UNSUPPORTED: return "unsupported";
    default: return "unknown status";
  }
}

const char *lmc_last_error(void) { return g_error.c_str(); }
const char *lmc_version(void) { return "lmc_gb300 0.1 sm_103a"; }

int lmc_model_create(const char *const *element_names, int num_elements, lmc_model **out) {
  return Guard([&] {
    Require(out != nullptr, LMC_ERR_INVALID_ARGUMENT, "out is null");
    auto m = std::make_unique<lmc_model>();
    m->m = lmc::MakeModel(Names(element_names, num_elements));
    *out = m.release();
  });
}

int lmc_model_load_json(const char *path, const char *const *element_names, int num_elements, lmc_model **out) {
  return Guard([&] {
    Require(out != nullptr && path != nullptr, LMC_ERR_INVALID_ARGUMENT, "null argument");
    auto m = std::make_unique<lmc_model>();
    m->m = lmc::MakeModel(Names(element_names, num_elements));
    lmc::LoadJson(m->m, path);
    *out = m.release();
  });
}

void lmc_model_destroy(lmc_model *model) { delete model; }

int lmc_model_num_species(const lmc_model *model) { return model ? model->m.NumSpecies() : -1; }

int lmc_model_species_code(const lmc_model *model, const char *name) {
  if (!model || !name) return -1;
  return model->m.Code(name);
}

int lmc_model_alphabet(const lmc_model *model, char *buf, int buflen) {
  return Guard([&] {
    Require(model && buf && buflen > 0, LMC_ERR_INVALID_ARGUMENT, "null argument");
    std::string s;
    for (size_t i = 0; i < model->m.alphabet.size(); ++i) s += (i ? " " : "") + model->m.alphabet[i];
    Require(static_cast<int>(s.size()) < buflen, LMC_ERR_INVALID_ARGUMENT, "buffer too small");
    std::memcpy(buf, s.c_str(), s.size() + 1);
  });
}

int lmc_model_layout(const lmc_model *model, int *num_theta, int *f_mmm, int *f_mm2) {
  return Guard([&] {
    Require(model != nullptr, LMC_ERR_INVALID_ARGUMENT, "model is null");
    if (num_theta) *num_theta = model->m.num_theta;
    if (f_mmm) *f_mmm = model->m.FeaturesMmm();
    if (f_mm2) *f_mm2 = model->m.FeaturesMm2();
  });
}

int lmc_model_feature_orbit_sizes(const lmc_model *model, int which, int32_t *sizes) {
  return Guard([&] {
    Require(model && sizes && (which == 0 || which == 1), LMC_ERR_INVALID_ARGUMENT, "bad argument");
    const auto &e = which == 0 ? lmc::GetPairTables().mmm : lmc::GetPairTables().mm2;
    const auto off = e.OrbitOffsets(model->m.NumOnehot());
    for (size_t o = 0; o < e.orbits.size(); ++o)
      for (int j = off[o]; j < off[o + 1]; ++j) sizes[j] = e.orbits[o].size;
  });
}

int lmc_model_set_base_theta(lmc_model *model, const double *theta, int n) {
  return Guard([&] {
    Require(model != nullptr, LMC_ERR_INVALID_ARGUMENT, "model is null");
    Require(n == model->m.num_theta, LMC_ERR_INVALID_ARGUMENT,
            "theta has " + std::to_string(n) + " entries, expected " + std::to_string(model->m.num_theta));
    model->m.base_theta = Vec(theta, n, "theta");
  });
}

int lmc_model_set_quartic(lmc_model *model, const char *migrant, const lmc_quartic_params *p) {
  return Guard([&] {
    Require(model && p, LMC_ERR_INVALID_ARGUMENT, "null argument");
    const int code = CodeOf(model->m, migrant);
    const int fm = model->m.FeaturesMmm(), f2 = model->m.FeaturesMm2();
    Require(p->k_mmm > 0 && p->k_mm2 > 0, LMC_ERR_INVALID_ARGUMENT, "k must be positive");
    lmc::QuarticBlock q;
    q.k_mmm = p->k_mmm;
    q.k_mm2 = p->k_mm2;
    q.mu_x_mmm = Vec(p->mu_x_mmm, fm, "mu_x_mmm");
    q.sigma_x_mmm = Vec(p->sigma_x_mmm, fm, "sigma_x_mmm");
    q.mu_x_mm2 = Vec(p->mu_x_mm2, f2, "mu_x_mm2");
    q.sigma_x_mm2 = Vec(p->sigma_x_mm2, f2, "sigma_x_mm2");
    q.u_mmm = Vec(p->u_mmm, p->k_mmm * fm, "u_mmm");
    q.u_mm2 = Vec(p->u_mm2, p->k_mm2 * f2, "u_mm2");
    q.theta_d = Vec(p->theta_d, p->k_mmm, "theta_d");
    q.theta_ks = Vec(p->theta_ks, p->k_mm2, "theta_ks");
    q.mu_d = p->mu_d;
    q.sigma_d = p->sigma_d;
    q.mu_ks = p->mu_ks;
    q.sigma_ks = p->sigma_ks;
    model->m.quartic[code] = std::move(q);
  });
}

int lmc_model_set_e0(lmc_model *model, const char *migrant, const lmc_e0_params *p) {
  return Guard([&] {
    Require(model && p, LMC_ERR_INVALID_ARGUMENT, "null argument");
    const int code = CodeOf(model->m, migrant);
    const int fm = model->m.FeaturesMmm();
    Require(p->k_mmm > 0, LMC_ERR_INVALID_ARGUMENT, "k must be positive");
    lmc::E0Block b;
    b.k_mmm = p->k_mmm;
    b.mu_x_mmm = Vec(p->mu_x_mmm, fm, "mu_x_mmm");
    b.sigma_x_mmm = Vec(p->sigma_x_mmm, fm, "sigma_x_mmm");
    b.u_mmm = Vec(p->u_mmm, p->k_mmm * fm, "u_mmm");
    b.theta_e0 = Vec(p->theta_e0, p->k_mmm, "theta_e0");
    b.mu_e0 = p->mu_e0;
    b.sigma_e0 = p->sigma_e0;
    model->m.e0[code] = std::move(b);
  });
}

int lmc_geom_neighbors(int n, int64_t site, int64_t *out42) {
  return Guard([&] {
    Require(n >= 6 && out42, LMC_ERR_INVALID_ARGUMENT, "n must be >= 6");
    const lmc::Fcc fcc{n};
    Require(site >= 0 && site < fcc.NumSites(), LMC_ERR_OUT_OF_RANGE, "site out of range");
    int k = 0;
    for (int shell = 1; shell <= 3; ++shell)
      for (auto id : lmc::SortedNeighbors(fcc, site, shell)) out42[k++] = id;
  });
}

int lmc_geom_pair_lists(int n, int64_t first, int64_t second, int64_t *state60, int64_t *mmm58, int64_t *mm258) {
  return Guard([&] {
    Require(n >= 6, LMC_ERR_INVALID_ARGUMENT, "n must be >= 6");
    const lmc::Fcc fcc{n};
    const auto &pt = lmc::GetPairTables();
    Require(first >= 0 && second >= 0 && first < fcc.NumSites() && second < fcc.NumSites(), LMC_ERR_OUT_OF_RANGE,
            "site out of range");
    const lmc::I3 hi = fcc.Coord(first), hj = fcc.Coord(second);
    auto mi = [&](int v) { const int m2 = 2 * n; v %= m2; if (v < 0) v += m2; return v >= n ? v - m2 : v; };
    const lmc::I3 d{mi(hj.x - hi.x), mi(hj.y - hi.y), mi(hj.z - hi.z)};
    const int di = lmc::DirectionIndex(d);
    Require(di >= 0, LMC_ERR_OUT_OF_RANGE, "Neighbor not found for lattice pair in GetPairFlatIndex");
    for (int k = 0; k < lmc::kStateSites && state60; ++k) state60[k] = fcc.Id(fcc.Wrap(hi + pt.state_off[di][k]));
    for (int k = 0; k < lmc::kEnvSites && mmm58; ++k) mmm58[k] = fcc.Id(fcc.Wrap(hi + pt.mmm_off[di][k]));
    for (int k = 0; k < lmc::kEnvSites && mm258; ++k) mm258[k] = fcc.Id(fcc.Wrap(hi + pt.mm2_off[di][k]));
  });
}

int lmc_geom_site_list(int n, int64_t site, int64_t *out43) {
  return Guard([&] {
    Require(n >= 6 && out43, LMC_ERR_INVALID_ARGUMENT, "n must be >= 6");
    const lmc::Fcc fcc{n};
    Require(site >= 0 && site < fcc.NumSites(), LMC_ERR_OUT_OF_RANGE, "site out of range");
    const auto &pt = lmc::GetPairTables();
    const lmc::I3 h = fcc.Coord(site);
    for (int k = 0; k < lmc::kSiteSites; ++k) out43[k] = fcc.Id(fcc.Wrap(h + pt.site_off[k]));
  });
}

int lmc_geom_mapping_sizes(int *counts20) {
  return Guard([&] {
    Require(counts20 != nullptr, LMC_ERR_INVALID_ARGUMENT, "null argument");
    const auto &pt = lmc::GetPairTables();
    std::fill(counts20, counts20 + 20, 0);
    for (const auto &c : pt.state_clusters) ++counts20[c.label];
    for (const auto &c : pt.site_clusters) ++counts20[8 + c.label];
    counts20[16] = static_cast<int>(pt.mmm.orbits.size());
    counts20[17] = static_cast<int>(pt.mm2.orbits.size());
    counts20[18] = static_cast<int>(pt.mmm.clusters.size());
    counts20[19] = static_cast<int>(pt.mm2.clusters.size());
  });
}

int lmc_geom_env_mapping(int which, int32_t *orbit_a_b, int cap, int *n) {
  return Guard([&] {
    Require(which == 0 || which == 1, LMC_ERR_INVALID_ARGUMENT, "which must be 0 (MMM) or 1 (MM2)");
    const auto &e = which == 0 ? lmc::GetPairTables().mmm : lmc::GetPairTables().mm2;
    if (n) *n = static_cast<int>(e.clusters.size());
    for (int i = 0; i < static_cast<int>(e.clusters.size()) && i < cap && orbit_a_b; ++i) {
      orbit_a_b[3 * i] = e.clusters[i].orbit;
      orbit_a_b[3 * i + 1] = e.clusters[i].a;
      orbit_a_b[3 * i + 2] = e.clusters[i].b;
    }
  });
}

int lmc_host_encode_pair(const lmc_model *model, int n, const int8_t *species, int64_t first, int64_t second,
                         int32_t *state_start, int32_t *state_end, int32_t *mmm, int32_t *mm2_fwd,
                         int32_t *mm2_bwd) {
  return Guard([&] {
    Require(model && species && n >= 6, LMC_ERR_INVALID_ARGUMENT, "bad argument");
    lmc::HostEncodePair(model->m, n, species, first, second, state_start, state_end, mmm, mm2_fwd, mm2_bwd);
  });
}

int lmc_ctx_create(const lmc_model *model, int device, lmc_ctx **out) {
  return Guard([&] {
    Require(model && out, LMC_ERR_INVALID_ARGUMENT, "null argument");
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
      cudaGetLastError();
      throw LmcError(LMC_ERR_NO_DEVICE, "no CUDA device available");
    }
    Require(device >= 0 && device < count, LMC_ERR_NO_DEVICE, "device index out of range");
    CudaCheck(cudaSetDevice(device), "cudaSetDevice");
    auto c = std::make_unique<lmc_ctx>();
    c->device = device;
    c->model = model->m;
    c->fm = lmc::Fold(c->model);
    CudaCheck(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking), "cudaStreamCreate");
    CudaCheck(cudaEventCreate(&c->ev0), "cudaEventCreate");
    CudaCheck(cudaEventCreate(&c->ev1), "cudaEventCreate");
    CudaCheck(cudaHostAlloc(reinterpret_cast<void **>(&c->h_stop), sizeof(int), cudaHostAllocMapped),
              "cudaHostAlloc");
    *c->h_stop = 0;
    CudaCheck(cudaHostGetDevicePointer(reinterpret_cast<void **>(&c->d_stop), c->h_stop, 0), "mapped pointer");
    BuildTables(c.get());
    c->status.Alloc(sizeof(int));
    c->counts.Alloc(sizeof(unsigned long long) * 256);
    c->energy.Alloc(sizeof(double) * 4);
    *out = c.release();
  });
}

void lmc_ctx_destroy(lmc_ctx *ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  delete ctx;
}

int lmc_ctx_synchronize(lmc_ctx *ctx) {
  return Guard([&] {
    Require(ctx != nullptr, LMC_ERR_INVALID_ARGUMENT, "ctx is null");
    ctx->Sync();
  });
}

int lmc_ctx_set_lattices(lmc_ctx *ctx, int num_replicas, const int32_t *n, const int8_t *species) {
  return Guard([&] {
    Require(ctx && n && species && num_replicas > 0, LMC_ERR_INVALID_ARGUMENT, "bad argument");
    CudaCheck(cudaSetDevice(ctx->device), "cudaSetDevice");
    std::vector<int> nn(n, n + num_replicas);
    std::vector<long long> off(num_replicas);
    long long total = 0;
    for (int r = 0; r < num_replicas; ++r) {
      Require(nn[r] >= 6 && nn[r] <= 1000, LMC_ERR_UNSUPPORTED, "supercell edge must be in [6, 1000]");
      off[r] = total;
      total += 4LL * nn[r] * nn[r] * nn[r];
    }
    if (total + 64 > static_cast<long long>(ctx->species.bytes)) ctx->species.Alloc(total + 64);
    ctx->lat_off.Ensure(sizeof(long long) * num_replicas);
    ctx->lat_n.Ensure(sizeof(int) * num_replicas);
    ctx->scan.Ensure(sizeof(unsigned long long) * (lmc::kMaxSpecies + 1) * num_replicas);
    CudaCheck(cudaMemcpyAsync(ctx->species.p, species, total, cudaMemcpyHostToDevice, ctx->stream), "H2D species");
    CudaCheck(cudaMemcpyAsync(ctx->lat_off.p, off.data(), sizeof(long long) * num_replicas, cudaMemcpyHostToDevice,
                              ctx->stream),
              "H2D offsets");
    CudaCheck(cudaMemcpyAsync(ctx->lat_n.p, nn.data(), sizeof(int) * num_replicas, cudaMemcpyHostToDevice, ctx->stream),
              "H2D n");
    // species codes are validated on the device (the last histogram column counts bad codes)
    CudaCheck(cudaMemsetAsync(ctx->scan.p, 0, sizeof(unsigned long long) * (lmc::kMaxSpecies + 1) * num_replicas,
                              ctx->stream),
              "memset");
    ctx->scan_fresh = false;
    ctx->first_host.assign(num_replicas, std::numeric_limits<long long>::max());
    ctx->scan_first.Ensure(sizeof(long long) * num_replicas);
    CudaCheck(cudaMemcpyAsync(ctx->scan_first.p, ctx->first_host.data(), sizeof(long long) * num_replicas,
                              cudaMemcpyHostToDevice, ctx->stream),
              "H2D");
    CudaCheck(lmc::LaunchReplicaScan(ctx->species.as<int8_t>(), ctx->lat_off.as<long long>(), ctx->lat_n.as<int>(),
                                     num_replicas, ctx->fm.x_code, ctx->fm.num_species,
                                     ctx->scan_first.as<long long>(), ctx->scan.as<unsigned long long>(),
                                     ctx->stream),
              "scan kernel");
    ctx->scan_host.resize(static_cast<size_t>(lmc::kMaxSpecies + 1) * num_replicas);
    CudaCheck(cudaMemcpyAsync(ctx->scan_host.data(), ctx->scan.p, sizeof(unsigned long long) * ctx->scan_host.size(),
                              cudaMemcpyDeviceToHost, ctx->stream),
              "D2H");
    CudaCheck(cudaMemcpyAsync(ctx->first_host.data(), ctx->scan_first.p, sizeof(long long) * num_replicas,
                              cudaMemcpyDeviceToHost, ctx->stream),
              "D2H");
    ctx->Sync();
    for (int r = 0; r < num_replicas; ++r)
      Require(ctx->scan_host[static_cast<size_t>(r) * (lmc::kMaxSpecies + 1) + lmc::kMaxSpecies] == 0,
              LMC_ERR_OUT_OF_RANGE, "species code out of range in replica " + std::to_string(r));
    ctx->num_replicas = num_replicas;
    ctx->n = nn;
    ctx->offsets = off;
    ctx->total_sites = total;
    ctx->kmc_ready = false;
    ctx->scan_fresh = true;
  });
}

int lmc_ctx_get_lattices(lmc_ctx *ctx, int8_t *species) {
  return Guard([&] {
    Require(ctx && species && ctx->num_replicas > 0, LMC_ERR_INVALID_ARGUMENT, "no lattices");
    CudaCheck(cudaMemcpyAsync(species, ctx->species.p, ctx->total_sites, cudaMemcpyDeviceToHost, ctx->stream), "D2H");
    ctx->Sync();
  });
}

int64_t lmc_ctx_total_sites(const lmc_ctx *ctx) { return ctx ? ctx->total_sites : -1; }
int64_t lmc_ctx_replica_offset(const lmc_ctx *ctx, int replica) {
  if (!ctx || replica < 0 || replica >= ctx->num_replicas) return -1;
  return ctx->offsets[replica];
}
void *lmc_ctx_species_device_ptr(lmc_ctx *ctx) { return ctx ? ctx->species.p : nullptr; }

// Dominant species of replica r with a one-hot slot (the base of the sparse evaluation), from the
// histogram of the last lmc_ctx_set_lattices (the kernels conserve every replica's composition);
// -1 if none, or if it fills less than 7/8 of the lattice: a 135-site neighbourhood then holds
// more than about 17 other sites on average, and the dense sums are cheaper than the lists.
static int SparseBaseOf(const lmc_ctx *ctx, int replica) {
  if (ctx->scan_host.size() < static_cast<size_t>(replica + 1) * (lmc::kMaxSpecies + 1)) return -1;
  const unsigned long long *h = &ctx->scan_host[static_cast<size_t>(replica) * (lmc::kMaxSpecies + 1)];
  int base = -1;
  unsigned long long total = 0;
  for (int c = 0; c < ctx->fm.num_species; ++c) {
    total += h[c];
    if (c != ctx->fm.x_code && ctx->fm.onehot_rank[c] >= 0 && (base < 0 || h[c] > h[base])) base = c;
  }
  if (base < 0 || 8 * h[base] < 7 * total) return -1;
  return base;
}

// The barrier kernels of the batch entry points: the sparse evaluation for runs of pairs that
// share a vacancy (LMC_EVAL_SPARSE, the default) or the dense per-pair sums; identical results.
static void LaunchBarriers(lmc_ctx *ctx, int replica, int kind, const long long *d_pairs, int m, const int *m_dev,
                           double *d_ea, double *d_de, double *d_x, double *d_ks) {
  const int8_t *sp = ctx->species.as<int8_t>() + ctx->offsets[replica];
  // a device-side count (the surrogate's fallback list: few, scattered pairs) takes the dense sums
  const int base = ctx->barrier_eval == LMC_EVAL_SPARSE && !m_dev ? SparseBaseOf(ctx, replica) : -1;
  if (base >= 0) {
    BuildSparse(ctx, base);
    lmc::BarrierGroupArgs a{};
    a.n = ctx->n[replica];
    a.pairs = d_pairs;
    a.m = m;
    a.m_dev = m_dev;
    a.kind = kind;
    a.ea = d_ea;
    a.de = d_de;
    a.d_or_e0 = d_x;
    a.ks = d_ks;
    a.status = ctx->status.as<int>();
    a.sp = ctx->sparse;
    CudaCheck(lmc::LaunchBarrierGroup(ctx->t, sp, a, ctx->stream), "barrier kernel");
  } else if (m_dev) {
    CudaCheck(lmc::LaunchBarrierBatchCounted(ctx->t, sp, ctx->n[replica], d_pairs, m, m_dev, kind, d_ea, d_de,
                                             ctx->status.as<int>(), ctx->stream),
              "barrier kernel");
  } else {
    CudaCheck(lmc::LaunchBarrierBatch(ctx->t, sp, ctx->n[replica], d_pairs, m, kind, d_ea, d_de, d_x, d_ks,
                                      ctx->status.as<int>(), ctx->stream),
              "barrier kernel");
  }
}

static void BarrierBatchImpl(lmc_ctx *ctx, int replica, int kind, const long long *d_pairs, int m, double *d_ea,
                             double *d_de, double *d_x, double *d_ks) {
  ctx->CheckReplica(replica);
  Require(kind == LMC_BARRIER_QUARTIC || kind == LMC_BARRIER_E0, LMC_ERR_INVALID_ARGUMENT, "unknown barrier kind");
  ctx->ClearStatus();
  LaunchBarriers(ctx, replica, kind, d_pairs, m, nullptr, d_ea, d_de, d_x, d_ks);
}

int lmc_ctx_set_barrier_evaluation(lmc_ctx *ctx, int evaluation) {
  return Guard([&] {
    Require(ctx != nullptr, LMC_ERR_INVALID_ARGUMENT, "ctx is null");
    Require(evaluation == LMC_EVAL_SPARSE || evaluation == LMC_EVAL_DENSE, LMC_ERR_INVALID_ARGUMENT,
            "unknown evaluation");
    ctx->barrier_eval = evaluation;
  });
}

int lmc_barrier_batch(lmc_ctx *ctx, int replica, int kind, const int64_t *pairs, int m, double *ea, double *de,
                      double *d_or_e0, double *ks) {
  return Guard([&] {
    Require(ctx && pairs && ea && de && m >= 0, LMC_ERR_INVALID_ARGUMENT, "bad argument");
    if (m == 0) return;
    CudaCheck(cudaSetDevice(ctx->device), "cudaSetDevice");
    ctx->pairs.Ensure(sizeof(long long) * 2 * m);
    for (DevBuf *b : {&ctx->out0, &ctx->out1, &ctx->out2, &ctx->out3}) b->Ensure(sizeof(double) * m);
    CudaCheck(cudaMemcpyAsync(ctx->pairs.p, pairs, sizeof(long long) * 2 * m, cudaMemcpyHostToDevice, ctx->stream),
              "H2D pairs");
    BarrierBatchImpl(ctx, replica, kind, ctx->pairs.as<long long>(), m, ctx->out0.as<double>(), ctx->out1.as<double>(),
                     ctx->out2.as<double>(), ctx->out3.as<double>());
    CudaCheck(cudaMemcpyAsync(ea, ctx->out0.p, sizeof(double) * m, cudaMemcpyDeviceToHost, ctx->stream), "D2H");
    CudaCheck(cudaMemcpyAsync(de, ctx->out1.p, sizeof(double) * m, cudaMemcpyDeviceToHost, ctx->stream), "D2H");
    if (d_or_e0)
      CudaCheck(cudaMemcpyAsync(d_or_e0, ctx->out2.p, sizeof(double) * m, cudaMemcpyDeviceToHost, ctx->stream), "D2H");
    if (ks) CudaCheck(cudaMemcpyAsync(ks, ctx->out3.p, sizeof(double) * m, cudaMemcpyDeviceToHost, ctx->stream), "D2H");
    RaiseStatus(ctx->ReadStatus(), "barrier batch");
  });
}

int lmc_barrier_batch_device(lmc_ctx *ctx, int replica, int kind, const int64_t *pairs_dev, int m, double *ea_dev,
                             double *de_dev) {
  return Guard([&] {
    Require(ctx && pairs_dev && ea_dev && de_dev && m >= 0, LMC_ERR_INVALID_ARGUMENT, "bad argument");
    if (m == 0) return;
    BarrierBatchImpl(ctx, replica, kind, reinterpret_cast<const long long *>(pairs_dev), m, ea_dev, de_dev, nullptr,
                     nullptr);
  });
}

int lmc_encode_batch(lmc_ctx *ctx, int replica, const int64_t *pairs, int m, int32_t *state_start,
                     int32_t *state_end, int32_t *mmm, int32_t *mm2_fwd, int32_t *mm2_bwd) {
  return Guard([&] {
    Require(ctx && pairs && m > 0 && state_start && state_end && mmm && mm2_fwd && mm2_bwd, LMC_ERR_INVALID_ARGUMENT,
            "bad argument");
    ctx->CheckReplica(replica);
    const auto &t = ctx->t;
    const size_t per = 2 * t.num_theta + t.f_mmm + 2 * t.f_mm2;
    ctx->enc.Ensure(sizeof(int) * per * m);
    ctx->pairs.Ensure(sizeof(long long) * 2 * m);
    CudaCheck(cudaMemcpyAsync(ctx->pairs.p, pairs, sizeof(long long) * 2 * m, cudaMemcpyHostToDevice, ctx->stream),
              "H2D pairs");
    CudaCheck(cudaMemsetAsync(ctx->enc.p, 0, sizeof(int) * per * m, ctx->stream), "memset");
    int *base = ctx->enc.as<int>();
    int *cs = base, *ce = cs + static_cast<size_t>(t.num_theta) * m, *om = ce + static_cast<size_t>(t.num_theta) * m;
    int *of = om + static_cast<size_t>(t.f_mmm) * m, *ob = of + static_cast<size_t>(t.f_mm2) * m;
    ctx->ClearStatus();
    CudaCheck(lmc::LaunchEncodeBatch(t, ctx->species.as<int8_t>() + ctx->offsets[replica], ctx->n[replica],
                                     ctx->pairs.as<long long>(), m, cs, ce, om, of, ob, ctx->status.as<int>(),
                                     ctx->stream),
              "encode kernel");
    auto d2h = [&](int32_t *dst, int *src, size_t cnt) {
      CudaCheck(cudaMemcpyAsync(dst, src, sizeof(int) * cnt, cudaMemcpyDeviceToHost, ctx->stream), "D2H");
    };
    d2h(state_start, cs, static_cast<size_t>(t.num_theta) * m);
    d2h(state_end, ce, static_cast<size_t>(t.num_theta) * m);
    d2h(mmm, om, static_cast<size_t>(t.f_mmm) * m);
    d2h(mm2_fwd, of, static_cast<size_t>(t.f_mm2) * m);
    d2h(mm2_bwd, ob, static_cast<size_t>(t.f_mm2) * m);
    RaiseStatus(ctx->ReadStatus(), "encode batch");
  });
}

int lmc_de_pairs(lmc_ctx *ctx, int replica, const int64_t *pairs, int m, double *de) {
  return Guard([&] {
    Require(ctx && pairs && de && m >= 0, LMC_ERR_INVALID_ARGUMENT, "bad argument");
    if (m == 0) return;
    ctx->CheckReplica(replica);
    ctx->pairs.Ensure(sizeof(long long) * 2 * m);
    ctx->out0.Ensure(sizeof(double) * m);
    CudaCheck(cudaMemcpyAsync(ctx->pairs.p, pairs, sizeof(long long) * 2 * m, cudaMemcpyHostToDevice, ctx->stream),
              "H2D pairs");
    ctx->ClearStatus();
    CudaCheck(lmc::LaunchDePairs(ctx->t, ctx->species.as<int8_t>() + ctx->offsets[replica], ctx->n[replica],
                                 ctx->pairs.as<long long>(), m, ctx->out0.as<double>(), ctx->status.as<int>(),
                                 ctx->stream),
              "dE kernel");
    CudaCheck(cudaMemcpyAsync(de, ctx->out0.p, sizeof(double) * m, cudaMemcpyDeviceToHost, ctx->stream), "D2H");
    RaiseStatus(ctx->ReadStatus(), "pair dE");
  });
}

int lmc_energy(lmc_ctx *ctx, int replica, double *energy, int64_t *counts) {
  return Guard([&] {
    Require(ctx && energy, LMC_ERR_INVALID_ARGUMENT, "bad argument");
    ctx->CheckReplica(replica);
    // dominant species of the lattice: the solvent for dilute alloys
    int base = 0;
    {
      const auto &fm = ctx->fm;
      base = fm.x_code == 0 ? 1 : 0;
      for (int c = 0; c < fm.num_species; ++c)
        if (ctx->model.alphabet[c] == "Al") base = c;
    }
    CudaCheck(lmc::LaunchCensus(ctx->t, ctx->species.as<int8_t>() + ctx->offsets[replica], ctx->n[replica], base,
                                ctx->counts.as<unsigned long long>(), ctx->energy.as<double>(), ctx->stream),
              "census kernel");
    CudaCheck(cudaMemcpyAsync(energy, ctx->energy.p, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream), "D2H");
    if (counts)
      CudaCheck(cudaMemcpyAsync(counts, ctx->counts.p, sizeof(int64_t) * ctx->t.num_theta, cudaMemcpyDeviceToHost,
                                ctx->stream),
                "D2H");
    ctx->Sync();
  });
}

int lmc_energy_noalloc(lmc_ctx *ctx, const int8_t *species_dev, int n, double *energy_dev) {
  return Guard([&] {
    Require(ctx && species_dev && energy_dev, LMC_ERR_INVALID_ARGUMENT, "null argument");
    Require(n >= 6 && n <= 1000, LMC_ERR_UNSUPPORTED, "supercell edge must be in [6, 1000]");
    Require(ctx->t.num_theta <= lmc::kNoAllocMaxTheta, LMC_ERR_UNSUPPORTED,
            "lmc_energy_noalloc: the model's " + std::to_string(ctx->t.num_theta) +
                " cluster counters exceed the " + std::to_string(lmc::kNoAllocMaxTheta) +
                "-entry static scratch");
    CudaCheck(cudaSetDevice(ctx->device), "cudaSetDevice");
    unsigned long long *scratch = nullptr;
    CudaCheck(lmc::NoAllocCensusScratch(ctx->device, &scratch), "cudaGetSymbolAddress");
    int base = ctx->fm.x_code == 0 ? 1 : 0;
    for (int c = 0; c < ctx->fm.num_species; ++c)
      if (ctx->model.alphabet[c] == "Al") base = c;
    // clears the scratch, range-checks every species code on the device (NaN energy on a bad one)
    CudaCheck(lmc::LaunchCensusCheckedNoAlloc(ctx->t, species_dev, n, base, scratch, energy_dev, ctx->stream),
              "census kernel");
  });
}

namespace {
int SurrogateBase(const lmc_ctx *ctx) {
  const int al = ctx->model.Code("Al");
  if (al >= 0 && al != ctx->fm.x_code) return al;
  for (int c = 0; c < ctx->fm.num_species; ++c)
    if (c != ctx->fm.x_code && ctx->fm.onehot_rank[c] >= 0) return c;
  return -1;
}

// Channels of a site for the context's feature encoding: the one-hot rank, or (solute
// channels) the ranks other than the base species' in their order.
lmc::FeatEnc FeatEncOf(const lmc_ctx *ctx) {
  const int eh = ctx->fm.num_onehot;
  lmc::FeatEnc f{~0ull, eh};
  const int base = SurrogateBase(ctx);
  const int rb = (ctx->feat_encoding == LMC_FEATURES_SOLUTE && base >= 0) ? ctx->fm.onehot_rank[base] : -1;
  if (rb >= 0) f.width = eh - 1;
  for (int r = 0; r < eh && r < lmc::kMaxOnehot - 1; ++r) {
    const int ch = rb < 0 ? r : (r == rb ? -1 : (r < rb ? r : r - 1));
    if (ch >= 0) {
      f.rank_ch &= ~(0xFFull << (8 * r));
      f.rank_ch |= static_cast<unsigned long long>(ch) << (8 * r);
    }
  }
  return f;
}

int FeatureCount(const lmc_ctx *ctx) { return (lmc::kEnvSites + 1) * FeatEncOf(ctx).width; }

// The fused jump kernel's description of the replica's lattice and the encoding (solute
// channels of a three- or four-species alphabet: two or three channels per site).
bool FusedJumpsFor(const lmc_ctx *ctx, int replica, const long long *pairs, long long m, float *mean, float *spread,
                   lmc::FusedJumps *j) {
  const lmc::FeatEnc f = FeatEncOf(ctx);
  if (ctx->feat_encoding != LMC_FEATURES_SOLUTE || (f.width != 2 && f.width != 3)) return false;
  *j = lmc::FusedJumps{};
  j->channels = f.width;
  j->species = ctx->species.as<int8_t>() + ctx->offsets[replica];
  j->n = ctx->n[replica];
  j->pairs = pairs;
  j->m = m;
  j->mmm_off = ctx->t.mmm_off;
  j->dir_of = ctx->t.dir_of;
  for (int c = 0; c < 8; ++c) {
    const int rank = c < ctx->fm.num_species ? ctx->fm.onehot_rank[c] : -1;
    const int ch = rank >= 0 ? lmc::FeatChannel(f, rank) : -1;
    j->site_word[c] = ch == 0 ? 0x3F80u : (ch == 1 ? 0x3F800000u : 0u);  // bf16 1.0 in the low / high half
    j->chan[c] = static_cast<int8_t>(ch);
    if (rank < 0) j->fallback_codes |= 1u << c;
  }
  j->mean = mean;
  j->spread = spread;
  j->pair_status = ctx->status.as<int>();
  return true;
}
}  // namespace

int lmc_surrogate_set_encoding(lmc_ctx *ctx, int encoding) {
  return Guard([&] {
    Require(ctx != nullptr, LMC_ERR_INVALID_ARGUMENT, "ctx is null");
    Require(encoding == LMC_FEATURES_ONEHOT || encoding == LMC_FEATURES_SOLUTE, LMC_ERR_INVALID_ARGUMENT,
            "unknown feature encoding");
    Require(encoding == LMC_FEATURES_ONEHOT || SurrogateBase(ctx) >= 0, LMC_ERR_INVALID_ARGUMENT,
            "no base species with a one-hot slot");
    ctx->feat_encoding = encoding;
  });
}

int lmc_surrogate_feature_count(const lmc_ctx *ctx, int *min_features, int *padded_features) {
  return Guard([&] {
    Require(ctx != nullptr, LMC_ERR_INVALID_ARGUMENT, "ctx is null");
    const int need = FeatureCount(ctx);
    if (min_features) *min_features = need;
    if (padded_features) *padded_features = (need + 63) / 64 * 64;
  });
}

int lmc_surrogate_dataset(lmc_ctx *ctx, uint64_t seed, int64_t count, double solute_lo, double solute_hi, int kind,
                          int in_features, uint16_t *features_dev, float *ea_dev, double *ea64_dev, double *de64_dev) {
  return Guard([&] {
    Require(ctx && features_dev && ea_dev, LMC_ERR_INVALID_ARGUMENT, "null argument");
    Require(count >= 0, LMC_ERR_INVALID_ARGUMENT, "count < 0");
    Require(0.0 <= solute_lo && solute_lo <= solute_hi && solute_hi <= 1.0, LMC_ERR_INVALID_ARGUMENT,
            "need 0 <= solute_lo <= solute_hi <= 1");
    Require(kind == LMC_BARRIER_QUARTIC || kind == LMC_BARRIER_E0, LMC_ERR_INVALID_ARGUMENT, "unknown barrier kind");
    Require(in_features >= FeatureCount(ctx), LMC_ERR_INVALID_ARGUMENT, "in_features below 59 x the site channels");
    CudaCheck(cudaSetDevice(ctx->device), "cudaSetDevice");
    lmc::SurrogateGen g{};
    g.enc = FeatEncOf(ctx);
    g.seed = seed;
    g.count = count;
    g.solute_lo = static_cast<float>(solute_lo);
    g.solute_hi = static_cast<float>(solute_hi);
    g.base_code = SurrogateBase(ctx);
    Require(g.base_code >= 0, LMC_ERR_INVALID_ARGUMENT, "no base species with a one-hot slot");
    g.kind = kind;
    g.in_pad = in_features;
    g.features = reinterpret_cast<__nv_bfloat16 *>(features_dev);
    g.ea = ea_dev;
    g.ea64 = ea64_dev;
    g.de64 = de64_dev;
    g.status = ctx->status.as<int>();
    ctx->ClearStatus();
    CudaCheck(lmc::LaunchSurrogateDataset(ctx->t, g, ctx->stream), "dataset kernel");
    RaiseStatus(ctx->ReadStatus(), "surrogate dataset");
  });
}

int lmc_surrogate_features(lmc_ctx *ctx, int replica, const int64_t *pairs_dev, int m, int in_features,
                           uint16_t *features_dev) {
  return Guard([&] {
    Require(ctx && pairs_dev && features_dev, LMC_ERR_INVALID_ARGUMENT, "null argument");
    ctx->CheckReplica(replica);
    Require(in_features >= FeatureCount(ctx), LMC_ERR_INVALID_ARGUMENT, "in_features below 59 x the site channels");
    CudaCheck(cudaSetDevice(ctx->device), "cudaSetDevice");
    ctx->ClearStatus();
    CudaCheck(lmc::LaunchSurrogateFeatures(ctx->t, ctx->species.as<int8_t>() + ctx->offsets[replica], ctx->n[replica],
                                           reinterpret_cast<const long long *>(pairs_dev), m, in_features,
                                           FeatEncOf(ctx), reinterpret_cast<__nv_bfloat16 *>(features_dev),
                                           ctx->status.as<int>(), ctx->stream),
              "features kernel");
    RaiseStatus(ctx->ReadStatus(), "surrogate features");
  });
}

namespace {
// The ensemble's mean and spread for m lattice jumps (device arrays) on the context stream:
// the fused jump kernel where the network and the encoding allow it (features gathered
// inside), else the feature kernel and then the feature-row inference (tcgen05 kernel on the
// context stream, or the mma.sync GEMMs on the network's stream, synchronised).
void NetworkOnJumps(lmc_ctx *ctx, lmc_mlp *mlp, int replica, const long long *pairs, int m, float *mean,
                    float *spread) {
  const int in = lmc::MlpInputs(mlp);
  Require(in >= FeatureCount(ctx), LMC_ERR_INVALID_ARGUMENT,
          "the network's input is narrower than the features of this model and encoding");
  lmc::FusedJumps j;
  if (FusedJumpsFor(ctx, replica, pairs, m, mean, spread, &j) && lmc::MlpFusedJumpsAsync(mlp, j, ctx->stream))
    return;
  ctx->s_feat.Ensure(sizeof(uint16_t) * static_cast<size_t>(m) * in);
  CudaCheck(lmc::LaunchSurrogateFeatures(ctx->t, ctx->species.as<int8_t>() + ctx->offsets[replica], ctx->n[replica],
                                         pairs, m, in, FeatEncOf(ctx), ctx->s_feat.as<__nv_bfloat16>(),
                                         ctx->status.as<int>(), ctx->stream),
            "features kernel");
  if (!lmc::MlpPredictAsync(mlp, ctx->s_feat.as<uint16_t>(), m, mean, spread, ctx->stream)) {
    ctx->Sync();
    const int st = lmc_mlp_predict(mlp, ctx->s_feat.as<uint16_t>(), m, mean, spread);
    if (st != LMC_OK) throw LmcError(st, lmc_last_error());
  }
}
}  // namespace

int lmc_surrogate_predict_device(lmc_ctx *ctx, lmc_mlp *mlp, int replica, const int64_t *pairs_dev, int m,
                                 float *mean_dev, float *spread_dev) {
  return Guard([&] {
    Require(ctx && mlp && pairs_dev && mean_dev && spread_dev, LMC_ERR_INVALID_ARGUMENT, "null argument");
    Require(m >= 0, LMC_ERR_INVALID_ARGUMENT, "m < 0");
    ctx->CheckReplica(replica);
    CudaCheck(cudaSetDevice(ctx->device), "cudaSetDevice");
    if (m == 0) return;
    ctx->ClearStatus();
    NetworkOnJumps(ctx, mlp, replica, reinterpret_cast<const long long *>(pairs_dev), m, mean_dev, spread_dev);
    int *h = ctx->Pinned();
    CudaCheck(cudaMemcpyAsync(h, lmc::MlpStatusDev(mlp), sizeof(int), cudaMemcpyDeviceToHost, ctx->stream), "D2H");
    CudaCheck(cudaMemcpyAsync(h + 1, ctx->status.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream), "D2H");
    ctx->Sync();
    const int net_status = h[0], st = h[1];
    Require(net_status == 0, LMC_ERR_STOPPED, "surrogate inference: a tensor-core wait expired");
    RaiseStatus(st, "surrogate network");
  });
}

int lmc_surrogate_barrier_batch_device(lmc_ctx *ctx, lmc_mlp *mlp, int replica, int kind, const int64_t *pairs_dev,
                                       int m, float threshold_ev, double *ea_dev, uint8_t *fallback_dev,
                                       int *num_fallback) {
  return Guard([&] {
    Require(ctx && mlp && pairs_dev && ea_dev, LMC_ERR_INVALID_ARGUMENT, "null argument");
    Require(m >= 0, LMC_ERR_INVALID_ARGUMENT, "m < 0");
    ctx->CheckReplica(replica);
    CudaCheck(cudaSetDevice(ctx->device), "cudaSetDevice");
    if (m == 0) {
      if (num_fallback) *num_fallback = 0;
      return;
    }
    const size_t mm = static_cast<size_t>(m);
    ctx->s_mean.Ensure(sizeof(float) * mm);
    ctx->s_spread.Ensure(sizeof(float) * mm);
    ctx->s_fb_pairs.Ensure(sizeof(long long) * 2 * mm);
    ctx->s_fb_index.Ensure(sizeof(int) * (mm + 1));
    ctx->s_fb_ea.Ensure(sizeof(double) * mm);
    ctx->s_fb_de.Ensure(sizeof(double) * mm);
    const auto *pairs = reinterpret_cast<const long long *>(pairs_dev);
    ctx->ClearStatus();
    NetworkOnJumps(ctx, mlp, replica, pairs, m, ctx->s_mean.as<float>(), ctx->s_spread.as<float>());
    int *d_count = ctx->s_fb_index.as<int>() + mm;
    CudaCheck(cudaMemsetAsync(d_count, 0, sizeof(int), ctx->stream), "memset");
    CudaCheck(lmc::LaunchFallbackCompact(pairs, ctx->s_mean.as<float>(), ctx->s_spread.as<float>(), m, threshold_ev,
                                         ctx->s_fb_pairs.as<long long>(), ctx->s_fb_index.as<int>(), d_count,
                                         fallback_dev, ctx->stream),
              "fallback kernel");
    // the plain predictor on the compacted pairs, sized by the device count (no host round trip)
    LaunchBarriers(ctx, replica, kind, ctx->s_fb_pairs.as<long long>(), m, d_count, ctx->s_fb_ea.as<double>(),
                   ctx->s_fb_de.as<double>(), nullptr, nullptr);
    CudaCheck(lmc::LaunchFallbackMerge(ctx->s_mean.as<float>(), m, ctx->s_fb_ea.as<double>(), ctx->s_fb_index.as<int>(),
                                       d_count, ea_dev, ctx->stream),
              "merge kernel");
    // one host round trip: fallback count, network status and kernel status into pinned words
    int *h = ctx->Pinned();
    CudaCheck(cudaMemcpyAsync(h, d_count, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream), "D2H");
    CudaCheck(cudaMemcpyAsync(h + 1, lmc::MlpStatusDev(mlp), sizeof(int), cudaMemcpyDeviceToHost, ctx->stream), "D2H");
    CudaCheck(cudaMemcpyAsync(h + 2, ctx->status.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream), "D2H");
    ctx->Sync();
    const int count = h[0], net_status = h[1], st = h[2];
    Require(net_status == 0, LMC_ERR_STOPPED, "surrogate inference: a tensor-core wait expired");
    RaiseStatus(st, "surrogate barriers");
    if (num_fallback) *num_fallback = count;
  });
}

int lmc_fastmath_check(lmc_ctx *ctx, int fn, const double *x, int64_t n, double *fast, double *ref) {
  return Guard([&] {
    Require(ctx && x && fast && ref && n >= 0, LMC_ERR_INVALID_ARGUMENT, "bad argument");
    Require(fn == 0 || fn == 1, LMC_ERR_INVALID_ARGUMENT, "fn must be 0 (exp) or 1 (reciprocal)");
    CudaCheck(cudaSetDevice(ctx->device), "cudaSetDevice");
    const size_t bytes = sizeof(double) * static_cast<size_t>(n);
    DevBuf dx, df, dr;
    dx.Alloc(bytes);
    df.Alloc(bytes);
    dr.Alloc(bytes);
    CudaCheck(cudaMemcpyAsync(dx.p, x, bytes, cudaMemcpyHostToDevice, ctx->stream), "H2D");
    CudaCheck(lmc::LaunchFastmathCheck(ctx->t, fn, dx.as<double>(), n, df.as<double>(), dr.as<double>(), ctx->stream),
              "fastmath kernel");
    CudaCheck(cudaMemcpyAsync(fast, df.p, bytes, cudaMemcpyDeviceToHost, ctx->stream), "D2H");
    CudaCheck(cudaMemcpyAsync(ref, dr.p, bytes, cudaMemcpyDeviceToHost, ctx->stream), "D2H");
    CudaCheck(cudaStreamSynchronize(ctx->stream), "sync");
    dx.Free();
    df.Free();
    dr.Free();
  });
}

int lmc_kmc_init(lmc_ctx *ctx, const double *temperature, const lmc_kmc_options *opt) {
  return Guard([&] {
    Require(ctx && temperature && opt && ctx->num_replicas > 0, LMC_ERR_INVALID_ARGUMENT, "bad argument");
    Require(opt->rng == LMC_RNG_MT19937_64 || opt->rng == LMC_RNG_PHILOX, LMC_ERR_INVALID_ARGUMENT, "unknown rng");
    Require(opt->barrier_kind == LMC_BARRIER_QUARTIC || opt->barrier_kind == LMC_BARRIER_E0, LMC_ERR_INVALID_ARGUMENT,
            "unknown barrier kind");
    Require(opt->rates == LMC_RATES_FP32 || opt->rates == LMC_RATES_FP64, LMC_ERR_INVALID_ARGUMENT,
            "unknown rate precision");
    CudaCheck(cudaSetDevice(ctx->device), "cudaSetDevice");
    const int R = ctx->num_replicas;
    for (int r = 0; r < R; ++r)
      Require(temperature[r] > 0 && std::isfinite(temperature[r]), LMC_ERR_INVALID_ARGUMENT, "temperature must be > 0");
    ctx->kmc_opt = *opt;
    ctx->k_vac.Ensure(sizeof(long long) * R);
    ctx->k_steps.Ensure(sizeof(unsigned long long) * R);
    ctx->k_time.Ensure(sizeof(double) * R);
    ctx->k_energy.Ensure(sizeof(double) * R);
    ctx->k_temp.Ensure(sizeof(double) * R);
    ctx->k_cvac.Ensure(sizeof(double) * R);
    ctx->k_csol.Ensure(sizeof(double) * R);
    ctx->k_rng.Ensure(sizeof(uint32_t) * lmc::kRngWords * R);
    Require(!(opt->chain && opt->early_stop), LMC_ERR_UNSUPPORTED, "the chain KMC has no early stop");
    ctx->k_solvent.Ensure(R);
    ctx->k_escaped.Ensure(R);
    ctx->k_prev.Ensure(sizeof(long long) * R);
    CudaCheck(cudaMemsetAsync(ctx->k_escaped.p, 0, R, ctx->stream), "memset");
    // first vacancy and species histogram of every replica: from set_lattices' scan while no
    // kernel has moved atoms since, else scanned again
    std::vector<long long> first;
    std::vector<unsigned long long> h;
    if (ctx->scan_fresh) {
      first = ctx->first_host;
      h = ctx->scan_host;
      CudaCheck(cudaMemcpyAsync(ctx->k_vac.p, first.data(), sizeof(long long) * R, cudaMemcpyHostToDevice, ctx->stream),
                "H2D");
    } else {
      DevBuf hist;
      hist.Alloc(sizeof(unsigned long long) * (lmc::kMaxSpecies + 1) * R);
      first.assign(R, std::numeric_limits<long long>::max());
      CudaCheck(cudaMemcpyAsync(ctx->k_vac.p, first.data(), sizeof(long long) * R, cudaMemcpyHostToDevice,
                                ctx->stream),
                "H2D");
      CudaCheck(cudaMemsetAsync(hist.p, 0, hist.bytes, ctx->stream), "memset");
      CudaCheck(lmc::LaunchReplicaScan(ctx->species.as<int8_t>(), ctx->lat_off.as<long long>(), ctx->lat_n.as<int>(),
                                       R, ctx->fm.x_code, ctx->fm.num_species, ctx->k_vac.as<long long>(),
                                       hist.as<unsigned long long>(), ctx->stream),
                "scan kernel");
      h.resize((lmc::kMaxSpecies + 1) * R);
      CudaCheck(cudaMemcpyAsync(first.data(), ctx->k_vac.p, sizeof(long long) * R, cudaMemcpyDeviceToHost,
                                ctx->stream),
                "D2H");
      CudaCheck(cudaMemcpyAsync(h.data(), hist.p, hist.bytes, cudaMemcpyDeviceToHost, ctx->stream), "D2H");
      ctx->Sync();
      hist.Free();
    }
    for (int r = 0; r < R; ++r)
      Require(first[r] != std::numeric_limits<long long>::max(), LMC_ERR_INVALID_ARGUMENT, "vacancy not found");
    if (opt->chain) {
      // previous_j_lattice_id_ of the chain KMC: the first (lowest-id) 1NN of the initial vacancy
      // (KineticMcAbstract.cpp:255)
      std::vector<long long> prev(R);
      for (int r = 0; r < R; ++r) prev[r] = lmc::SortedNeighbors(lmc::Fcc{ctx->n[r]}, first[r], 1).front();
      CudaCheck(cudaMemcpyAsync(ctx->k_prev.p, prev.data(), 8 * R, cudaMemcpyHostToDevice, ctx->stream), "H2D");
      ctx->Sync();
    }
    // dominant species with a one-hot slot: the base of the sparse evaluation
    {
      std::vector<unsigned long long> tot(ctx->fm.num_species, 0);
      for (int r = 0; r < R; ++r)
        for (int c = 0; c < ctx->fm.num_species; ++c) tot[c] += h[r * (lmc::kMaxSpecies + 1) + c];
      int base = -1;
      for (int c = 0; c < ctx->fm.num_species; ++c)
        if (c != ctx->fm.x_code && ctx->fm.onehot_rank[c] >= 0 && (base < 0 || tot[c] > tot[base])) base = c;
      Require(base >= 0, LMC_ERR_INVALID_ARGUMENT, "no element of the barrier set in the lattices");
      BuildSparse(ctx, base);
    }
    {
      // Config::GetSolventElement (Config.cpp:411-422): most frequent species per replica
      std::vector<int8_t> solvent(R, 0);
      for (int r = 0; r < R; ++r)
        for (int c = 1; c < ctx->fm.num_species; ++c)
          if (h[r * (lmc::kMaxSpecies + 1) + c] > h[r * (lmc::kMaxSpecies + 1) + solvent[r]])
            solvent[r] = static_cast<int8_t>(c);
      CudaCheck(cudaMemcpyAsync(ctx->k_solvent.p, solvent.data(), R, cudaMemcpyHostToDevice, ctx->stream), "H2D");
      ctx->Sync();
    }
    const int al = ctx->model.Code("Al");
    std::vector<double> cvac(R, -1.0), csol(R, 0.0);
    if (opt->rate_corrector) {
      for (int r = 0; r < R; ++r) {
        const double nsites = 4.0 * ctx->n[r] * ctx->n[r] * ctx->n[r];
        unsigned long long sol = 0;
        for (int c = 0; c < ctx->fm.num_species; ++c)
          if (c != ctx->fm.x_code && c != al) sol += h[r * (lmc::kMaxSpecies + 1) + c];
        cvac[r] = static_cast<double>(h[r * (lmc::kMaxSpecies + 1) + ctx->fm.x_code]) / nsites;
        csol[r] = static_cast<double>(sol) / nsites;
      }
    }
    std::vector<uint32_t> rng;
    if (opt->rng == LMC_RNG_MT19937_64) {
      rng.assign(static_cast<size_t>(lmc::kRngWords) * R, 0);
      for (int r = 0; r < R; ++r)
        lmc::MtSeed(opt->seed + static_cast<uint64_t>(r), rng.data() + static_cast<size_t>(lmc::kRngWords) * r);
    } else {
      rng.resize(2 * static_cast<size_t>(R));  // Philox: the key words only
      for (int r = 0; r < R; ++r) {
        rng[2 * r] = static_cast<uint32_t>(opt->seed);
        rng[2 * r + 1] = static_cast<uint32_t>(opt->seed >> 32);
      }
    }
    std::vector<unsigned long long> zeros_u(R, 0);
    std::vector<double> zeros_d(R, 0.0), temp(temperature, temperature + R);
    CudaCheck(cudaMemcpyAsync(ctx->k_steps.p, zeros_u.data(), 8 * R, cudaMemcpyHostToDevice, ctx->stream), "H2D");
    CudaCheck(cudaMemcpyAsync(ctx->k_time.p, zeros_d.data(), 8 * R, cudaMemcpyHostToDevice, ctx->stream), "H2D");
    CudaCheck(cudaMemcpyAsync(ctx->k_energy.p, zeros_d.data(), 8 * R, cudaMemcpyHostToDevice, ctx->stream), "H2D");
    CudaCheck(cudaMemcpyAsync(ctx->k_temp.p, temp.data(), 8 * R, cudaMemcpyHostToDevice, ctx->stream), "H2D");
    CudaCheck(cudaMemcpyAsync(ctx->k_cvac.p, cvac.data(), 8 * R, cudaMemcpyHostToDevice, ctx->stream), "H2D");
    CudaCheck(cudaMemcpyAsync(ctx->k_csol.p, csol.data(), 8 * R, cudaMemcpyHostToDevice, ctx->stream), "H2D");
    if (opt->rng == LMC_RNG_MT19937_64)
      CudaCheck(cudaMemcpyAsync(ctx->k_rng.p, rng.data(), rng.size() * 4, cudaMemcpyHostToDevice, ctx->stream), "H2D");
    else  // two words at the start of each replica's record
      CudaCheck(cudaMemcpy2DAsync(ctx->k_rng.p, sizeof(uint32_t) * lmc::kRngWords, rng.data(), 8, 8, R,
                                  cudaMemcpyHostToDevice, ctx->stream),
                "H2D keys");
    ctx->tt_len = 0;
    if (opt->tt_len > 0) {
      Require(opt->tt_time && opt->tt_temp, LMC_ERR_INVALID_ARGUMENT, "T(t) table pointers are null");
      std::vector<std::pair<double, double>> pts;
      for (int i = 0; i < opt->tt_len; ++i) pts.emplace_back(opt->tt_time[i], opt->tt_temp[i]);
      std::sort(pts.begin(), pts.end());
      for (size_t i = 1; i < pts.size(); ++i)
        Require(std::abs(pts[i].first - pts[i - 1].first) >= 1e-12, LMC_ERR_INVALID_ARGUMENT,
                "2 adjacent x values are equal.");
      std::vector<double> tt, tv;
      for (auto &p : pts) {
        tt.push_back(p.first);
        tv.push_back(p.second);
      }
      ctx->k_tt_time.Ensure(8 * tt.size());
      ctx->k_tt_temp.Ensure(8 * tv.size());
      CudaCheck(cudaMemcpyAsync(ctx->k_tt_time.p, tt.data(), 8 * tt.size(), cudaMemcpyHostToDevice, ctx->stream), "H2D");
      CudaCheck(cudaMemcpyAsync(ctx->k_tt_temp.p, tv.data(), 8 * tv.size(), cudaMemcpyHostToDevice, ctx->stream), "H2D");
      ctx->tt_len = opt->tt_len;
    }
    ctx->Sync();
    ctx->kmc_ready = true;
  });
}

int lmc_kmc_launch_info(lmc_ctx *ctx, int *warps_per_replica, int *replicas_per_block, int *blocks_per_sm,
                        int64_t *shared_bytes) {
  return Guard([&] {
    Require(ctx && ctx->kmc_ready, LMC_ERR_INVALID_ARGUMENT, "lmc_kmc_init has not been called");
    CudaCheck(cudaSetDevice(ctx->device), "cudaSetDevice");
    const lmc::KmcLaunch l = KmcShape(ctx);
    int per_sm = 0;
    size_t bytes = 0;
    CudaCheck(lmc::KmcOccupancy(ctx->t, l, &per_sm, &bytes), "KMC occupancy");
    if (warps_per_replica) *warps_per_replica = l.warps_per_replica;
    if (replicas_per_block) *replicas_per_block = l.replicas_per_block;
    if (blocks_per_sm) *blocks_per_sm = per_sm;
    if (shared_bytes) *shared_bytes = static_cast<int64_t>(bytes);
  });
}

int lmc_kmc_run(lmc_ctx *ctx, uint64_t steps, int trace_replica, lmc_kmc_step *trace, double *events12) {
  return Guard([&] {
    if (ctx) ctx->scan_fresh = false;  // atoms move
    Require(ctx && ctx->kmc_ready, LMC_ERR_INVALID_ARGUMENT, "lmc_kmc_init has not been called");
    CudaCheck(cudaSetDevice(ctx->device), "cudaSetDevice");
    if (steps == 0) return;
    static_assert(sizeof(lmc_kmc_step) == sizeof(lmc::KmcTraceRec), "trace record layout");
    const lmc::KmcDevState s = KmcState(ctx);
    lmc::KmcLaunch l = KmcShape(ctx);
    l.steps = steps;
    l.trace_replica = -1;
    if (trace || events12) {
      ctx->CheckReplica(trace_replica);
      l.trace_replica = trace_replica;
      if (trace) {
        ctx->k_trace.Ensure(sizeof(lmc::KmcTraceRec) * steps);
        l.trace = ctx->k_trace.as<lmc::KmcTraceRec>();
      }
      if (events12) {
        ctx->k_events.Ensure(sizeof(double) * 36 * steps);
        l.events12 = ctx->k_events.as<double>();
      }
    }
    l.stop_flag = ctx->d_stop;
    l.status = ctx->status.as<int>();
    ctx->ClearStatus();
    Require(!(ctx->kmc_opt.chain && events12), LMC_ERR_UNSUPPORTED, "the chain KMC has no events12 output");
    CudaCheck(cudaEventRecord(ctx->ev0, ctx->stream), "event");
    if (ctx->kmc_opt.chain)
      CudaCheck(lmc::LaunchKmcChain(ctx->t, ctx->species.as<int8_t>(), s, l, ctx->stream), "chain KMC kernel");
    else
      CudaCheck(lmc::LaunchKmc(ctx->t, ctx->species.as<int8_t>(), s, l, ctx->stream), "KMC kernel");
    CudaCheck(cudaEventRecord(ctx->ev1, ctx->stream), "event");
    if (trace)
      CudaCheck(cudaMemcpyAsync(trace, l.trace, sizeof(lmc::KmcTraceRec) * steps, cudaMemcpyDeviceToHost, ctx->stream),
                "D2H trace");
    if (events12)
      CudaCheck(cudaMemcpyAsync(events12, l.events12, sizeof(double) * 36 * steps, cudaMemcpyDeviceToHost, ctx->stream),
                "D2H events");
    const int st = ctx->ReadStatus();
    float ms = 0;
    CudaCheck(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1), "elapsed");
    ctx->last_ms = ms;
    RaiseStatus(st, "KMC run");
  });
}

int lmc_kmc_run_graph(lmc_ctx *ctx, uint64_t steps_per_launch, int launches) {
  return Guard([&] {
    if (ctx) ctx->scan_fresh = false;  // atoms move
    Require(ctx && ctx->kmc_ready, LMC_ERR_INVALID_ARGUMENT, "lmc_kmc_init has not been called");
    Require(steps_per_launch > 0 && launches > 0, LMC_ERR_INVALID_ARGUMENT, "steps_per_launch and launches must be > 0");
    Require(!ctx->kmc_opt.chain, LMC_ERR_UNSUPPORTED, "graph runs cover the first-order KMC");
    CudaCheck(cudaSetDevice(ctx->device), "cudaSetDevice");
    const lmc::KmcDevState s = KmcState(ctx);
    lmc::KmcLaunch l = KmcShape(ctx);
    l.steps = steps_per_launch;
    l.trace_replica = -1;
    l.stop_flag = ctx->d_stop;
    l.status = ctx->status.as<int>();
    int8_t *species = ctx->species.as<int8_t>();
    // every byte the recorded launches depend on: a change re-records the graph
    std::vector<unsigned char> key(sizeof(ctx->t) + sizeof(s) + sizeof(l) + sizeof(species) + sizeof(launches));
    {
      unsigned char *k = key.data();
      std::memcpy(k, &ctx->t, sizeof(ctx->t));
      k += sizeof(ctx->t);
      std::memcpy(k, &s, sizeof(s));
      k += sizeof(s);
      std::memcpy(k, &l, sizeof(l));
      k += sizeof(l);
      std::memcpy(k, &species, sizeof(species));
      k += sizeof(species);
      std::memcpy(k, &launches, sizeof(launches));
    }
    ctx->Pinned();
    if (!ctx->kmc_graph || key != ctx->kmc_graph_key) {
      if (ctx->kmc_graph) CudaCheck(cudaGraphExecDestroy(ctx->kmc_graph), "cudaGraphExecDestroy");
      ctx->kmc_graph = nullptr;
      ctx->kmc_graph_key.clear();
      int per_sm = 0;
      size_t bytes = 0;
      CudaCheck(lmc::KmcOccupancy(ctx->t, l, &per_sm, &bytes), "KMC occupancy");  // sets the smem attribute
      Require(per_sm >= 1, LMC_ERR_INVALID_ARGUMENT, "KMC launch shape does not fit on an SM");
      CudaCheck(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
      cudaError_t err = cudaMemsetAsync(l.status, 0, sizeof(int), ctx->stream);
      for (int i = 0; i < launches && err == cudaSuccess; ++i)
        err = lmc::LaunchKmc(ctx->t, species, s, l, ctx->stream, /*prepare=*/false);
      if (err == cudaSuccess)
        err = cudaMemcpyAsync(ctx->h_status, l.status, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
      cudaGraph_t graph = nullptr;
      const cudaError_t end = cudaStreamEndCapture(ctx->stream, &graph);  // always ends the capture
      if (err == cudaSuccess) err = end;
      if (err == cudaSuccess) err = cudaGraphInstantiate(&ctx->kmc_graph, graph, 0);
      if (graph) cudaGraphDestroy(graph);
      CudaCheck(err, "KMC graph capture");
      ctx->kmc_graph_key = std::move(key);
    }
    *ctx->h_status = 0;
    CudaCheck(cudaEventRecord(ctx->ev0, ctx->stream), "event");
    CudaCheck(cudaGraphLaunch(ctx->kmc_graph, ctx->stream), "cudaGraphLaunch");
    CudaCheck(cudaEventRecord(ctx->ev1, ctx->stream), "event");
    ctx->Sync();
    float ms = 0;
    CudaCheck(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1), "elapsed");
    ctx->last_ms = ms;
    RaiseStatus(*ctx->h_status, "KMC graph run");
  });
}

int lmc_kmc_autotune(lmc_ctx *ctx, uint64_t probe_steps, const char *cache_path, int *warps_per_replica,
                     int *replicas_per_block, int *evaluation, int *from_cache) {
  return Guard([&] {
    Require(ctx && ctx->kmc_ready, LMC_ERR_INVALID_ARGUMENT, "lmc_kmc_init has not been called");
    Require(probe_steps > 0, LMC_ERR_INVALID_ARGUMENT, "probe_steps must be > 0");
    Require(!ctx->kmc_opt.chain, LMC_ERR_UNSUPPORTED, "the chain KMC has a fixed launch shape");
    CudaCheck(cudaSetDevice(ctx->device), "cudaSetDevice");
    const std::string key = KmcTuneKey(ctx);
    std::map<std::string, KmcTuneEntry> cache;
    if (cache_path && *cache_path) cache = ReadTuneCache(cache_path);
    KmcTuneEntry best{};
    bool cached = false;
    auto hit = cache.find(key);
    if (hit != cache.end()) {
      lmc_kmc_options o = ctx->kmc_opt;
      o.warps_per_replica = hit->second.g;
      o.replicas_per_block = hit->second.rpb;
      o.evaluation = hit->second.eval;
      const lmc_kmc_options saved = ctx->kmc_opt;
      ctx->kmc_opt = o;
      try {
        int per_sm = 0;
        size_t bytes = 0;
        CudaCheck(lmc::KmcOccupancy(ctx->t, KmcShape(ctx), &per_sm, &bytes), "KMC occupancy");
        cached = per_sm >= 1;
      } catch (const LmcError &) {
        cached = false;
      }
      ctx->kmc_opt = saved;
      if (cached) best = hit->second;
    }
    if (!cached) {
      best = SweepKmcShapes(ctx, probe_steps);
      if (cache_path && *cache_path) {
        cache[key] = best;
        WriteTuneCache(cache_path, cache);
      }
    }
    ctx->kmc_opt.warps_per_replica = best.g;
    ctx->kmc_opt.replicas_per_block = best.rpb;
    ctx->kmc_opt.evaluation = best.eval;
    if (warps_per_replica) *warps_per_replica = best.g;
    if (replicas_per_block) *replicas_per_block = best.rpb;
    if (evaluation) *evaluation = best.eval;
    if (from_cache) *from_cache = cached ? 1 : 0;
  });
}

int lmc_kmc_get_escaped(lmc_ctx *ctx, uint8_t *escaped) {
  return Guard([&] {
    Require(ctx && ctx->kmc_ready && escaped, LMC_ERR_INVALID_ARGUMENT, "lmc_kmc_init has not been called");
    CudaCheck(cudaSetDevice(ctx->device), "cudaSetDevice");
    CudaCheck(cudaMemcpyAsync(escaped, ctx->k_escaped.p, ctx->num_replicas, cudaMemcpyDeviceToHost, ctx->stream),
              "D2H");
    ctx->Sync();
  });
}

int lmc_kmc_multi_init(lmc_ctx *ctx, const double *temperature, uint64_t seed, int barrier_kind, int evaluation) {
  return Guard([&] {
    Require(ctx && temperature && ctx->num_replicas > 0, LMC_ERR_INVALID_ARGUMENT, "bad argument");
    Require(barrier_kind == LMC_BARRIER_QUARTIC || barrier_kind == LMC_BARRIER_E0, LMC_ERR_INVALID_ARGUMENT,
            "unknown barrier kind");
    Require(evaluation == LMC_EVAL_SPARSE || evaluation == LMC_EVAL_DENSE, LMC_ERR_INVALID_ARGUMENT,
            "unknown evaluation");
    CudaCheck(cudaSetDevice(ctx->device), "cudaSetDevice");
    const int R = ctx->num_replicas;
    for (int r = 0; r < R; ++r)
      Require(temperature[r] > 0 && std::isfinite(temperature[r]), LMC_ERR_INVALID_ARGUMENT, "temperature must be > 0");
    ctx->multi_ready = false;
    // vacancy slots of every lattice (ascending site id) and the species histogram
    std::vector<int8_t> host(static_cast<size_t>(ctx->total_sites));
    ctx->Sync();
    CudaCheck(cudaMemcpy(host.data(), ctx->species.p, host.size(), cudaMemcpyDeviceToHost), "D2H species");
    const int e = ctx->fm.num_species, x = ctx->fm.x_code;
    std::vector<long long> pos;
    std::vector<int> off(R + 1, 0);
    std::vector<unsigned long long> tot(e, 0);
    for (int r = 0; r < R; ++r) {
      const long long nsites = 4LL * ctx->n[r] * ctx->n[r] * ctx->n[r];
      const int8_t *sp = host.data() + ctx->offsets[r];
      for (long long i = 0; i < nsites; ++i) {
        const int c = sp[i];
        Require(c >= 0 && c < e, LMC_ERR_INVALID_ARGUMENT, "species code out of range");
        ++tot[c];
        if (c == x) pos.push_back(i);
      }
      off[r + 1] = static_cast<int>(pos.size());
      const int nv = off[r + 1] - off[r];
      Require(nv >= 1 && nv <= lmc::kMaxMultiVac, LMC_ERR_UNSUPPORTED, "every lattice needs 1 to 256 vacancies");
    }
    int base = -1;
    for (int c = 0; c < e; ++c)
      if (c != x && ctx->fm.onehot_rank[c] >= 0 && (base < 0 || tot[c] > tot[base])) base = c;
    Require(base >= 0, LMC_ERR_INVALID_ARGUMENT, "no element of the barrier set in the lattices");
    BuildSparse(ctx, base);
    const size_t slots = pos.size();
    ctx->m_pos.Ensure(8 * slots);
    ctx->m_off.Ensure(sizeof(int) * (R + 1));
    ctx->m_steps.Ensure(8 * R);
    ctx->m_time.Ensure(8 * R);
    ctx->m_energy.Ensure(8 * R);
    ctx->m_temp.Ensure(8 * R);
    ctx->m_key.Ensure(8 * R);
    std::vector<uint32_t> key(2 * R);
    for (int r = 0; r < R; ++r) {
      key[2 * r] = static_cast<uint32_t>(seed);
      key[2 * r + 1] = static_cast<uint32_t>(seed >> 32);
    }
    std::vector<double> zeros(R, 0.0), temp(temperature, temperature + R);
    std::vector<unsigned long long> zu(R, 0);
    auto h2d = [&](DevBuf &d, const void *src, size_t bytes) {
      CudaCheck(cudaMemcpyAsync(d.p, src, bytes, cudaMemcpyHostToDevice, ctx->stream), "H2D");
    };
    h2d(ctx->m_pos, pos.data(), 8 * slots);
    h2d(ctx->m_off, off.data(), sizeof(int) * (R + 1));
    h2d(ctx->m_steps, zu.data(), 8 * R);
    h2d(ctx->m_time, zeros.data(), 8 * R);
    h2d(ctx->m_energy, zeros.data(), 8 * R);
    h2d(ctx->m_temp, temp.data(), 8 * R);
    h2d(ctx->m_key, key.data(), 8 * R);
    ctx->Sync();
    ctx->m_off_host = off;
    ctx->multi_kind = barrier_kind;
    ctx->multi_eval = evaluation;
    ctx->multi_ready = true;
  });
}

int lmc_kmc_multi_set_rates(lmc_ctx *ctx, int rates) {
  return Guard([&] {
    Require(ctx, LMC_ERR_INVALID_ARGUMENT, "null context");
    Require(rates == LMC_RATES_FP32 || rates == LMC_RATES_FP64, LMC_ERR_INVALID_ARGUMENT, "unknown rates mode");
    ctx->multi_rates = rates;
  });
}

int lmc_kmc_multi_run(lmc_ctx *ctx, uint64_t steps, int trace_replica, lmc_kmc_step *trace) {
  return Guard([&] {
    if (ctx) ctx->scan_fresh = false;  // atoms move
    Require(ctx && ctx->multi_ready, LMC_ERR_INVALID_ARGUMENT, "lmc_kmc_multi_init has not been called");
    CudaCheck(cudaSetDevice(ctx->device), "cudaSetDevice");
    if (steps == 0) return;
    lmc::KmcMultiArgs a{};
    a.vac_pos = ctx->m_pos.as<long long>();
    a.vac_off = ctx->m_off.as<int>();
    a.steps = ctx->m_steps.as<unsigned long long>();
    a.time = ctx->m_time.as<double>();
    a.energy = ctx->m_energy.as<double>();
    a.temperature = ctx->m_temp.as<double>();
    a.key = ctx->m_key.as<uint32_t>();
    a.lat_off = ctx->lat_off.as<long long>();
    a.lat_n = ctx->lat_n.as<int>();
    a.num_replicas = ctx->num_replicas;
    a.barrier_kind = ctx->multi_kind;
    a.f32 = ctx->multi_rates == LMC_RATES_FP32 ? 1 : 0;
    a.nsteps = steps;
    a.trace_replica = -1;
    if (trace) {
      ctx->CheckReplica(trace_replica);
      a.trace_replica = trace_replica;
      ctx->m_trace.Ensure(sizeof(lmc::KmcTraceRec) * steps);
      CudaCheck(cudaMemsetAsync(ctx->m_trace.p, 0, sizeof(lmc::KmcTraceRec) * steps, ctx->stream), "memset");
      a.trace = ctx->m_trace.as<lmc::KmcTraceRec>();
    }
    a.stop_flag = ctx->d_stop;
    a.status = ctx->status.as<int>();
    a.sp = ctx->sparse;
    std::copy(ctx->local_bits.begin(), ctx->local_bits.end(), a.local_bits);
    ctx->ClearStatus();
    CudaCheck(cudaEventRecord(ctx->ev0, ctx->stream), "event");
    CudaCheck(lmc::LaunchKmcMulti(ctx->t, ctx->species.as<int8_t>(), a, ctx->multi_eval == LMC_EVAL_SPARSE,
                                  ctx->stream),
              "multi-vacancy KMC kernel");
    CudaCheck(cudaEventRecord(ctx->ev1, ctx->stream), "event");
    if (trace)
      CudaCheck(cudaMemcpyAsync(trace, a.trace, sizeof(lmc::KmcTraceRec) * steps, cudaMemcpyDeviceToHost, ctx->stream),
                "D2H trace");
    const int st = ctx->ReadStatus();
    float ms = 0;
    CudaCheck(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1), "elapsed");
    ctx->last_ms = ms;
    RaiseStatus(st, "multi-vacancy KMC run");
  });
}

int lmc_kmc_multi_surrogate_run(lmc_ctx *ctx, lmc_mlp *mlp, uint64_t steps, float threshold_ev,
                                lmc_kmc_step *trace, double *plain_barrier, uint64_t *num_fallback) {
  return Guard([&] {
    if (ctx) ctx->scan_fresh = false;  // atoms move
    Require(ctx && mlp, LMC_ERR_INVALID_ARGUMENT, "null argument");
    Require(ctx->multi_ready, LMC_ERR_INVALID_ARGUMENT, "lmc_kmc_multi_init has not been called");
    Require(ctx->num_replicas == 1, LMC_ERR_UNSUPPORTED, "the surrogate-assisted run takes one lattice");
    Require(ctx->multi_kind == LMC_BARRIER_QUARTIC, LMC_ERR_UNSUPPORTED, "the surrogate predicts Quartic barriers");
    Require(threshold_ev >= 0.f, LMC_ERR_INVALID_ARGUMENT, "threshold_ev < 0");
    CudaCheck(cudaSetDevice(ctx->device), "cudaSetDevice");
    if (num_fallback) *num_fallback = 0;
    if (steps == 0) return;
    const int nv = ctx->m_off_host.back();
    const size_t rows = static_cast<size_t>(nv) * 12;
    ctx->su_pairs.Ensure(16 * rows);
    ctx->su_dirty.Ensure(4 * nv);
    ctx->su_mean.Ensure(4 * rows);
    ctx->su_spread.Ensure(4 * rows);
    ctx->su_cum.Ensure(8 * rows);
    ctx->su_ea.Ensure(8 * rows);
    ctx->su_tgt.Ensure(8 * rows);
    ctx->su_kmask.Ensure(4 * nv);
    ctx->su_pair_ea.Ensure(8 * rows);
    ctx->su_fb.Ensure(8);
    ctx->su_halt.Ensure(8);
    // the lattice and encoding of the network's gather
    lmc::FusedJumps j;
    Require(FusedJumpsFor(ctx, 0, nullptr, 0, nullptr, nullptr, &j) &&
                lmc::MlpFusedChannels(lmc::MlpDevOf(mlp)) == j.channels,
            LMC_ERR_UNSUPPORTED,
            "the surrogate-assisted run needs the solute-channel encoding and a network the fused jump kernel serves "
            "(2 members, hidden 128, 128 / 192 inputs)");
    lmc::MlpLabelScaleOf(mlp, &j.mean_label, &j.std_label);
    unsigned long long step0 = 0;
    CudaCheck(cudaMemcpy(&step0, ctx->m_steps.p, 8, cudaMemcpyDeviceToHost), "D2H");
    uint32_t key[2] = {0, 0};
    CudaCheck(cudaMemcpy(key, ctx->m_key.p, 8, cudaMemcpyDeviceToHost), "D2H");
    double temp = 0;
    CudaCheck(cudaMemcpy(&temp, ctx->m_temp.p, 8, cudaMemcpyDeviceToHost), "D2H");
    lmc::KmcSurrogateArgs a{};
    a.vac_pos = ctx->m_pos.as<long long>();
    a.nv = nv;
    a.nsteps = steps;
    a.steps = ctx->m_steps.as<unsigned long long>();
    a.time = ctx->m_time.as<double>();
    a.energy = ctx->m_energy.as<double>();
    a.temperature = temp;
    a.key0 = key[0];
    a.key1 = key[1];
    a.replica = 0;
    a.lat_off = ctx->offsets[0];
    a.n = ctx->n[0];
    a.barrier_kind = ctx->multi_kind;
    a.threshold = threshold_ev;
    a.mean = ctx->su_mean.as<float>();
    a.spread = ctx->su_spread.as<float>();
    a.pairs = ctx->su_pairs.as<long long>();
    a.dirty = ctx->su_dirty.as<int>();
    a.cum = ctx->su_cum.as<double>();
    a.ea = ctx->su_ea.as<double>();
    a.tgt = ctx->su_tgt.as<long long>();
    a.kmask = ctx->su_kmask.as<uint32_t>();
    a.pair_ea = ctx->su_pair_ea.as<double>();
    a.fallbacks = ctx->su_fb.as<unsigned long long>();
    a.halt = ctx->su_halt.as<int>();
    a.net_status = ctx->su_halt.as<int>() + 1;
    a.trace_base = step0;
    if (trace || plain_barrier) {
      ctx->su_trace.Ensure(sizeof(lmc::KmcTraceRec) * steps);
      ctx->su_plain.Ensure(8 * steps);
      CudaCheck(cudaMemsetAsync(ctx->su_trace.p, 0, sizeof(lmc::KmcTraceRec) * steps, ctx->stream), "memset");
      a.trace = ctx->su_trace.as<lmc::KmcTraceRec>();
      a.plain_ea = ctx->su_plain.as<double>();
      a.trace_len = steps;
    }
    a.stop_flag = ctx->d_stop;
    a.status = ctx->status.as<int>();
    std::copy(ctx->local_bits.begin(), ctx->local_bits.end(), a.local_bits);
    ctx->ClearStatus();
    CudaCheck(cudaMemsetAsync(ctx->su_fb.p, 0, 8, ctx->stream), "memset");
    CudaCheck(cudaMemsetAsync(ctx->su_halt.p, 0, 8, ctx->stream), "memset");
    // one persistent launch: the network's weights stay in shared memory for the whole run
    CudaCheck(cudaEventRecord(ctx->ev0, ctx->stream), "event");
    CudaCheck(lmc::LaunchKmcSurrogate(ctx->t, ctx->species.as<int8_t>(), a, lmc::MlpDevOf(mlp), j, ctx->stream),
              "surrogate-assisted KMC kernel");
    CudaCheck(cudaEventRecord(ctx->ev1, ctx->stream), "event");
    if (trace)
      CudaCheck(cudaMemcpyAsync(trace, ctx->su_trace.p, sizeof(lmc::KmcTraceRec) * steps, cudaMemcpyDeviceToHost,
                                ctx->stream),
                "D2H trace");
    if (plain_barrier)
      CudaCheck(cudaMemcpyAsync(plain_barrier, ctx->su_plain.p, 8 * steps, cudaMemcpyDeviceToHost, ctx->stream), "D2H");
    int *h = ctx->Pinned();
    CudaCheck(cudaMemcpyAsync(h, ctx->su_halt.p, 2 * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream), "D2H");
    unsigned long long fb = 0;
    CudaCheck(cudaMemcpyAsync(&fb, ctx->su_fb.p, 8, cudaMemcpyDeviceToHost, ctx->stream), "D2H");
    const int st = ctx->ReadStatus();  // synchronises
    float ms = 0;
    CudaCheck(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1), "elapsed");
    ctx->last_ms = ms;
    if (num_fallback) *num_fallback = fb;
    Require(h[1] == 0, LMC_ERR_STOPPED, "surrogate-assisted KMC: a tensor-core wait expired");
    RaiseStatus(st, "surrogate-assisted multi-vacancy KMC run");
  });
}

int lmc_kmc_multi_slots(lmc_ctx *ctx, int32_t *slot_offsets) {
  return Guard([&] {
    Require(ctx && ctx->multi_ready && slot_offsets, LMC_ERR_INVALID_ARGUMENT, "lmc_kmc_multi_init has not been called");
    std::copy(ctx->m_off_host.begin(), ctx->m_off_host.end(), slot_offsets);
  });
}

int lmc_kmc_multi_get_state(lmc_ctx *ctx, int64_t *vacancies, uint64_t *steps, double *time, double *energy) {
  return Guard([&] {
    Require(ctx && ctx->multi_ready, LMC_ERR_INVALID_ARGUMENT, "lmc_kmc_multi_init has not been called");
    CudaCheck(cudaSetDevice(ctx->device), "cudaSetDevice");
    const size_t R = ctx->num_replicas, slots = ctx->m_off_host.back();
    if (vacancies)
      CudaCheck(cudaMemcpyAsync(vacancies, ctx->m_pos.p, 8 * slots, cudaMemcpyDeviceToHost, ctx->stream), "D2H");
    if (steps) CudaCheck(cudaMemcpyAsync(steps, ctx->m_steps.p, 8 * R, cudaMemcpyDeviceToHost, ctx->stream), "D2H");
    if (time) CudaCheck(cudaMemcpyAsync(time, ctx->m_time.p, 8 * R, cudaMemcpyDeviceToHost, ctx->stream), "D2H");
    if (energy) CudaCheck(cudaMemcpyAsync(energy, ctx->m_energy.p, 8 * R, cudaMemcpyDeviceToHost, ctx->stream), "D2H");
    ctx->Sync();
  });
}

int lmc_sa_init(lmc_ctx *ctx, int replica, uint64_t seed, uint64_t maximum_steps, double initial_temperature,
                double initial_energy) {
  return Guard([&] {
    Require(ctx != nullptr, LMC_ERR_INVALID_ARGUMENT, "ctx is null");
    ctx->CheckReplica(replica);
    Require(initial_temperature > 0 && std::isfinite(initial_temperature), LMC_ERR_INVALID_ARGUMENT,
            "initial_temperature must be > 0");
    CudaCheck(cudaSetDevice(ctx->device), "cudaSetDevice");
    Require(SpeciesPresent(ctx, replica) >= 2, LMC_ERR_INVALID_ARGUMENT,
            "simulated annealing needs at least two species in the lattice");
    lmc::SaState st{};
    st.steps = 0;
    st.maximum_steps = maximum_steps;
    // SimulatedAnnealing constructor (SimulatedAnnealing.cpp:53-56): schedule lengths from maximum_steps
    auto frac = [&](double r) {
      return std::max<unsigned long long>(1ULL, static_cast<unsigned long long>(static_cast<double>(maximum_steps) * r));
    };
    st.reheat_trigger = frac(0.05);
    st.reheat_cooldown = frac(0.10);
    st.window_size = frac(0.001);
    st.temperature = initial_temperature;
    st.beta = 1.0 / 8.617333262145e-5 / initial_temperature;
    st.energy = st.lowest = st.recent_best = initial_energy;
    ctx->sa_state.Ensure(sizeof(lmc::SaState));
    ctx->sa_rng.Ensure(sizeof(uint32_t) * lmc::kRngWords);
    std::vector<uint32_t> w(lmc::kRngWords, 0);
    lmc::MtSeed(seed, w.data());
    CudaCheck(cudaMemcpy(ctx->sa_state.p, &st, sizeof(st), cudaMemcpyHostToDevice), "H2D");
    CudaCheck(cudaMemcpy(ctx->sa_rng.p, w.data(), 4 * w.size(), cudaMemcpyHostToDevice), "H2D");
    ctx->sa_replica = replica;
    ctx->sa_ready = true;
  });
}

int lmc_sa_run(lmc_ctx *ctx, uint64_t steps, lmc_sa_step *trace) {
  return Guard([&] {
    if (ctx) ctx->scan_fresh = false;  // atoms move
    Require(ctx && ctx->sa_ready, LMC_ERR_INVALID_ARGUMENT, "lmc_sa_init has not been called");
    CudaCheck(cudaSetDevice(ctx->device), "cudaSetDevice");
    if (steps == 0) return;
    static_assert(sizeof(lmc_sa_step) == sizeof(lmc::SaStepRec), "trace record layout");
    lmc::SaArgs a{};
    a.n = ctx->n[ctx->sa_replica];
    a.steps = steps;
    a.rng = ctx->sa_rng.as<uint32_t>();
    a.state = ctx->sa_state.as<lmc::SaState>();
    if (trace) {
      ctx->sa_trace.Ensure(sizeof(lmc::SaStepRec) * steps);
      a.trace = ctx->sa_trace.as<lmc::SaStepRec>();
    }
    a.stop_flag = ctx->d_stop;
    a.status = ctx->status.as<int>();
    ctx->ClearStatus();
    CudaCheck(cudaEventRecord(ctx->ev0, ctx->stream), "event");
    CudaCheck(lmc::LaunchSa(ctx->t, ctx->species.as<int8_t>() + ctx->offsets[ctx->sa_replica], a, ctx->stream),
              "annealing kernel");
    CudaCheck(cudaEventRecord(ctx->ev1, ctx->stream), "event");
    if (trace)
      CudaCheck(cudaMemcpyAsync(trace, a.trace, sizeof(lmc::SaStepRec) * steps, cudaMemcpyDeviceToHost, ctx->stream),
                "D2H trace");
    const int st = ctx->ReadStatus();
    float ms = 0;
    CudaCheck(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1), "elapsed");
    ctx->last_ms = ms;
    RaiseStatus(st, "simulated annealing");
  });
}

int lmc_sa_get_state(lmc_ctx *ctx, uint64_t *steps, double *temperature, double *energy, double *lowest_energy) {
  return Guard([&] {
    Require(ctx && ctx->sa_ready, LMC_ERR_INVALID_ARGUMENT, "lmc_sa_init has not been called");
    lmc::SaState st{};
    CudaCheck(cudaMemcpyAsync(&st, ctx->sa_state.p, sizeof(st), cudaMemcpyDeviceToHost, ctx->stream), "D2H");
    ctx->Sync();
    if (steps) *steps = st.steps;
    if (temperature) *temperature = st.temperature;
    if (energy) *energy = st.energy;
    if (lowest_energy) *lowest_energy = st.lowest;
  });
}

int lmc_site_de_batch(lmc_ctx *ctx, int replica, const int64_t *sites, const int8_t *from_codes,
                      const int8_t *to_codes, int64_t m, int64_t fill_site, int fill_code, double *de) {
  return Guard([&] {
    Require(ctx && sites && to_codes && de, LMC_ERR_INVALID_ARGUMENT, "null argument");
    ctx->CheckReplica(replica);
    Require(m >= 0, LMC_ERR_INVALID_ARGUMENT, "m < 0");
    if (m == 0) return;
    CudaCheck(cudaSetDevice(ctx->device), "cudaSetDevice");
    const int n = ctx->n[replica];
    const long long nsites = 4LL * n * n * n;
    const int e = ctx->fm.num_species;
    Require(fill_site < nsites, LMC_ERR_OUT_OF_RANGE, "fill_site out of range");
    Require(fill_site < 0 || (fill_code >= 0 && fill_code < e), LMC_ERR_INVALID_ARGUMENT, "fill_code out of range");
    for (int64_t q = 0; q < m; ++q) {
      Require(sites[q] >= 0 && sites[q] < nsites, LMC_ERR_OUT_OF_RANGE, "site out of range");
      Require(to_codes[q] >= 0 && to_codes[q] < e, LMC_ERR_INVALID_ARGUMENT, "species code out of range");
      Require(!from_codes || (from_codes[q] >= 0 && from_codes[q] < e), LMC_ERR_INVALID_ARGUMENT,
              "species code out of range");
    }
    DevBuf d_sites, d_from, d_to, d_de;
    d_sites.Alloc(sizeof(long long) * m);
    d_to.Alloc(m);
    d_de.Alloc(sizeof(double) * m);
    CudaCheck(cudaMemcpyAsync(d_sites.p, sites, sizeof(long long) * m, cudaMemcpyHostToDevice, ctx->stream), "H2D");
    CudaCheck(cudaMemcpyAsync(d_to.p, to_codes, m, cudaMemcpyHostToDevice, ctx->stream), "H2D");
    if (from_codes) {
      d_from.Alloc(m);
      CudaCheck(cudaMemcpyAsync(d_from.p, from_codes, m, cudaMemcpyHostToDevice, ctx->stream), "H2D");
    }
    CudaCheck(cudaEventRecord(ctx->ev0, ctx->stream), "event");
    CudaCheck(lmc::LaunchSiteDe(ctx->t, ctx->species.as<int8_t>() + ctx->offsets[replica], n, d_sites.as<long long>(),
                                from_codes ? d_from.as<int8_t>() : nullptr, d_to.as<int8_t>(), m, fill_site, fill_code,
                                d_de.as<double>(), ctx->stream),
              "site dE kernel");
    CudaCheck(cudaEventRecord(ctx->ev1, ctx->stream), "event");
    CudaCheck(cudaMemcpyAsync(de, d_de.p, sizeof(double) * m, cudaMemcpyDeviceToHost, ctx->stream), "D2H");
    ctx->Sync();
    float ms = 0;
    CudaCheck(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1), "elapsed");
    ctx->last_ms = ms;
  });
}

int lmc_exit_time_energies(lmc_ctx *ctx, int replica, int solvent_code, const double *chemical_potential,
                           double *binding, double *profile) {
  return Guard([&] {
    Require(ctx && chemical_potential, LMC_ERR_INVALID_ARGUMENT, "null argument");
    ctx->CheckReplica(replica);
    Require(solvent_code >= 0 && solvent_code < ctx->fm.num_species && solvent_code != ctx->fm.x_code,
            LMC_ERR_INVALID_ARGUMENT, "solvent code out of range");
    Require(ctx->fm.num_species - 1 <= 5, LMC_ERR_UNSUPPORTED, "at most 5 elements besides X");
    CudaCheck(cudaSetDevice(ctx->device), "cudaSetDevice");
    const int n = ctx->n[replica];
    const long long nsites = 4LL * n * n * n;
    const int e = ctx->fm.num_species;
    // the lattice's vacancy (Config::GetVacancyAtomId: its first X), from the replica scan
    DevBuf hist, first, d_mu, d_bind, d_prof;
    hist.Alloc(sizeof(unsigned long long) * (lmc::kMaxSpecies + 1));
    first.Alloc(sizeof(long long));
    const long long big = std::numeric_limits<long long>::max();
    CudaCheck(cudaMemcpyAsync(first.p, &big, sizeof(big), cudaMemcpyHostToDevice, ctx->stream), "H2D");
    CudaCheck(cudaMemsetAsync(hist.p, 0, hist.bytes, ctx->stream), "memset");
    CudaCheck(lmc::LaunchReplicaScan(ctx->species.as<int8_t>(), ctx->lat_off.as<long long>() + replica,
                                     ctx->lat_n.as<int>() + replica, 1, ctx->fm.x_code, e, first.as<long long>(),
                                     hist.as<unsigned long long>(), ctx->stream),
              "scan kernel");
    d_mu.Alloc(sizeof(double) * e);
    d_bind.Alloc(sizeof(double) * (e - 1) * nsites);
    d_prof.Alloc(sizeof(double) * nsites);
    CudaCheck(cudaMemcpyAsync(d_mu.p, chemical_potential, sizeof(double) * e, cudaMemcpyHostToDevice, ctx->stream),
              "H2D");
    long long vac = big;
    CudaCheck(cudaMemcpyAsync(&vac, first.p, sizeof(vac), cudaMemcpyDeviceToHost, ctx->stream), "D2H");
    ctx->Sync();
    if (vac == big) vac = -1;
    CudaCheck(cudaEventRecord(ctx->ev0, ctx->stream), "event");
    CudaCheck(lmc::LaunchExitEnergies(ctx->t, ctx->species.as<int8_t>() + ctx->offsets[replica], n, vac, solvent_code,
                                      d_mu.as<double>(), d_bind.as<double>(), d_prof.as<double>(), ctx->stream),
              "exit energy kernel");
    CudaCheck(cudaEventRecord(ctx->ev1, ctx->stream), "event");
    if (binding)
      CudaCheck(cudaMemcpyAsync(binding, d_bind.p, d_bind.bytes, cudaMemcpyDeviceToHost, ctx->stream), "D2H");
    if (profile)
      CudaCheck(cudaMemcpyAsync(profile, d_prof.p, d_prof.bytes, cudaMemcpyDeviceToHost, ctx->stream), "D2H");
    ctx->Sync();
    float ms = 0;
    CudaCheck(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1), "elapsed");
    ctx->last_ms = ms;
  });
}

int lmc_solute_clusters(lmc_ctx *ctx, int replica, int solvent_code, int64_t smallest, int64_t solvent_bond,
                        const double *chemical_potential, int64_t *num_clusters, int64_t *num_members) {
  return Guard([&] {
    Require(ctx != nullptr, LMC_ERR_INVALID_ARGUMENT, "ctx is null");
    ctx->CheckReplica(replica);
    Require(solvent_code >= 0 && solvent_code < ctx->fm.num_species && solvent_code != ctx->fm.x_code,
            LMC_ERR_INVALID_ARGUMENT, "solvent code out of range");
    Require(smallest >= 0 && solvent_bond >= 0, LMC_ERR_INVALID_ARGUMENT, "criteria must be >= 0");
    CudaCheck(cudaSetDevice(ctx->device), "cudaSetDevice");
    const int n = ctx->n[replica];
    const long long nsites = 4LL * n * n * n;
    const int8_t *d_sp = ctx->species.as<int8_t>() + ctx->offsets[replica];
    // components of the non-solvent sites on the GPU
    DevBuf parent;
    parent.Alloc(sizeof(uint32_t) * nsites);
    ctx->ClearStatus();
    CudaCheck(lmc::LaunchSoluteLabels(ctx->t, d_sp, n, solvent_code, parent.as<uint32_t>(), ctx->status.as<int>(),
                                      ctx->stream),
              "cluster label kernels");
    std::vector<uint32_t> root(nsites);
    std::vector<int8_t> sp(nsites);
    CudaCheck(cudaMemcpyAsync(root.data(), parent.p, sizeof(uint32_t) * nsites, cudaMemcpyDeviceToHost, ctx->stream),
              "D2H");
    CudaCheck(cudaMemcpyAsync(sp.data(), d_sp, nsites, cudaMemcpyDeviceToHost, ctx->stream), "D2H");
    ctx->Sync();
    RaiseStatus(ctx->ReadStatus(), "solute clusters");
    // SoluteCluster::FindAtomListOfClusters (SoluteCluster.cpp:324-372): the components, those
    // smaller than `smallest` dropped; a component of more than `solvent_bond` sites gains every
    // 1NN-shell site with more than `solvent_bond` bonds to it
    std::vector<std::pair<uint32_t, uint32_t>> by_root;
    for (long long i = 0; i < nsites; ++i)
      if (root[i] != 0xFFFFFFFFu) by_root.emplace_back(root[i], static_cast<uint32_t>(i));
    std::sort(by_root.begin(), by_root.end());
    lmc::Fcc fcc{n};
    const auto &nn1 = lmc::ShellOffsets(1);
    std::vector<std::vector<int64_t>> clusters;
    std::vector<int> mark(nsites, -1);
    for (size_t a = 0; a < by_root.size();) {
      size_t b = a;
      while (b < by_root.size() && by_root[b].first == by_root[a].first) ++b;
      const int64_t size = static_cast<int64_t>(b - a);
      if (size >= smallest) {
        const int id = static_cast<int>(clusters.size());
        std::vector<int64_t> c;
        for (size_t q = a; q < b; ++q) c.push_back(by_root[q].second), mark[by_root[q].second] = id;
        if (size > solvent_bond) {
          for (int64_t q = 0; q < size; ++q) {
            const lmc::I3 h = fcc.Coord(c[q]);
            for (const auto &o : nn1) {
              const int64_t x = fcc.Id(fcc.Wrap(h + o));
              if (mark[x] == id) continue;
              const lmc::I3 hx = fcc.Coord(x);
              int64_t bonds = 0;
              for (const auto &o2 : nn1) {
                const int64_t y = fcc.Id(fcc.Wrap(hx + o2));
                bonds += mark[y] == id && sp[y] != solvent_code;
              }
              if (bonds > solvent_bond) {
                c.push_back(x);
                mark[x] = id;
              }
            }
          }
          for (int64_t x : c)
            if (sp[x] == solvent_code) mark[x] = -1;  // solvent sites may join several clusters
        }
        std::sort(c.begin(), c.end());
        clusters.push_back(std::move(c));
      }
      a = b;
    }
    // larger clusters first; equal sizes by their first site id
    std::sort(clusters.begin(), clusters.end(), [](const std::vector<int64_t> &x, const std::vector<int64_t> &y) {
      return x.size() != y.size() ? x.size() > y.size() : x[0] < y[0];
    });
    const long long K = static_cast<long long>(clusters.size());
    ctx->cl_offsets.assign(1, 0);
    ctx->cl_members.clear();
    for (const auto &c : clusters) {
      ctx->cl_members.insert(ctx->cl_members.end(), c.begin(), c.end());
      ctx->cl_offsets.push_back(static_cast<int64_t>(ctx->cl_members.size()));
    }
    ctx->cl_energy.assign(K, std::numeric_limits<double>::quiet_NaN());
    if (chemical_potential && K > 0) {
      // SoluteCluster::GetFormationEnergy (SoluteCluster.cpp:395-410): GetEnergyOfCluster on the
      // members' species over a solvent background minus that of the pure solvent, on the set of
      // the members and their 1-3NN shells (one GPU block per cluster), minus the members'
      // chemical potentials
      std::vector<long long> s_off(1, 0), s_ids;
      std::vector<int64_t> shell;
      for (const auto &c : clusters) {
        shell.clear();
        for (int64_t x : c) {
          shell.push_back(x);
          const lmc::I3 h = fcc.Coord(x);
          for (int sh = 1; sh <= 3; ++sh)
            for (const auto &o : lmc::ShellOffsets(sh)) shell.push_back(fcc.Id(fcc.Wrap(h + o)));
        }
        std::sort(shell.begin(), shell.end());
        shell.erase(std::unique(shell.begin(), shell.end()), shell.end());
        s_ids.insert(s_ids.end(), shell.begin(), shell.end());
        s_off.push_back(static_cast<long long>(s_ids.size()));
      }
      DevBuf d_soff, d_sids, d_loff, d_lids, d_e;
      d_soff.Alloc(sizeof(long long) * s_off.size());
      d_sids.Alloc(sizeof(long long) * s_ids.size());
      d_loff.Alloc(sizeof(long long) * ctx->cl_offsets.size());
      d_lids.Alloc(sizeof(long long) * ctx->cl_members.size());
      d_e.Alloc(sizeof(double) * 2 * K);
      CudaCheck(cudaMemcpyAsync(d_soff.p, s_off.data(), d_soff.bytes, cudaMemcpyHostToDevice, ctx->stream), "H2D");
      CudaCheck(cudaMemcpyAsync(d_sids.p, s_ids.data(), d_sids.bytes, cudaMemcpyHostToDevice, ctx->stream), "H2D");
      CudaCheck(cudaMemcpyAsync(d_loff.p, ctx->cl_offsets.data(), d_loff.bytes, cudaMemcpyHostToDevice, ctx->stream),
                "H2D");
      CudaCheck(cudaMemcpyAsync(d_lids.p, ctx->cl_members.data(), d_lids.bytes, cudaMemcpyHostToDevice, ctx->stream),
                "H2D");
      CudaCheck(lmc::LaunchClusterCensus(ctx->t, d_sp, n, solvent_code, K, d_soff.as<long long>(),
                                         d_sids.as<long long>(), d_loff.as<long long>(), d_lids.as<long long>(),
                                         d_e.as<double>(), ctx->stream),
                "cluster census kernel");
      std::vector<double> e(2 * K);
      CudaCheck(cudaMemcpyAsync(e.data(), d_e.p, sizeof(double) * 2 * K, cudaMemcpyDeviceToHost, ctx->stream), "D2H");
      ctx->Sync();
      for (long long k = 0; k < K; ++k) {
        double mu = 0.0;
        for (int64_t q = ctx->cl_offsets[k]; q < ctx->cl_offsets[k + 1]; ++q) mu += chemical_potential[sp[ctx->cl_members[q]]];
        ctx->cl_energy[k] = (e[2 * k] - e[2 * k + 1]) - mu;
      }
    }
    if (num_clusters) *num_clusters = K;
    if (num_members) *num_members = static_cast<int64_t>(ctx->cl_members.size());
  });
}

int lmc_solute_cluster_get(lmc_ctx *ctx, int64_t *offsets, int64_t *members, double *formation_energy) {
  return Guard([&] {
    Require(ctx != nullptr, LMC_ERR_INVALID_ARGUMENT, "ctx is null");
    if (offsets) std::copy(ctx->cl_offsets.begin(), ctx->cl_offsets.end(), offsets);
    if (members) std::copy(ctx->cl_members.begin(), ctx->cl_members.end(), members);
    if (formation_energy) std::copy(ctx->cl_energy.begin(), ctx->cl_energy.end(), formation_energy);
  });
}

int lmc_site_jump_energetics(lmc_ctx *ctx, int replica, int kind, int solvent_code, double escape_temperature,
                             const int64_t *sites, int64_t m, double *ea12, double *de12, int64_t *nb12,
                             double *average, double *exit_time) {
  return Guard([&] {
    Require(ctx != nullptr, LMC_ERR_INVALID_ARGUMENT, "ctx is null");
    ctx->CheckReplica(replica);
    Require(kind == LMC_BARRIER_QUARTIC || kind == LMC_BARRIER_E0, LMC_ERR_INVALID_ARGUMENT, "unknown barrier kind");
    Require(solvent_code >= 0 && solvent_code < ctx->fm.num_species && solvent_code != ctx->fm.x_code,
            LMC_ERR_INVALID_ARGUMENT, "solvent code out of range");
    Require(escape_temperature > 0, LMC_ERR_INVALID_ARGUMENT, "escape_temperature must be > 0");
    CudaCheck(cudaSetDevice(ctx->device), "cudaSetDevice");
    const int n = ctx->n[replica];
    const long long nsites = 4LL * n * n * n;
    if (!sites) m = nsites;
    Require(m >= 0, LMC_ERR_INVALID_ARGUMENT, "m < 0");
    if (m == 0) return;
    if (sites)
      for (long long i = 0; i < m; ++i)
        Require(sites[i] >= 0 && sites[i] < nsites, LMC_ERR_OUT_OF_RANGE, "site out of range");
    // the lattice's own vacancy (Config::GetVacancyAtomId: the first X) and the sparse base
    DevBuf hist, first;
    hist.Alloc(sizeof(unsigned long long) * (lmc::kMaxSpecies + 1));
    first.Alloc(sizeof(long long));
    const long long big = std::numeric_limits<long long>::max();
    CudaCheck(cudaMemcpyAsync(first.p, &big, sizeof(big), cudaMemcpyHostToDevice, ctx->stream), "H2D");
    CudaCheck(cudaMemsetAsync(hist.p, 0, hist.bytes, ctx->stream), "memset");
    CudaCheck(lmc::LaunchReplicaScan(ctx->species.as<int8_t>(), ctx->lat_off.as<long long>() + replica,
                                     ctx->lat_n.as<int>() + replica, 1, ctx->fm.x_code, ctx->fm.num_species,
                                     first.as<long long>(), hist.as<unsigned long long>(), ctx->stream),
              "scan kernel");
    unsigned long long h[lmc::kMaxSpecies + 1];
    long long vac = big;
    CudaCheck(cudaMemcpyAsync(h, hist.p, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream), "D2H");
    CudaCheck(cudaMemcpyAsync(&vac, first.p, sizeof(vac), cudaMemcpyDeviceToHost, ctx->stream), "D2H");
    ctx->Sync();
    int base = -1;
    for (int c = 0; c < ctx->fm.num_species; ++c)
      if (c != ctx->fm.x_code && ctx->fm.onehot_rank[c] >= 0 && (base < 0 || h[c] > h[base])) base = c;
    Require(base >= 0, LMC_ERR_INVALID_ARGUMENT, "no element of the barrier set in the lattice");
    BuildSparse(ctx, base);
    DevBuf d_sites, d_ea, d_de, d_nb, d_avg, d_exit;
    lmc::SiteJumpArgs a{};
    a.n = n;
    if (sites) {
      d_sites.Alloc(8 * m);
      CudaCheck(cudaMemcpyAsync(d_sites.p, sites, 8 * m, cudaMemcpyHostToDevice, ctx->stream), "H2D");
      a.sites = d_sites.as<long long>();
    }
    a.m = m;
    a.vacancy = vac == big ? -1 : vac;
    a.solvent = solvent_code;
    a.barrier_kind = kind;
    a.beta_escape = 1.0 / 8.617333262145e-5 / escape_temperature;
    if (ea12) a.ea12 = (d_ea.Alloc(8 * 12 * m), d_ea.as<double>());
    if (de12) a.de12 = (d_de.Alloc(8 * 12 * m), d_de.as<double>());
    if (nb12) a.nb12 = (d_nb.Alloc(8 * 12 * m), d_nb.as<long long>());
    if (average) a.average = (d_avg.Alloc(8 * m), d_avg.as<double>());
    if (exit_time) a.exit_time = (d_exit.Alloc(8 * m), d_exit.as<double>());
    a.status = ctx->status.as<int>();
    a.sp = ctx->sparse;
    a.sparse = 1;
    ctx->ClearStatus();
    CudaCheck(cudaEventRecord(ctx->ev0, ctx->stream), "event");
    CudaCheck(lmc::LaunchSiteJumps(ctx->t, ctx->species.as<int8_t>() + ctx->offsets[replica], a, ctx->stream),
              "site jumps kernel");
    CudaCheck(cudaEventRecord(ctx->ev1, ctx->stream), "event");
    auto d2h = [&](void *dst, const DevBuf &src, size_t bytes) {
      if (dst) CudaCheck(cudaMemcpyAsync(dst, src.p, bytes, cudaMemcpyDeviceToHost, ctx->stream), "D2H");
    };
    d2h(ea12, d_ea, 8 * 12 * m);
    d2h(de12, d_de, 8 * 12 * m);
    d2h(nb12, d_nb, 8 * 12 * m);
    d2h(average, d_avg, 8 * m);
    d2h(exit_time, d_exit, 8 * m);
    const int st = ctx->ReadStatus();
    float ms = 0;
    CudaCheck(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1), "elapsed");
    ctx->last_ms = ms;
    RaiseStatus(st, "site jump energetics");
  });
}

int lmc_kmc_get_state(lmc_ctx *ctx, int64_t *vacancy, uint64_t *steps, double *time, double *energy) {
  return Guard([&] {
    Require(ctx && ctx->kmc_ready, LMC_ERR_INVALID_ARGUMENT, "lmc_kmc_init has not been called");
    const size_t R = ctx->num_replicas;
    if (vacancy) CudaCheck(cudaMemcpyAsync(vacancy, ctx->k_vac.p, 8 * R, cudaMemcpyDeviceToHost, ctx->stream), "D2H");
    if (steps) CudaCheck(cudaMemcpyAsync(steps, ctx->k_steps.p, 8 * R, cudaMemcpyDeviceToHost, ctx->stream), "D2H");
    if (time) CudaCheck(cudaMemcpyAsync(time, ctx->k_time.p, 8 * R, cudaMemcpyDeviceToHost, ctx->stream), "D2H");
    if (energy) CudaCheck(cudaMemcpyAsync(energy, ctx->k_energy.p, 8 * R, cudaMemcpyDeviceToHost, ctx->stream), "D2H");
    ctx->Sync();
  });
}

int lmc_last_run_ms(lmc_ctx *ctx, double *ms) {
  return Guard([&] {
    Require(ctx && ms, LMC_ERR_INVALID_ARGUMENT, "bad argument");
    *ms = ctx->last_ms;
  });
}

int lmc_cmc_run(lmc_ctx *ctx, int replica, double temperature, uint64_t attempts, const lmc_cmc_options *opt,
                double *energy_io, uint64_t *attempts_done, uint64_t *accepted) {
  return Guard([&] {
    if (ctx) ctx->scan_fresh = false;  // atoms move
    Require(ctx && opt && energy_io, LMC_ERR_INVALID_ARGUMENT, "bad argument");
    ctx->CheckReplica(replica);
    Require(temperature > 0 && std::isfinite(temperature), LMC_ERR_INVALID_ARGUMENT, "temperature must be > 0");
    CudaCheck(cudaSetDevice(ctx->device), "cudaSetDevice");
    const int n = ctx->n[replica];
    const long long nsites = 4LL * n * n * n;
    int8_t *lat = ctx->species.as<int8_t>() + ctx->offsets[replica];
    const double beta = 1.0 / 8.617333262145e-5 / temperature;  // McAbstract.cpp:29
    ctx->c_stats.Ensure(sizeof(unsigned long long) * 4 + sizeof(double) * 2);
    unsigned long long *d_done = ctx->c_stats.as<unsigned long long>();
    int *d_quit = reinterpret_cast<int *>(d_done + 2);
    double *d_energy = reinterpret_cast<double *>(d_done + 4);
    CudaCheck(cudaMemsetAsync(d_done, 0, sizeof(unsigned long long) * 4, ctx->stream), "memset");
    // both CMC modes redraw pairs until the two species differ: refuse a
    // lattice with a single species instead of spinning on it
    Require(SpeciesPresent(ctx, replica) >= 2, LMC_ERR_INVALID_ARGUMENT,
            "canonical MC needs at least two species in the lattice");
    CudaCheck(cudaMemcpyAsync(d_energy, energy_io, sizeof(double), cudaMemcpyHostToDevice, ctx->stream), "H2D");
    ctx->ClearStatus();
    double e_out = *energy_io;
    if (opt->mode == LMC_CMC_REFERENCE_BATCH) {
      Require(opt->batch >= 1 && opt->batch <= 256, LMC_ERR_INVALID_ARGUMENT, "batch must be in [1, 256]");
      auto &slot = ctx->c_mt[replica];
      if (slot.second.p == nullptr || slot.first != opt->seed) {
        std::vector<uint32_t> w(lmc::kRngWords);
        lmc::MtSeed(opt->seed, w.data());
        slot.second.Alloc(sizeof(uint32_t) * lmc::kRngWords);
        CudaCheck(cudaMemcpy(slot.second.p, w.data(), sizeof(uint32_t) * lmc::kRngWords, cudaMemcpyHostToDevice), "H2D");
        slot.first = opt->seed;
      }
      lmc::CmcRefArgs a{};
      a.n = n;
      a.beta = beta;
      a.attempts = attempts;
      a.batch = opt->batch;
      a.rng = slot.second.as<uint32_t>();
      a.energy = d_energy;
      a.done = d_done;
      a.accepted = d_done + 1;
      a.status = ctx->status.as<int>();
      const size_t trace_n = static_cast<size_t>(attempts) + opt->batch;
      if (opt->energy_trace) {
        ctx->c_trace.Ensure(sizeof(double) * trace_n);
        a.energy_trace = ctx->c_trace.as<double>();
      }
      CudaCheck(cudaEventRecord(ctx->ev0, ctx->stream), "event");
      CudaCheck(lmc::LaunchCmcReference(ctx->t, lat, a, ctx->stream), "CMC kernel");
      CudaCheck(cudaEventRecord(ctx->ev1, ctx->stream), "event");
      CudaCheck(cudaMemcpyAsync(&e_out, d_energy, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream), "D2H");
      if (opt->energy_trace)
        CudaCheck(cudaMemcpyAsync(opt->energy_trace, ctx->c_trace.p, sizeof(double) * trace_n, cudaMemcpyDeviceToHost,
                                  ctx->stream),
                  "D2H");
    } else if (opt->mode == LMC_CMC_THROUGHPUT) {
      int cand = opt->candidates;
      if (cand <= 0) {
        // Surviving pairs per round grow with the candidates until the lattice
        // is saturated (about N / 172 pairs fit 3NN apart); the round's latency
        // grows once candidates outnumber the resident warps (measured on GB300:
        // the optimum is near N / 80 at n = 30, and at n = 64 near 4/5 of the
        // resident warps: 2.1e8 swaps/s against 1.95e8 at 3/5 and 1.6e8 at 1.03x).
        const long long warps = lmc::CmcThroughputResidentWarps(ctx->t, ctx->device);
        long long c = nsites / 80;
        if (warps > 0) c = std::min(c, warps * 4 / 5);
        cand = static_cast<int>(std::min<long long>(65535, std::max<long long>(32, c)));
      }
      Require(cand <= 65535, LMC_ERR_INVALID_ARGUMENT, "at most 65535 candidates per round");
      ctx->c_claim.Ensure(sizeof(unsigned long long) * nsites);
      ctx->c_cand.Ensure(sizeof(long long) * 2 * cand);
      int sms = 0;
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
      ctx->c_eacc.Ensure(sizeof(double) * sms * 8);
      CudaCheck(cudaMemsetAsync(ctx->c_claim.p, 0, sizeof(unsigned long long) * nsites, ctx->stream), "memset");
      CudaCheck(cudaMemsetAsync(ctx->c_eacc.p, 0, sizeof(double) * sms * 8, ctx->stream), "memset");
      lmc::CmcTpArgs a{};
      a.n = n;
      a.beta = beta;
      a.attempts = attempts;
      a.candidates = cand;
      a.seed = opt->seed;
      a.claim = ctx->c_claim.as<unsigned long long>();
      a.cand = ctx->c_cand.as<long long>();
      a.energy_acc = ctx->c_eacc.as<double>();
      a.done = d_done;
      a.accepted = d_done + 1;
      a.quit = d_quit;
      a.status = ctx->status.as<int>();
      a.stop_flag = ctx->d_stop;
      a.rounds = d_done + 3;
      CudaCheck(cudaEventRecord(ctx->ev0, ctx->stream), "event");
      CudaCheck(lmc::LaunchCmcThroughput(ctx->t, lat, a, ctx->device, ctx->stream), "CMC kernel");
      CudaCheck(cudaEventRecord(ctx->ev1, ctx->stream), "event");
      std::vector<double> eacc(sms * 8);
      CudaCheck(cudaMemcpyAsync(eacc.data(), ctx->c_eacc.p, sizeof(double) * sms * 8, cudaMemcpyDeviceToHost,
                                ctx->stream),
                "D2H");
      ctx->Sync();
      for (double v : eacc) e_out += v;
    } else {
      throw LmcError(LMC_ERR_INVALID_ARGUMENT, "unknown CMC mode");
    }
    unsigned long long stats[4] = {0, 0, 0, 0};
    CudaCheck(cudaMemcpyAsync(stats, d_done, sizeof(stats), cudaMemcpyDeviceToHost, ctx->stream), "D2H");
    const int st = ctx->ReadStatus();
    float ms = 0;
    CudaCheck(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1), "elapsed");
    ctx->last_ms = ms;
    ctx->cmc_rounds = opt->mode == LMC_CMC_THROUGHPUT ? stats[3] : 0;
    RaiseStatus(st, "CMC run");
    *energy_io = e_out;
    if (attempts_done) *attempts_done = stats[0];
    if (accepted) *accepted = stats[1];
  });
}

int lmc_cmc_rounds(const lmc_ctx *ctx, uint64_t *rounds) {
  return Guard([&] {
    Require(ctx && rounds, LMC_ERR_INVALID_ARGUMENT, "null argument");
    *rounds = ctx->cmc_rounds;
  });
}

int lmc_request_stop(lmc_ctx *ctx, int value) {
  return Guard([&] {
    Require(ctx != nullptr, LMC_ERR_INVALID_ARGUMENT, "ctx is null");
    *reinterpret_cast<volatile int *>(ctx->h_stop) = value;
  });
}

}  // extern "C"
