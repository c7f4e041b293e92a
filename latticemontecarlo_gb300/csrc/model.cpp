// Species alphabet, ElementCluster indexing, coefficient loading and folding.
#include "model.hpp"

#include <algorithm>
#include <array>
#include <cmath>
#include <fstream>
#include <set>
#include <sstream>
#include <stdexcept>
#include <tuple>

#include "json.hpp"

namespace lmc {

// Label-indexed cluster counters: the energy-change predictors'
// (VacancyMigrationPredictorQuartic.cpp:13-15, EnergyChangePredictorPairSite.cpp:11)
// and the full-lattice census's (EnergyPredictor.cpp:8).
const double kDeClusterCounter[11] = {256, 1536, 768, 3072, 2048, 3072, 6144, 6144, 6144, 6144, 2048};
const double kCensusClusterCounter[11] = {256, 3072, 1536, 6144, 12288, 6144, 12288, 6144, 12288, 12288, 12288};

namespace {
const std::vector<std::string> kKnownElements = {"X", "Al", "Mg", "Zn", "Cu", "Sn"};

int Sz(int e) { return e; }

std::vector<double> Checked(const JsonValue &obj, const char *key) { return obj.At(key).Vector(); }

int ShiftFor(long double bound) {
  if (!(bound > 0)) return 62;
  const int s = static_cast<int>(std::floor(61.0L - std::log2(bound)));
  return std::max(0, std::min(62, s));
}
}  // namespace

int Model::Code(const std::string &name) const {
  for (int i = 0; i < NumSpecies(); ++i)
    if (alphabet[i] == name) return i;
  return -1;
}

int Model::FeaturesMmm() const { return GetPairTables().mmm.NumFeatures(NumOnehot()); }
int Model::FeaturesMm2() const { return GetPairTables().mm2.NumFeatures(NumOnehot()); }

int Model::ClusterIdx(int label, int c1, int c2, int c3) const {
  const int e = NumSpecies();
  return cluster_index[((label * e + c1) * e + c2) * e + c3];
}

Model MakeModel(const std::vector<std::string> &element_names) {
  Model m;
  std::set<std::string> names;
  for (const auto &raw : element_names) {
    if (!raw.empty() && raw[0] == 'p')
      throw std::invalid_argument("pseudo elements (" + raw + ") are not supported");
    const bool known = std::find(kKnownElements.begin(), kKnownElements.end(), raw) != kKnownElements.end();
    names.insert(known ? raw : std::string("X"));  // Element(std::string) maps unknown names to X
  }
  if (names.empty()) throw std::invalid_argument("empty element set");
  m.onehot.assign(names.begin(), names.end());
  names.insert("X");
  m.alphabet.assign(names.begin(), names.end());
  if (m.NumSpecies() > kMaxSpecies) throw std::invalid_argument("too many elements");
  m.x_code = m.Code("X");
  for (int c = 0; c < m.NumSpecies(); ++c) {
    auto it = std::find(m.onehot.begin(), m.onehot.end(), m.alphabet[c]);
    m.onehot_rank.push_back(it == m.onehot.end() ? -1 : static_cast<int>(it - m.onehot.begin()));
  }
  // ElementCluster keys of InitializeClusterHashMap (EnergyUtility.cpp:314-343)
  // in std::map order: size, then label, then the sorted element names.
  const int e = m.NumSpecies();
  const int x = m.x_code;
  std::vector<std::tuple<int, int, std::array<int, 3>>> keys;  // (size, label, codes)
  for (int c1 = 0; c1 < e; ++c1) keys.push_back({1, 0, {c1, -1, -1}});
  std::set<std::tuple<int, int, std::array<int, 3>>> uniq;
  for (int c1 = 0; c1 < e; ++c1)
    for (int c2 = 0; c2 < e; ++c2) {
      if (c2 == x) continue;
      for (int label = 1; label <= 3; ++label) {
        std::array<int, 3> s{std::min(c1, c2), std::max(c1, c2), -1};
        uniq.insert({2, label, s});
      }
      for (int c3 = 0; c3 < e; ++c3) {
        if (c3 == x) continue;
        std::array<int, 3> s{c1, c2, c3};
        std::sort(s.begin(), s.end());
        for (int label = 4; label < 8; ++label) uniq.insert({3, label, s});
      }
    }
  keys.insert(keys.end(), uniq.begin(), uniq.end());
  std::sort(keys.begin(), keys.end());
  m.num_theta = static_cast<int>(keys.size());
  m.cluster_index.assign(static_cast<size_t>(kMaxLabel * e * e * e), -1);
  for (int idx = 0; idx < m.num_theta; ++idx) {
    const auto &[size, label, c] = keys[idx];
    m.theta_label.push_back(label);
    std::array<int, 3> p = c;
    if (size == 1) {
      m.cluster_index[((label * e + p[0]) * e + 0) * e + 0] = idx;
    } else if (size == 2) {
      m.cluster_index[((label * e + p[0]) * e + p[1]) * e + 0] = idx;
      m.cluster_index[((label * e + p[1]) * e + p[0]) * e + 0] = idx;
    } else {
      std::sort(p.begin(), p.end());
      do {
        m.cluster_index[((label * e + p[0]) * e + p[1]) * e + p[2]] = idx;
      } while (std::next_permutation(p.begin(), p.end()));
    }
  }
  return m;
}

void LoadJson(Model &m, const std::string &path) {
  std::ifstream ifs(path);
  if (!ifs) throw std::ios_base::failure("Cannot open " + path);
  std::stringstream ss;
  ss << ifs.rdbuf();
  const JsonValue root = JsonValue::Parse(ss.str());
  if (!root.IsObject()) throw std::invalid_argument("coefficient file is not a JSON object");
  const int f_mmm = m.FeaturesMmm(), f_mm2 = m.FeaturesMm2();
  for (const auto &[name, obj] : root.Object()) {
    if (name == "Base") {
      m.base_theta = Checked(obj, "theta");
      continue;
    }
    const bool known = std::find(kKnownElements.begin(), kKnownElements.end(), name) != kKnownElements.end();
    const int code = m.Code(known ? name : std::string("X"));
    if (code < 0) continue;  // block for an element outside this model's alphabet: never queried
    if (obj.Has("U_mm2")) {
      QuarticBlock q;
      q.mu_x_mmm = Checked(obj, "mu_x_mmm");
      q.mu_x_mm2 = Checked(obj, "mu_x_mm2");
      q.sigma_x_mmm = Checked(obj, "sigma_x_mmm");
      q.sigma_x_mm2 = Checked(obj, "sigma_x_mm2");
      int r, c;
      q.u_mmm = obj.At("U_mmm").Matrix(&r, &c);
      q.k_mmm = r;
      if (c != f_mmm) throw std::invalid_argument(name + ": U_mmm has " + std::to_string(c) + " columns, expected " + std::to_string(f_mmm));
      q.u_mm2 = obj.At("U_mm2").Matrix(&r, &c);
      q.k_mm2 = r;
      if (c != f_mm2) throw std::invalid_argument(name + ": U_mm2 has " + std::to_string(c) + " columns, expected " + std::to_string(f_mm2));
      q.theta_d = Checked(obj, "theta_D");
      q.theta_ks = Checked(obj, "theta_Ks");
      q.mu_d = obj.At("mu_D").Number();
      q.mu_ks = obj.At("mu_Ks").Number();
      q.sigma_d = obj.At("sigma_D").Number();
      q.sigma_ks = obj.At("sigma_Ks").Number();
      m.quartic[code] = std::move(q);
    }
    if (obj.Has("theta_e0")) {
      E0Block b;
      b.mu_x_mmm = Checked(obj, "mu_x_mmm");
      b.sigma_x_mmm = Checked(obj, "sigma_x_mmm");
      int r, c;
      b.u_mmm = obj.At("U_mmm").Matrix(&r, &c);
      b.k_mmm = r;
      if (c != f_mmm) throw std::invalid_argument(name + ": U_mmm has wrong column count");
      b.theta_e0 = Checked(obj, "theta_e0");
      b.mu_e0 = obj.At("mu_e0").Number();
      b.sigma_e0 = obj.At("sigma_e0").Number();
      m.e0[code] = std::move(b);
    }
  }
  if (static_cast<int>(m.base_theta.size()) != m.num_theta)
    throw std::invalid_argument("Base.theta has " + std::to_string(m.base_theta.size()) + " entries, expected " +
                                std::to_string(m.num_theta));
}

int PairType(int mode, int ra, int rb, int e) {
  if (mode == 0) return ra;
  if (mode == 1) return ra * e + rb;
  const int lo = std::min(ra, rb), hi = std::max(ra, rb);
  return lo * e - lo * (lo - 1) / 2 + (hi - lo);
}

namespace {
// b = (U^T theta) / sigma folded with the orbit sizes of `enc`; `twice` when the
// same table is summed over two cluster lists (MM2 forward + backward).
FoldedForm FoldForm(const EnvEncoding &enc, int e, int k, const std::vector<double> &u, const std::vector<double> &theta,
                    const std::vector<double> &mu, const std::vector<double> &sigma, double mu_y, double sigma_y,
                    bool twice, const std::string &what) {
  const int f = enc.NumFeatures(e);
  if (static_cast<int>(mu.size()) != f || static_cast<int>(sigma.size()) != f)
    throw std::invalid_argument(what + ": mu/sigma length " + std::to_string(mu.size()) + " != " + std::to_string(f));
  if (static_cast<int>(theta.size()) != k || static_cast<int>(u.size()) != k * f)
    throw std::invalid_argument(what + ": theta/U shape mismatch");
  const auto offsets = enc.OrbitOffsets(e);
  std::vector<long double> v(f), b(f);
  long double c = 0;
  for (int j = 0; j < f; ++j) {
    long double a = 0;
    for (int r = 0; r < k; ++r) a += static_cast<long double>(u[static_cast<size_t>(r) * f + j]) * theta[r];
    b[j] = a / static_cast<long double>(sigma[j]);
    c += b[j] * static_cast<long double>(mu[j]);
  }
  for (size_t o = 0; o < enc.orbits.size(); ++o)
    for (int j = offsets[o]; j < offsets[o + 1]; ++j) v[j] = b[j] / static_cast<long double>(enc.orbits[o].size);
  long double bound = 0;
  for (const auto &cl : enc.clusters) {
    long double mx = 0;
    for (int j = offsets[cl.orbit]; j < offsets[cl.orbit + 1]; ++j) mx = std::max(mx, std::fabs(v[j]));
    bound += mx;
  }
  if (twice) bound *= 2;
  FoldedForm out;
  out.shift = ShiftFor(bound);
  out.w.resize(f);
  for (int j = 0; j < f; ++j) out.w[j] = static_cast<int64_t>(std::llround(std::ldexp(v[j], out.shift)));
  out.c = static_cast<double>(c);
  out.mu = mu_y;
  out.sigma = sigma_y;
  for (double s : sigma)
    if (!(std::isfinite(s)) || s == 0.0) throw std::invalid_argument(what + ": sigma_x has a zero or non-finite entry");
  return out;
}
}  // namespace

FoldedModel Fold(const Model &m) {
  const auto &t = GetPairTables();
  FoldedModel fm;
  const int e = m.NumSpecies();
  fm.num_species = e;
  fm.num_onehot = m.NumOnehot();
  fm.x_code = m.x_code;
  fm.num_theta = m.num_theta;
  fm.f_mmm = m.FeaturesMmm();
  fm.f_mm2 = m.FeaturesMm2();
  for (int r : m.onehot_rank) fm.onehot_rank.push_back(static_cast<int8_t>(r));
  fm.cluster_index.assign(m.cluster_index.begin(), m.cluster_index.end());
  if (static_cast<int>(m.base_theta.size()) != m.num_theta) throw std::invalid_argument("Base.theta not set");
  fm.theta = m.base_theta;
  long double wmax = 0;
  for (int idx = 0; idx < m.num_theta; ++idx)
    wmax = std::max(wmax, std::fabs(static_cast<long double>(m.base_theta[idx]) / kDeClusterCounter[m.theta_label[idx]]));
  fm.de_shift = ShiftFor(4096.0L * wmax);
  fm.w_de.assign(m.cluster_index.size(), 0);
  for (size_t i = 0; i < m.cluster_index.size(); ++i) {
    const int idx = m.cluster_index[i];
    if (idx < 0) continue;
    const long double w = static_cast<long double>(m.base_theta[idx]) / kDeClusterCounter[m.theta_label[idx]];
    fm.w_de[i] = static_cast<int64_t>(std::llround(std::ldexp(w, fm.de_shift)));
  }
  for (int idx = 0; idx < m.num_theta; ++idx) {
    fm.census_bonds.push_back(kCensusClusterCounter[m.theta_label[idx]]);
    fm.de_bonds.push_back(kDeClusterCounter[m.theta_label[idx]]);
    fm.census_weight.push_back(m.base_theta[idx] / kCensusClusterCounter[m.theta_label[idx]]);
  }
  fm.migrant_slot.assign(e, -1);
  std::set<int> codes;
  for (const auto &kv : m.quartic) codes.insert(kv.first);
  for (const auto &kv : m.e0) codes.insert(kv.first);
  for (int code : codes) {
    const int slot = static_cast<int>(fm.slot_code.size());
    fm.migrant_slot[code] = static_cast<int8_t>(slot);
    fm.slot_code.push_back(code);
    const std::string name = m.alphabet[code];
    auto q = m.quartic.find(code);
    if (q != m.quartic.end()) {
      const auto &b = q->second;
      fm.quartic_d.push_back(FoldForm(t.mmm, fm.num_onehot, b.k_mmm, b.u_mmm, b.theta_d, b.mu_x_mmm, b.sigma_x_mmm,
                                      b.mu_d, b.sigma_d, false, name + " D"));
      fm.quartic_ks.push_back(FoldForm(t.mm2, fm.num_onehot, b.k_mm2, b.u_mm2, b.theta_ks, b.mu_x_mm2, b.sigma_x_mm2,
                                       b.mu_ks, b.sigma_ks, true, name + " Ks"));
      fm.has_quartic.push_back(1);
    } else {
      fm.quartic_d.push_back(FoldedForm{std::vector<int64_t>(fm.f_mmm, 0), 0, 0, 0, 0});
      fm.quartic_ks.push_back(FoldedForm{std::vector<int64_t>(fm.f_mm2, 0), 0, 0, 0, 0});
      fm.has_quartic.push_back(0);
    }
    auto z = m.e0.find(code);
    if (z != m.e0.end()) {
      const auto &b = z->second;
      fm.e0.push_back(FoldForm(t.mmm, fm.num_onehot, b.k_mmm, b.u_mmm, b.theta_e0, b.mu_x_mmm, b.sigma_x_mmm, b.mu_e0,
                               b.sigma_e0, false, name + " e0"));
      fm.has_e0.push_back(1);
    } else {
      fm.e0.push_back(FoldedForm{std::vector<int64_t>(fm.f_mmm, 0), 0, 0, 0, 0});
      fm.has_e0.push_back(0);
    }
  }
  return fm;
}

void HostEncodePair(const Model &m, int n, const int8_t *species, int64_t first, int64_t second,
                    int32_t *state_start, int32_t *state_end, int32_t *mmm, int32_t *mm2_fwd, int32_t *mm2_bwd) {
  const auto &t = GetPairTables();
  const Fcc fcc{n};
  if (first < 0 || second < 0 || first >= fcc.NumSites() || second >= fcc.NumSites())
    throw std::out_of_range("lattice id out of range");
  const I3 hi = fcc.Coord(first), hj = fcc.Coord(second);
  I3 d = hj - hi;
  auto mi = [&](int v) { const int m2 = 2 * n; v %= m2; if (v < 0) v += m2; return v >= n ? v - m2 : v; };
  d = {mi(d.x), mi(d.y), mi(d.z)};
  const int di = DirectionIndex(d);
  if (di < 0) throw std::out_of_range("Neighbor not found for lattice pair in GetPairFlatIndex");
  const int db = DirectionIndex(I3{0, 0, 0} - d);
  auto sp = [&](I3 h) { return static_cast<int>(species[fcc.Id(fcc.Wrap(h))]); };
  const int e = m.NumSpecies();
  const int eh = m.NumOnehot();
  const int migrant = sp(hj);
  if (state_start || state_end) {
    std::vector<int32_t> cs(m.num_theta, 0), ce(m.num_theta, 0);
    int st[kStateSites], en[kStateSites];
    for (int k = 0; k < kStateSites; ++k) {
      st[k] = sp(hi + t.state_off[di][k]);
      en[k] = st[k];
    }
    en[t.pos_first] = migrant;
    en[t.pos_second] = m.x_code;
    for (const auto &c : t.state_clusters) {
      int a[3] = {0, 0, 0}, b[3] = {0, 0, 0};
      for (int s = 0; s < c.size; ++s) {
        a[s] = st[c.idx[s]];
        b[s] = en[c.idx[s]];
      }
      const int ia = m.ClusterIdx(c.label, a[0], a[1], a[2]);
      const int ib = m.ClusterIdx(c.label, b[0], b[1], b[2]);
      if (ia < 0 || ib < 0) throw std::out_of_range("Cluster not found in ClusterIndexer");
      ++cs[ia];
      ++ce[ib];
    }
    if (state_start) std::copy(cs.begin(), cs.end(), state_start);
    if (state_end) std::copy(ce.begin(), ce.end(), state_end);
  }
  auto env = [&](const EnvEncoding &enc, const I3 (*off)[kEnvSites], int dir, I3 origin, int32_t *out) {
    const auto offsets = enc.OrbitOffsets(eh);
    std::fill(out, out + offsets.back(), 0);
    int r[kEnvSites];
    for (int k = 0; k < kEnvSites; ++k) {
      r[k] = m.onehot_rank[sp(origin + off[dir][k])];
      if (r[k] < 0) throw std::out_of_range("element without a one-hot slot in the jump environment");
    }
    for (const auto &c : enc.clusters) {
      const int ra = r[c.a];
      const int rb = c.b >= 0 ? r[c.b] : 0;
      ++out[offsets[c.orbit] + PairType(c.mode, ra, rb, eh)];
    }
  };
  if (mmm) env(t.mmm, t.mmm_off, di, hi, mmm);
  if (mm2_fwd) env(t.mm2, t.mm2_off, di, hi, mm2_fwd);
  if (mm2_bwd) env(t.mm2, t.mm2_off, db, hj, mm2_bwd);
  (void)e;
  (void)Sz;
}

}  // namespace lmc
