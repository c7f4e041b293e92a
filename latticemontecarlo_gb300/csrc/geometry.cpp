// Exact-integer construction of the pair/site neighbourhood orders and cluster
// lists of the lattice-MC hot path. See geometry.hpp for the coordinate
// conventions and for why integer keys reproduce the reference's order.
#include "geometry.hpp"

#include <algorithm>
#include <map>
#include <stdexcept>
#include <tuple>

namespace lmc {
namespace {

std::vector<I3> MakeShell(int norm2) {
  std::vector<I3> out;
  for (int x = -2; x <= 2; ++x)
    for (int y = -2; y <= 2; ++y)
      for (int z = -2; z <= 2; ++z) {
        const I3 s{x, y, z};
        if (((x + y + z) & 1) == 0 && Norm2(s) == norm2) out.push_back(s);
      }
  // Lexicographic (x, y, z) order equals lattice-id order for an interior site.
  std::sort(out.begin(), out.end(), [](I3 a, I3 b) { return std::tie(a.x, a.y, a.z) < std::tie(b.x, b.y, b.z); });
  return out;
}

bool LexLess(I3 a, I3 b) { return std::tie(a.x, a.y, a.z) < std::tie(b.x, b.y, b.z); }

// Rotated integer coordinates of a site offset s (half units, from the pair
// origin) in the frame (d, v): q = 2s - d, then (q.d, q.v, q.(d x v)).
struct Rot {
  int n2, x, y, z;
};
Rot Rotate(I3 s, I3 d, I3 v) {
  const I3 q = 2 * s - d;
  return {Norm2(q), Dot(q, d), Dot(q, v), Dot(q, Cross(d, v))};
}

std::vector<I3> PairSet(I3 d) {
  std::vector<I3> set{I3{0, 0, 0}, d};
  for (int shell = 1; shell <= 3; ++shell)
    for (const auto &s : ShellOffsets(shell)) {
      for (const I3 c : {s, d + s})
        if (std::find(set.begin(), set.end(), c) == set.end()) set.push_back(c);
    }
  return set;
}

int TripletLabel(I3 a, I3 b, I3 c) {
  int l[3] = {DistanceLabel(a - b), DistanceLabel(b - c), DistanceLabel(c - a)};
  std::sort(l, l + 3);
  if (l[0] == 1 && l[1] == 1 && l[2] == 1) return 4;
  if (l[0] == 1 && l[1] == 1 && l[2] == 2) return 5;
  if (l[0] == 1 && l[1] == 1 && l[2] == 3) return 6;
  if (l[0] == 1 && l[1] == 2 && l[2] == 3) return 7;
  return -1;  // labels 8-10 are not part of the reference's encodings
}

// Loop structure of GetClusterParametersMappingState{Pair,Site}
// (lmc/pred/src/EnergyUtility.cpp:393-581): singlets of the centre sites, then
// pairs (labels 1-3) and triplets (labels 4-7) that contain a centre site.
std::vector<StateCluster> StateClusters(const std::vector<I3> &sorted, const std::vector<int> &centers) {
  auto is_center = [&](int k) { return std::find(centers.begin(), centers.end(), k) != centers.end(); };
  std::vector<StateCluster> by_label[8];
  const int m = static_cast<int>(sorted.size());
  for (int i1 = 0; i1 < m; ++i1) {
    if (is_center(i1)) by_label[0].push_back({0, {i1, -1, -1}, 1});
    for (int i2 = 0; i2 < i1; ++i2) {
      const bool c12 = is_center(i1) || is_center(i2);
      if (c12) {
        const int l = DistanceLabel(sorted[i1] - sorted[i2]);
        if (l < 1) continue;  // the reference skips the triplet loop here too
        by_label[l].push_back({l, {i1, i2, -1}, 2});
      }
      for (int i3 = 0; i3 < i2; ++i3) {
        if (!(c12 || is_center(i3))) continue;
        const int l = TripletLabel(sorted[i1], sorted[i2], sorted[i3]);
        if (l >= 4) by_label[l].push_back({l, {i1, i2, i3}, 3});
      }
    }
  }
  std::vector<StateCluster> out;
  for (auto &v : by_label) out.insert(out.end(), v.begin(), v.end());
  return out;
}

// Orbit construction of GetAverageClusterParametersMapping{MMM,MM2}
// (EnergyUtility.cpp:106-259): singlet orbits then 1NN / 2NN / 3NN pair orbits,
// each sorted by the group keys of the cluster's sites.
template <typename GroupKey>
EnvEncoding BuildEnv(const std::vector<I3> &sorted, GroupKey key) {
  EnvEncoding enc;
  const int m = static_cast<int>(sorted.size());
  using K1 = decltype(key(0));
  // singlets
  {
    std::map<K1, std::vector<int>> groups;
    for (int k = 0; k < m; ++k) groups[key(k)].push_back(k);
    for (auto &g : groups) {
      EnvOrbit o{0, static_cast<int>(g.second.size()), static_cast<int>(enc.clusters.size())};
      for (int k : g.second) enc.clusters.push_back({k, -1, static_cast<int>(enc.orbits.size()), 0});
      enc.orbits.push_back(o);
    }
  }
  for (int label = 1; label <= 3; ++label) {
    std::map<std::pair<K1, K1>, std::vector<std::pair<int, int>>> groups;
    for (int i1 = 0; i1 < m; ++i1)
      for (int i2 = 0; i2 < i1; ++i2)
        if (DistanceLabel(sorted[i1] - sorted[i2]) == label) groups[{key(i2), key(i1)}].push_back({i2, i1});
    for (auto &g : groups) {
      const int mode = g.first.first == g.first.second ? 2 : 1;
      EnvOrbit o{mode, static_cast<int>(g.second.size()), static_cast<int>(enc.clusters.size())};
      for (auto &ab : g.second) enc.clusters.push_back({ab.first, ab.second, static_cast<int>(enc.orbits.size()), mode});
      enc.orbits.push_back(o);
    }
  }
  return enc;
}

PairTables Build() {
  PairTables t;
  const auto &nn1 = ShellOffsets(1);
  for (int di = 0; di < kDirections; ++di) {
    const I3 d = nn1[di];
    t.dir[di] = d;
    // Vertical vector: the first perpendicular 1NN in id order of an interior
    // site (Config.cpp:247-264), i.e. the lexicographically smaller one.
    bool found = false;
    for (const auto &v : nn1)
      if (Dot(v, d) == 0) { t.vert[di] = v; found = true; break; }
    if (!found) throw std::logic_error("no perpendicular 1NN direction");
    const I3 v = t.vert[di];
    std::vector<I3> set = PairSet(d);
    if (set.size() != kStateSites) throw std::logic_error("pair neighbourhood is not 60 sites");
    auto rot = [&](I3 s) { return Rotate(s, d, v); };
    std::vector<I3> state = set;
    std::sort(state.begin(), state.end(), [&](I3 a, I3 b) {
      const Rot ra = rot(a), rb = rot(b);
      return std::tie(ra.x, ra.y, ra.z) < std::tie(rb.x, rb.y, rb.z);
    });
    std::vector<I3> env;
    for (const auto &s : set)
      if (!(s == I3{0, 0, 0}) && !(s == d)) env.push_back(s);
    std::vector<I3> mmm = env, mm2 = env;
    std::sort(mmm.begin(), mmm.end(), [&](I3 a, I3 b) {
      const Rot ra = rot(a), rb = rot(b);
      const int ax = std::abs(ra.x), bx = std::abs(rb.x);
      return std::tie(ra.n2, ax, ra.x, ra.y, ra.z) < std::tie(rb.n2, bx, rb.x, rb.y, rb.z);
    });
    std::sort(mm2.begin(), mm2.end(), [&](I3 a, I3 b) {
      const Rot ra = rot(a), rb = rot(b);
      return std::tie(ra.n2, ra.x, ra.y, ra.z) < std::tie(rb.n2, rb.x, rb.y, rb.z);
    });
    for (int k = 0; k < kStateSites; ++k) t.state_off[di][k] = state[k];
    for (int k = 0; k < kEnvSites; ++k) {
      t.mmm_off[di][k] = mmm[k];
      t.mm2_off[di][k] = mm2[k];
    }
    if (di == 0) {
      for (int k = 0; k < kStateSites; ++k) {
        if (state[k] == I3{0, 0, 0}) t.pos_first = k;
        if (state[k] == d) t.pos_second = k;
      }
      t.state_clusters = StateClusters(state, {t.pos_first, t.pos_second});
      t.mmm = BuildEnv(mmm, [&](int k) {
        const Rot r = rot(mmm[k]);
        return std::make_pair(r.n2, std::abs(r.x));
      });
      t.mm2 = BuildEnv(mm2, [&](int k) {
        const Rot r = rot(mm2[k]);
        return std::make_pair(r.n2, r.x);
      });
    }
  }
  // All frames must see the same rotated point set in the same sorted order.
  for (int di = 1; di < kDirections; ++di)
    for (int k = 0; k < kStateSites; ++k) {
      const Rot a = Rotate(t.state_off[0][k], t.dir[0], t.vert[0]);
      const Rot b = Rotate(t.state_off[di][k], t.dir[di], t.vert[di]);
      if (a.n2 != b.n2 || a.x != b.x || a.y != b.y || a.z != b.z)
        throw std::logic_error("pair frames are not equivalent");
    }
  // Site list: GetSortedLatticeVectorStateOfSite (no rotation), x/y/z order.
  std::vector<I3> site{I3{0, 0, 0}};
  for (int shell = 1; shell <= 3; ++shell)
    for (const auto &s : ShellOffsets(shell)) site.push_back(s);
  std::sort(site.begin(), site.end(), LexLess);
  for (int k = 0; k < kSiteSites; ++k) {
    t.site_off[k] = site[k];
    if (site[k] == I3{0, 0, 0}) t.site_center = k;
  }
  t.site_clusters = StateClusters(site, {t.site_center});
  // Census triplets in the loop order of EnergyPredictor::GetEncode.
  auto in_shell = [](I3 s, int shell) { return DistanceLabel(s) == shell; };
  for (const auto &s2 : nn1) {
    for (const auto &t1 : nn1) {
      const I3 s3 = s2 + t1;
      if (in_shell(s3, 1)) t.census_triplets.push_back({s2, s3, 4});
      else if (in_shell(s3, 2)) t.census_triplets.push_back({s2, s3, 5});
      else if (in_shell(s3, 3)) t.census_triplets.push_back({s2, s3, 6});
    }
    for (const auto &t2 : ShellOffsets(2)) {
      const I3 s3 = s2 + t2;
      if (in_shell(s3, 3)) t.census_triplets.push_back({s2, s3, 7});
    }
  }
  return t;
}

}  // namespace

const std::vector<I3> &ShellOffsets(int shell) {
  static const std::vector<I3> s1 = MakeShell(2), s2 = MakeShell(4), s3 = MakeShell(6);
  if (shell == 1) return s1;
  if (shell == 2) return s2;
  if (shell == 3) return s3;
  throw std::invalid_argument("shell must be 1, 2 or 3");
}

int DistanceLabel(I3 s) {
  if (((s.x + s.y + s.z) & 1) != 0) return -1;
  switch (Norm2(s)) {
    case 2: return 1;
    case 4: return 2;
    case 6: return 3;
    default: return -1;
  }
}

std::vector<int64_t> SortedNeighbors(const Fcc &fcc, int64_t id, int shell) {
  const I3 h = fcc.Coord(id);
  std::vector<int64_t> out;
  for (const auto &s : ShellOffsets(shell)) out.push_back(fcc.Id(fcc.Wrap(h + s)));
  std::sort(out.begin(), out.end());
  return out;
}

std::vector<int> EnvEncoding::OrbitOffsets(int e) const {
  std::vector<int> off;
  int acc = 0;
  for (const auto &o : orbits) {
    off.push_back(acc);
    acc += o.mode == 0 ? e : (o.mode == 1 ? e * e : e * (e + 1) / 2);
  }
  off.push_back(acc);
  return off;
}

int EnvEncoding::NumFeatures(int e) const { return OrbitOffsets(e).back(); }

const PairTables &GetPairTables() {
  static const PairTables tables = Build();
  return tables;
}

int DirectionIndex(I3 d) {
  const auto &nn1 = ShellOffsets(1);
  for (int i = 0; i < kDirections; ++i)
    if (nn1[i] == d) return i;
  return -1;
}

}  // namespace lmc
