// Host-side FCC geometry and cluster tables for the lattice-MC hot path.
//
// Everything here is exact integer geometry on a perfect cubic FCC supercell
// of n x n x n conventional cells. Sites are addressed by half-lattice
// coordinates h = (hx, hy, hz), each in [0, 2n), with hx + hy + hz even.
//
// Lattice ids follow the order the reference assigns after
// Config::ReassignLatticeVector (lmc/cfg/src/Config.cpp:466-552): sites sorted
// by fractional x, then y, then z. In half-lattice units that order is the
// closed form  id = hx * 2n^2 + hy * n + floor(hz / 2).
//
// The pair-neighbourhood orders (state / MMM / MM2 sorted site lists,
// lmc/pred/src/EnergyUtility.cpp:45-104,261-287) are computed once in the
// rotated pair frame with integer keys: quarter-unit coordinates
// q = 2 s - d relative to the pair centre, projected on (d, v, d x v). For
// n <= 49 every comparison the reference makes with its 1e-4 tolerance on
// fractional coordinates (lmc/cfg/include/LatticeCluster.hpp:62-154) has a gap
// larger than the tolerance, so the integer keys reproduce its order exactly;
// for n >= 50 the reference's tolerance merges distinct shells and this module
// keeps the well-separated layout instead.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace lmc {

struct I3 {
  int x{0}, y{0}, z{0};
};
inline I3 operator+(I3 a, I3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline I3 operator-(I3 a, I3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline I3 operator*(int k, I3 a) { return {k * a.x, k * a.y, k * a.z}; }
inline bool operator==(I3 a, I3 b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
inline int Dot(I3 a, I3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline int Norm2(I3 a) { return Dot(a, a); }
inline I3 Cross(I3 a, I3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }

// Closed-form FCC indexing for a cubic n^3 supercell.
struct Fcc {
  int n{0};
  int64_t NumSites() const { return 4LL * n * n * n; }
  I3 Wrap(I3 h) const {
    const int m = 2 * n;
    auto w = [m](int v) { v %= m; return v < 0 ? v + m : v; };
    return {w(h.x), w(h.y), w(h.z)};
  }
  int64_t Id(I3 h) const { return static_cast<int64_t>(h.x) * 2 * n * n + static_cast<int64_t>(h.y) * n + h.z / 2; }
  I3 Coord(int64_t id) const {
    const int64_t plane = 2LL * n * n;
    const int hx = static_cast<int>(id / plane);
    const int64_t r = id % plane;
    const int hy = static_cast<int>(r / n);
    const int k = static_cast<int>(r % n);
    return {hx, hy, 2 * k + ((hx + hy) & 1)};
  }
};

// Shell offsets in half-lattice units: shell 1 (|s|^2 = 2, 12 sites),
// shell 2 (|s|^2 = 4, 6 sites), shell 3 (|s|^2 = 6, 24 sites).
const std::vector<I3> &ShellOffsets(int shell);
// Distance label of a half-unit offset: 1, 2, 3 for the first three shells,
// -1 otherwise (the reference's FindDistanceLabelBetweenLattice, Config.cpp:354-371).
int DistanceLabel(I3 s);
// Neighbour ids of `id` in shell 1/2/3, each shell sorted by id (Config.cpp:1037-1044).
std::vector<int64_t> SortedNeighbors(const Fcc &fcc, int64_t id, int shell);

constexpr int kStateSites = 60;  // 1-3NN set of a 1NN pair including the pair
constexpr int kEnvSites = 58;    // same set without the pair
constexpr int kSiteSites = 43;   // 1-3NN set of a single site including it
constexpr int kDirections = 12;

// A cluster of the pair/site state lists: label 0..7 and up to three indices
// into the sorted list (unused slots are 0xFF).
struct StateCluster {
  int label;
  int idx[3];
  int size;
};

// A cluster of the MMM / MM2 symmetric-orbit encodings.
struct EnvCluster {
  int a, b;      // sorted-list indices; b = -1 for singlets
  int orbit;     // orbit index in mapping order
  int mode;      // 0 singlet, 1 ordered pair, 2 symmetric pair
};
struct EnvOrbit {
  int mode;      // 0 singlet, 1 ordered pair, 2 symmetric pair
  int size;      // clusters in the orbit
  int first;     // first cluster index in the cluster array
};

struct EnvEncoding {
  std::vector<EnvCluster> clusters;  // grouped by orbit, orbits in mapping order
  std::vector<EnvOrbit> orbits;
  // Feature layout for an alphabet of e one-hot elements.
  std::vector<int> OrbitOffsets(int e) const;
  int NumFeatures(int e) const;
};

// Translation-invariant pair and site tables.
struct PairTables {
  I3 dir[kDirections];                          // 1NN directions d (half units)
  I3 vert[kDirections];                         // frame vertical vector v for each d
  I3 state_off[kDirections][kStateSites];       // offsets from pair origin, state order
  I3 mmm_off[kDirections][kEnvSites];           // MMM order
  I3 mm2_off[kDirections][kEnvSites];           // MM2 order
  int pos_first{-1}, pos_second{-1};            // state-list positions of the pair sites
  std::vector<StateCluster> state_clusters;     // GetClusterParametersMappingStatePair
  EnvEncoding mmm, mm2;                         // GetAverageClusterParametersMapping{MMM,MM2}
  I3 site_off[kSiteSites];                      // GetSortedLatticeVectorStateOfSite order
  int site_center{-1};
  std::vector<StateCluster> site_clusters;      // GetClusterParametersMappingStateSite
  // EnergyPredictor census enumerations per site (EnergyPredictor.cpp:40-96):
  // triplets (s2, s3, label) with the centre as the first site.
  struct CensusTriplet { I3 s2, s3; int label; };
  std::vector<CensusTriplet> census_triplets;
};

// Builds the tables (deterministic; independent of n and of the element set).
const PairTables &GetPairTables();
// Direction index of a 1NN offset, or -1.
int DirectionIndex(I3 d);

}  // namespace lmc
