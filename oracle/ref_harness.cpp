// Test-infrastructure harness around the reference's own hot-path classes
// (compiled unmodified from the reference sources against the shim headers in
// oracle/ref_shim). It builds a perfect FCC supercell with
// cfg::GenerateFCC + Config::ReassignLatticeVector (the id order of the
// parameter-file path, lmc/api/src/Home.cpp:166-167), assigns species per
// lattice id from a text file, and prints the reference's results as plain
// text lines that tests/golden/make_golden.py turns into fixtures.
//
// Commands (all outputs go to stdout):
//   geom   <n> <pairs_file>
//       neighbour lists of every site, sorted state/MMM/MM2 id lists for the
//       listed pairs, sorted state list of site 0, and the cluster mappings
//       (lmc/pred/src/EnergyUtility.cpp:169-259,393-581).
//   pred   <n> <species_file> <json> <elements> <pairs_file>
//       per pair: Quartic {Ea, dE, D, Ks} (VacancyMigrationPredictorQuartic.cpp:112-276),
//       the integer state counts behind GetDe, the MMM / MM2 one-hot numerators
//       (EnergyUtility.cpp:743-796), E0 {Ea, dE} (VacancyMigrationPredictorE0.cpp:128-159),
//       PairSite dE (EnergyChangePredictorPairSite.cpp:69-192); plus the
//       EnergyPredictor census counts and energy (EnergyPredictor.cpp:40-96,173-177).
//   kmc    <n> <species_file> <json> <elements> <T> <seed> <steps> <detail_steps>
//       KineticMcFirstOmp trajectory with std::mt19937_64 seeded by <seed>
//       (lmc/mc/src/KineticMcAbstract.cpp:140-182, KineticMcFirstOmp.cpp:52-82).
//   cmc    <n> <species_file> <json> <elements> <T> <seed> <max_steps>
//       CanonicalMcOmp run (batch = OMP thread count) with the seeded generator
//       (lmc/mc/src/CanonicalMcOmp.cpp:40-92); prints per-step energies
//       read back from cmc_log.txt and the final lattice.
//   cluster <n> <species_file> <json> <elements> <solvent> <lists_file>
//       per line of lists_file (lattice ids of one cluster): EnergyPredictor::GetEnergyOfCluster
//       on the lattice, on the solvent lattice carrying the listed sites' species (the solute_config
//       of SoluteCluster::GetFormationEnergy) and on the pure solvent lattice (EnergyPredictor.cpp:
//       97-184, SoluteCluster.cpp:395-410); then GetChemicalPotential(solvent) (EnergyPredictor.cpp:
//       196-214).
//   sitede <n> <species_file> <json> <elements> <queries_file>
//       per line "lattice_id from to" of queries_file: the site set to `from`, then
//       EnergyChangePredictorPairSite::GetDeFromAtomIdSite(config, atom, to)
//       (EnergyChangePredictorPairSite.cpp:148-192), the site restored.
//   writemap <n> <species_file> <outdir>
//       the configuration written by Config::WriteConfig (start.cfg) and by WriteLattice /
//       WriteElement / WriteMap (lattice.txt, element.txt, map.txt; Config.cpp:651-692,887-922).
//   rng    <seed> <count> <range>
//       raw mt19937_64 outputs, uniform_real_distribution<double>(0,1) and
//       uniform_int_distribution<size_t>(0, range-1) draws from libstdc++.
#include <cmath>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <random>
#include <set>
#include <sstream>
#include <string>
#include <vector>

#include "CanonicalMcOmp.h"
#include "Config.h"
#include "EnergyChangePredictorPairSite.h"
#include "EnergyPredictor.h"
#include "EnergyUtility.h"
#include "KineticMcFirstOmp.h"
#include "VacancyMigrationPredictorE0.h"
#include "VacancyMigrationPredictorQuartic.h"

namespace {

cfg::Config MakeConfig(size_t n) {
  auto config = cfg::GenerateFCC({n, n, n}, Element("Al"));
  config.ReassignLatticeVector();
  return config;
}

void LoadSpecies(cfg::Config &config, const std::string &path) {
  std::ifstream ifs(path);
  if (!ifs) throw std::runtime_error("cannot open " + path);
  std::string name;
  for (size_t l = 0; l < config.GetNumAtoms(); ++l) {
    if (!(ifs >> name)) throw std::runtime_error("species file too short");
    config.SetAtomElementTypeAtLattice(l, Element(name));
  }
}

std::set<Element> ParseElements(const std::string &csv) {
  std::set<Element> s;
  std::stringstream ss(csv);
  std::string tok;
  while (std::getline(ss, tok, ',')) s.insert(Element(tok));
  return s;
}

std::vector<std::pair<size_t, size_t>> LoadPairs(const std::string &path) {
  std::ifstream ifs(path);
  if (!ifs) throw std::runtime_error("cannot open " + path);
  std::vector<std::pair<size_t, size_t>> pairs;
  size_t a, b;
  while (ifs >> a >> b) pairs.emplace_back(a, b);
  return pairs;
}

template <typename V>
void PrintList(const char *key, const V &v) {
  std::cout << key;
  for (const auto &x : v) std::cout << ' ' << x;
  std::cout << '\n';
}

void PrintMapping(const char *key, const std::vector<std::vector<std::vector<size_t>>> &m) {
  // one line per orbit: "<key> <orbit> <cluster0 indices , ...>" (SIZE_MAX shown as -1)
  for (size_t o = 0; o < m.size(); ++o) {
    std::cout << key << ' ' << o;
    for (const auto &cl : m[o]) {
      std::cout << " |";
      for (auto idx : cl) {
        if (idx == SIZE_MAX) std::cout << " -1";
        else std::cout << ' ' << idx;
      }
    }
    std::cout << '\n';
  }
}

std::vector<size_t> Ids(const std::vector<cfg::Lattice> &v) {
  std::vector<size_t> out;
  for (const auto &l : v) out.push_back(l.GetId());
  return out;
}

// Exposes the protected pieces of the Quartic predictor.
class QuarticProbe : public pred::VacancyMigrationPredictorQuartic {
 public:
  using VacancyMigrationPredictorQuartic::VacancyMigrationPredictorQuartic;
  double De(const cfg::Config &c, const std::pair<size_t, size_t> &p) const { return GetDe(c, p); }
  double D(const cfg::Config &c, const std::pair<size_t, size_t> &p) const { return GetD(c, p); }
  double Ks(const cfg::Config &c, const std::pair<size_t, size_t> &p) const { return GetKs(c, p); }
  const std::vector<std::vector<std::vector<size_t>>> &Mmm() const { return mapping_mmm_; }
  const std::vector<std::vector<std::vector<size_t>>> &Mm2() const { return mapping_mm2_; }
  const std::set<Element> &Elements() const { return element_set_; }
  const std::unordered_map<std::string, std::vector<double>> &OneHot() const { return one_hot_encode_hash_map_; }
};

int CmdGeom(size_t n, const std::string &pairs_file) {
  auto config = MakeConfig(n);
  std::cout.precision(17);
  for (size_t l = 0; l < config.GetNumAtoms(); ++l) {
    std::cout << "nn " << l;
    for (auto x : config.GetFirstNeighborsAdjacencyList()[l]) std::cout << ' ' << x;
    for (auto x : config.GetSecondNeighborsAdjacencyList()[l]) std::cout << ' ' << x;
    for (auto x : config.GetThirdNeighborsAdjacencyList()[l]) std::cout << ' ' << x;
    const auto &p = config.GetLatticeVector()[l].GetRelativePosition();
    std::cout << " pos " << p[0] << ' ' << p[1] << ' ' << p[2] << '\n';
  }
  for (const auto &pr : LoadPairs(pairs_file)) {
    std::cout << "pair " << pr.first << ' ' << pr.second << '\n';
    PrintList("state", Ids(pred::GetSortedLatticeVectorStateOfPair(config, pr)));
    PrintList("mmm", Ids(pred::GetSymmetricallySortedLatticeVectorMMM(config, pr)));
    PrintList("mm2", Ids(pred::GetSymmetricallySortedLatticeVectorMM2(config, pr)));
  }
  PrintList("site0", Ids(pred::GetSortedLatticeVectorStateOfSite(config, 0)));
  PrintMapping("map_state", pred::GetClusterParametersMappingStatePair(config));
  PrintMapping("map_site", pred::GetClusterParametersMappingStateSite(config));
  PrintMapping("map_mmm", pred::GetAverageClusterParametersMappingMMM(config));
  PrintMapping("map_mm2", pred::GetAverageClusterParametersMappingMM2(config));
  return 0;
}

int CmdPred(size_t n, const std::string &species, const std::string &json, const std::string &elements,
            const std::string &pairs_file) {
  auto config = MakeConfig(n);
  LoadSpecies(config, species);
  const auto element_set = ParseElements(elements);
  const QuarticProbe quartic(json, config, element_set);
  const pred::VacancyMigrationPredictorE0 e0(json, config, element_set);
  const pred::EnergyChangePredictorPairSite pair_site(json, config, element_set);
  const pred::EnergyPredictor energy(json, element_set);
  std::cout.precision(17);
  const size_t n_elem = element_set.size();
  for (const auto &pr : LoadPairs(pairs_file)) {
    std::cout << "pair " << pr.first << ' ' << pr.second << '\n';
    const bool nn1 = config.FindDistanceLabelBetweenLattice(pr.first, pr.second) == 1;
    // Only evaluated for first-neighbour pairs: GetLatticePairCenter
    // (Config.cpp:228-245) never terminates when a coordinate separation is
    // exactly half the box, which non-neighbour pairs can hit.
    const bool encodable = nn1 && [&] {
      // The Quartic/E0 encoders have no one-hot slot for X outside the pair.
      for (auto id : Ids(pred::GetSymmetricallySortedLatticeVectorMMM(config, pr)))
        if (config.GetElementAtLatticeId(id) == ElementName::X) return false;
      return true;
    }();
    if (nn1 && encodable) {
      const auto ea_de = quartic.GetBarrierAndDiffFromLatticeIdPair(config, pr);
      const double de = quartic.De(config, pr);
      const auto start = pred::GetThreadLocalStartCountsBuffer();
      const auto end = pred::GetThreadLocalEndCountsBuffer();
      std::cout << "quartic " << ea_de.first << ' ' << ea_de.second << ' ' << quartic.D(config, pr) << ' '
                << quartic.Ks(config, pr) << ' ' << de << '\n';
      PrintList("state_start", start);
      PrintList("state_end", end);
      std::vector<Element> ev;
      std::vector<double> enc;
      for (auto id : Ids(pred::GetSymmetricallySortedLatticeVectorMMM(config, pr)))
        ev.push_back(config.GetElementAtLatticeId(id));
      pred::GetOneHotParametersFromMap(ev, quartic.OneHot(), n_elem, quartic.Mmm(), enc);
      PrintList("enc_mmm", enc);
      ev.clear();
      for (auto id : Ids(pred::GetSymmetricallySortedLatticeVectorMM2(config, pr)))
        ev.push_back(config.GetElementAtLatticeId(id));
      pred::GetOneHotParametersFromMap(ev, quartic.OneHot(), n_elem, quartic.Mm2(), enc);
      PrintList("enc_mm2_fwd", enc);
      ev.clear();
      for (auto id : Ids(pred::GetSymmetricallySortedLatticeVectorMM2(config, {pr.second, pr.first})))
        ev.push_back(config.GetElementAtLatticeId(id));
      pred::GetOneHotParametersFromMap(ev, quartic.OneHot(), n_elem, quartic.Mm2(), enc);
      PrintList("enc_mm2_bwd", enc);
      const auto e0r = e0.GetBarrierAndDiffFromLatticeIdPair(config, pr);
      std::cout << "e0 " << e0r.first << ' ' << e0r.second << '\n';
    }
    std::cout << "pairsite " << pair_site.GetDeFromLatticeIdPair(config, pr) << '\n';
  }
  const auto enc = energy.GetEncode(config);
  PrintList("census_encode", enc);
  std::cout << "energy " << energy.GetEnergy(config) << '\n';
  return 0;
}

class KmcProbe : public mc::KineticMcFirstOmp {
 public:
  using KineticMcFirstOmp::KineticMcFirstOmp;
  void Seed(unsigned long long s) { generator_.seed(s); }
  void Step(bool detail) {
    const size_t vac = vacancy_lattice_id_;
    OneStepSimulation();
    size_t sel = 0;
    for (size_t i = 0; i < event_k_i_list_.size(); ++i)
      if (event_k_i_list_[i].GetIdJumpPair() == event_k_i_.GetIdJumpPair()) sel = i;
    std::cout << "step " << steps_ << ' ' << vac << ' ' << event_k_i_.GetIdJumpPair().second << ' ' << sel << ' '
              << event_k_i_.GetForwardBarrier() << ' ' << event_k_i_.GetEnergyChange() << ' ' << total_rate_k_ << ' '
              << time_ << ' ' << energy_ << '\n';
    if (detail) {
      std::cout << "events";
      for (const auto &e : event_k_i_list_)
        std::cout << ' ' << e.GetIdJumpPair().second << ' ' << e.GetForwardBarrier() << ' ' << e.GetEnergyChange();
      std::cout << '\n';
    }
  }
  double AbsoluteEnergy() const { return absolute_energy_; }
};

int CmdKmc(size_t n, const std::string &species, const std::string &json, const std::string &elements, double T,
           unsigned long long seed, size_t steps, size_t detail_steps) {
  auto config = MakeConfig(n);
  LoadSpecies(config, species);
  KmcProbe kmc(config, 1000000000000ULL, 1000000000000000ULL, 1000000000000000ULL, 0, 0, 0.0, 0.0, T,
               ParseElements(elements), json, "", false, false, false);
  kmc.Seed(seed);
  std::cout.precision(17);
  std::cout << "absolute_energy " << kmc.AbsoluteEnergy() << '\n';
  for (size_t s = 0; s < steps; ++s) kmc.Step(s < detail_steps);
  return 0;
}

class CmcProbe : public mc::CanonicalMcOmp {
 public:
  using CanonicalMcOmp::CanonicalMcOmp;
  void Seed(unsigned long long s) { generator_.seed(s); }
  const cfg::Config &Cfg() const { return config_; }
  unsigned long long Steps() const { return steps_; }
  double Energy() const { return energy_; }
  double AbsoluteEnergy() const { return absolute_energy_; }
};

int CmdCmc(size_t n, const std::string &species, const std::string &json, const std::string &elements, double T,
           unsigned long long seed, unsigned long long max_steps) {
  auto config = MakeConfig(n);
  LoadSpecies(config, species);
  double e_abs0 = 0.0;
  std::vector<std::string> final_species;
  unsigned long long final_steps = 0;
  double final_energy = 0.0, final_abs = 0.0;
  {
    CmcProbe cmc(config, 1, 1000000000000000ULL, max_steps, 0, 0, 0.0, T, ParseElements(elements), json);
    cmc.Seed(seed);
    e_abs0 = cmc.AbsoluteEnergy();
    cmc.Simulate();
    for (size_t l = 0; l < cmc.Cfg().GetNumAtoms(); ++l)
      final_species.push_back(cmc.Cfg().GetElementAtLatticeId(l).GetString());
    final_steps = cmc.Steps();
    final_energy = cmc.Energy();
    final_abs = cmc.AbsoluteEnergy();
  }
  std::cout.precision(17);
  std::cout << "absolute_energy0 " << e_abs0 << '\n';
  std::cout << "final_steps " << final_steps << '\n';
  std::cout << "final_energy " << final_energy << ' ' << final_abs << '\n';
  PrintList("final_species", final_species);
  std::ifstream log("cmc_log.txt");
  std::string line;
  std::getline(log, line);  // header
  while (std::getline(log, line)) std::cout << "log " << line << '\n';
  return 0;
}

int CmdRng(unsigned long long seed, size_t count, size_t range) {
  std::mt19937_64 g(seed);
  std::cout.precision(17);
  std::cout << "raw";
  for (size_t i = 0; i < count; ++i) std::cout << ' ' << g();
  std::cout << '\n';
  std::uniform_real_distribution<double> u(0.0, 1.0);
  std::cout << "real";
  for (size_t i = 0; i < count; ++i) std::cout << ' ' << u(g);
  std::cout << '\n';
  std::uniform_int_distribution<size_t> d(0, range - 1);
  std::cout << "int";
  for (size_t i = 0; i < count; ++i) std::cout << ' ' << d(g);
  std::cout << '\n';
  return 0;
}
}  // namespace

int CmdCluster(size_t n, const std::string &species_file, const std::string &json, const std::string &elements,
               const std::string &solvent, const std::string &lists_file) {
  auto config = MakeConfig(n);
  LoadSpecies(config, species_file);
  const pred::EnergyPredictor energy(json, ParseElements(elements));
  const Element solvent_element(solvent);
  auto solvent_config = config;
  for (size_t a = 0; a < solvent_config.GetNumAtoms(); ++a) solvent_config.SetAtomElementTypeAtAtom(a, solvent_element);
  std::cout.precision(17);
  std::ifstream ifs(lists_file);
  if (!ifs) throw std::runtime_error("cannot open " + lists_file);
  std::string line;
  while (std::getline(ifs, line)) {
    std::stringstream ss(line);
    std::vector<size_t> atoms;
    size_t l;
    while (ss >> l) atoms.push_back(config.GetAtomIdFromLatticeId(l));
    if (atoms.empty()) continue;
    auto solute_config = solvent_config;
    for (size_t a : atoms) solute_config.SetAtomElementTypeAtAtom(a, config.GetElementAtAtomId(a));
    std::cout << "cluster " << energy.GetEnergyOfCluster(config, atoms) << ' '
              << energy.GetEnergyOfCluster(solute_config, atoms) << ' '
              << energy.GetEnergyOfCluster(solvent_config, atoms) << '\n';
  }
  for (const auto &[element, mu] : energy.GetChemicalPotential(solvent_element))
    std::cout << "mu " << element.GetString() << ' ' << mu << '\n';
  return 0;
}

int CmdSiteDe(size_t n, const std::string &species_file, const std::string &json, const std::string &elements,
              const std::string &queries_file) {
  auto config = MakeConfig(n);
  LoadSpecies(config, species_file);
  const auto element_set = ParseElements(elements);
  const pred::EnergyChangePredictorPairSite pair_site(json, config, element_set);
  std::cout.precision(17);
  std::ifstream ifs(queries_file);
  if (!ifs) throw std::runtime_error("cannot open " + queries_file);
  size_t l;
  std::string from, to;
  while (ifs >> l >> from >> to) {
    const size_t atom = config.GetAtomIdFromLatticeId(l);
    const Element keep = config.GetElementAtAtomId(atom);
    config.SetAtomElementTypeAtAtom(atom, Element(from));
    std::cout << "sitede " << pair_site.GetDeFromAtomIdSite(config, atom, Element(to)) << '\n';
    config.SetAtomElementTypeAtAtom(atom, keep);
  }
  return 0;
}

int CmdWriteMap(size_t n, const std::string &species_file, const std::string &outdir) {
  auto config = MakeConfig(n);
  LoadSpecies(config, species_file);
  config.WriteConfig(outdir + "/start.cfg");
  config.WriteLattice(outdir + "/lattice.txt");
  config.WriteElement(outdir + "/element.txt");
  config.WriteMap(outdir + "/map.txt");
  return 0;
}

int main(int argc, char **argv) {
  if (argc < 2) {
    std::cerr << "usage: ref_harness <geom|pred|kmc|cmc|rng> ...\n";
    return 2;
  }
  const std::string cmd = argv[1];
  try {
    if (cmd == "geom" && argc == 4) return CmdGeom(std::stoul(argv[2]), argv[3]);
    if (cmd == "pred" && argc == 7) return CmdPred(std::stoul(argv[2]), argv[3], argv[4], argv[5], argv[6]);
    if (cmd == "kmc" && argc == 10)
      return CmdKmc(std::stoul(argv[2]), argv[3], argv[4], argv[5], std::stod(argv[6]), std::stoull(argv[7]),
                    std::stoul(argv[8]), std::stoul(argv[9]));
    if (cmd == "cmc" && argc == 9)
      return CmdCmc(std::stoul(argv[2]), argv[3], argv[4], argv[5], std::stod(argv[6]), std::stoull(argv[7]),
                    std::stoull(argv[8]));
    if (cmd == "cluster" && argc == 8) return CmdCluster(std::stoul(argv[2]), argv[3], argv[4], argv[5], argv[6], argv[7]);
    if (cmd == "sitede" && argc == 7) return CmdSiteDe(std::stoul(argv[2]), argv[3], argv[4], argv[5], argv[6]);
    if (cmd == "writemap" && argc == 5) return CmdWriteMap(std::stoul(argv[2]), argv[3], argv[4]);
    if (cmd == "rng" && argc == 5) return CmdRng(std::stoull(argv[2]), std::stoul(argv[3]), std::stoul(argv[4]));
  } catch (const std::exception &e) {
    std::cerr << "error: " << e.what() << '\n';
    return 1;
  }
  std::cerr << "bad arguments\n";
  return 2;
}
