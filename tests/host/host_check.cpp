// Test driver for the C++ host mirror (lmc_host.hpp), used by tests/test_host.py.
//   host_check cfg-roundtrip <dir>              CFG write/read (plain and gzip) with atom tracking
//   host_check map-write <cfg> <dir>            Config::WriteLattice / WriteElement / WriteMap of a CFG
//   host_check map-read <dir> <cfg>             Config::ReadMap of <dir>'s map files against the CFG
//   host_check element-order <e1,e2,...>         the names in std::set<Element> iteration order
//   host_check param <file>                     parsed api::Parameter keys
//   host_check param-analysis <file>            the analysis / schedule keys of api::Parameter
//   host_check predict <json> <cfg> <elements,comma> <m> <a b> x m <a b> ...
//                                               Ea dE (Quartic) and Ea (E0) for the m jump pairs, swap dE
//                                               for the remaining pairs, then the energy
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <sstream>
#include <string>

#include "lmc_host.hpp"

static int Fail(const std::string &m) {
  std::cerr << "FAIL " << m << std::endl;
  return 1;
}

int main(int argc, char **argv) {
  if (argc < 3) return Fail("usage");
  const std::string cmd = argv[1];
  try {
    if (cmd == "cfg-roundtrip") {
      const std::string dir = argv[2];
      cfg::Config c = cfg::Config::GenerateFCC(8, Element("Al"));
      c.SetElementAtLatticeId(0, Element("X"));
      c.SetElementAtLatticeId(5, Element("Mg"));
      c.SetElementAtLatticeId(700, Element("Zn"));
      // walk the vacancy across the periodic boundary a few times
      size_t vac = 0;
      for (int s = 0; s < 40; ++s) {
        const auto nb = c.GetNeighborLatticeIdVector(vac, 1);
        const size_t to = nb[(s * 7) % 12];
        c.LatticeJump({vac, to});
        vac = to;
      }
      for (const std::string name : {dir + "/a.cfg", dir + "/a.cfg.gz"}) {
        c.WriteConfig(name);
        const cfg::Config r = cfg::Config::ReadConfig(name);
        if (r.GetNumAtoms() != c.GetNumAtoms()) return Fail("atom count");
        for (size_t id = 0; id < c.GetNumLattices(); ++id) {
          if (r.GetElementAtLatticeId(id) != c.GetElementAtLatticeId(id)) return Fail("element at " + std::to_string(id));
          if (r.GetAtomIdFromLatticeId(id) != c.GetAtomIdFromLatticeId(id)) return Fail("atom id at " + std::to_string(id));
          const auto a = r.GetUnwrappedCartesianPositionOfLattice(id), b = c.GetUnwrappedCartesianPositionOfLattice(id);
          for (int d = 0; d < 3; ++d)
            if (std::abs(a[d] - b[d]) > 1e-9) return Fail("unwrapped position at " + std::to_string(id));
        }
        if (r.GetVacancyLatticeId() != vac) return Fail("vacancy");
      }
      const auto u = c.GetUnwrappedCartesianPositionOfLattice(vac);
      std::cout.precision(17);
      std::cout << "OK " << vac << ' ' << u[0] << ' ' << u[1] << ' ' << u[2] << ' '
                << c.GetSolventElement().GetString() << std::endl;
      return 0;
    }
    if (cmd == "map-write" && argc == 4) {
      cfg::Config c = cfg::Config::ReadConfig(argv[2]);
      c.ReassignLatticeVector();
      const std::string dir = argv[3];
      c.WriteLattice(dir + "/lattice.txt");
      c.WriteElement(dir + "/element.txt");
      c.WriteMap(dir + "/map.txt");
      std::cout << "OK" << std::endl;
      return 0;
    }
    if (cmd == "map-read" && argc == 4) {
      const std::string dir = argv[2];
      const cfg::Config m = cfg::Config::ReadMap(dir + "/lattice.txt", dir + "/element.txt", dir + "/map.txt");
      const cfg::Config c = cfg::Config::ReadConfig(argv[3]);
      if (m.GetNumAtoms() != c.GetNumAtoms()) return Fail("atom count");
      for (size_t id = 0; id < c.GetNumLattices(); ++id) {
        if (m.GetElementAtLatticeId(id) != c.GetElementAtLatticeId(id)) return Fail("element at " + std::to_string(id));
        if (m.GetAtomIdFromLatticeId(id) != c.GetAtomIdFromLatticeId(id)) return Fail("atom id at " + std::to_string(id));
      }
      std::cout << "OK " << m.GetVacancyLatticeId() << std::endl;
      return 0;
    }
    if (cmd == "param") {
      const api::Parameter p(argv[2]);
      std::cout << p.method << '|' << p.config_filename_ << '|' << p.json_coefficients_filename_ << '|'
                << p.log_dump_steps_ << '|' << p.config_dump_steps_ << '|' << p.maximum_steps_ << '|' << p.temperature_
                << '|' << p.rate_corrector_ << p.early_stop_ << p.solute_disp_ << '|' << p.seed_ << '|';
      for (const auto &e : p.element_set_) std::cout << e << ',';
      std::cout << std::endl;
      return 0;
    }
    if (cmd == "param-analysis") {
      const api::Parameter p(argv[2]);
      std::cout << p.initial_steps_ << '|' << p.increment_steps_ << '|' << p.smallest_cluster_criteria_ << '|'
                << p.solvent_bond_criteria_ << '|' << p.escape_temperature_ << '|' << p.decrement_temperature_ << '|'
                << p.early_stop_steps_ << '|' << p.map_filename_ << std::endl;
      return 0;
    }
    if (cmd == "element-order") {
      std::set<Element> els;
      std::stringstream ss(argv[2]);
      std::string e;
      while (std::getline(ss, e, ',')) els.insert(Element(e));
      for (const auto &el : els) std::cout << el.GetString() << ' ';
      std::cout << std::endl;
      return 0;
    }
    if (cmd == "predict") {
      if (argc < 7) return Fail("usage");
      std::set<Element> els;
      std::stringstream ss(argv[4]);
      std::string e;
      while (std::getline(ss, e, ',')) els.insert(Element(e));
      const cfg::Config c = cfg::Config::ReadConfig(argv[3]);
      const pred::VacancyMigrationPredictorQuarticLru quartic(argv[2], c, els, 100000);
      const pred::VacancyMigrationPredictorE0 e0(argv[2], c, els);
      const pred::EnergyChangePredictorPairSite pair_site(argv[2], c, els);
      const pred::EnergyPredictor energy(argv[2], els);
      std::cout.precision(17);
      const int jumps = std::atoi(argv[5]);
      for (int i = 6, k = 0; i + 1 < argc; i += 2, ++k) {
        const std::pair<size_t, size_t> p{std::strtoull(argv[i], nullptr, 10), std::strtoull(argv[i + 1], nullptr, 10)};
        if (k < jumps) {
          const auto q = quartic.GetBarrierAndDiffFromLatticeIdPair(c, p);
          const auto z = e0.GetBarrierAndDiffFromLatticeIdPair(c, p);
          std::cout << q.first << ' ' << q.second << ' ' << z.first << '\n';
        } else {
          std::cout << pair_site.GetDeFromLatticeIdPair(c, p) << '\n';
        }
      }
      // a non-neighbour pair is out of range for the barrier predictor, as GetPairFlatIndex
      try {
        (void)quartic.GetBarrierAndDiffFromLatticeIdPair(c, {0, c.GetNumLattices() / 2});
        std::cout << "no exception\n";
      } catch (const std::out_of_range &) {
        std::cout << "out_of_range\n";
      }
      std::cout << energy.GetEnergy(c) << std::endl;
      return 0;
    }
  } catch (const std::exception &ex) {
    std::cout << "EXCEPTION " << ex.what() << std::endl;
    return 2;
  }
  return Fail("unknown command");
}
