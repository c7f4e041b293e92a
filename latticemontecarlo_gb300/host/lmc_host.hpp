// C++ host mirror of LatticeMC's hot-path interfaces over the C ABI of
// liblmc_gb300.so: the same namespaces, class names, constructor arguments and
// method signatures as the reference, so its callers compile against this
// header unchanged, while every barrier, energy change, census and Monte Carlo
// step runs in the GB300 kernels.
//
//   Element                                   lmc/cfg/include/Element.hpp
//   cfg::Config                               lmc/cfg/include/Config.h (perfect cubic FCC supercells)
//   pred::VacancyMigrationPredictorQuartic    lmc/pred/include/VacancyMigrationPredictorQuartic.h:25-27
//   pred::VacancyMigrationPredictorQuarticLru lmc/pred/include/VacancyMigrationPredictorQuarticLru.h:16-18
//   pred::VacancyMigrationPredictorE0         lmc/pred/include/VacancyMigrationPredictorE0.h:22-24
//   pred::EnergyChangePredictorPairSite       lmc/pred/include/EnergyChangePredictorPairSite.h:22-23
//   pred::EnergyPredictor                     lmc/pred/include/EnergyPredictor.h:19
//   pred::TimeTemperatureInterpolator         lmc/pred/include/TimeTemperatureInterpolator.h
//   mc::KineticMcFirstOmp                     lmc/mc/include/KineticMcFirstOmp.h
//   mc::KineticMcChainOmpi                    lmc/mc/include/KineticMcChainOmpi.h
//   mc::CanonicalMcOmp                        lmc/mc/include/CanonicalMcOmp.h
//   api::Parameter, api::Run                  lmc/api/include/Parameter.h, Home.h
//
// Errors: C ABI status codes become the exception types the reference throws
// (std::runtime_error("Cannot open ..."), std::out_of_range, std::invalid_argument).
// Threading: predictor methods are const and may be called from several
// threads; calls on one predictor are serialised (one CUDA stream each).
#pragma once

#include <array>
#include <cstdint>
#include <deque>
#include <fstream>
#include <map>
#include <random>
#include <memory>
#include <mutex>
#include <set>
#include <string>
#include <utility>
#include <vector>

#include "../../include/lmc_gb300.h"

enum class ElementName { X, Al, Mg, Zn, Cu, Sn };

// Element (Element.hpp): ordered by name string (Element.hpp:44-46), so a std::set<Element> or
// std::map<Element, ...> iterates Al, Cu, Mg, Sn, X, Zn as the reference's does.
class Element {
 public:
  Element() = default;
  explicit Element(ElementName name) : name_(name) {}
  explicit Element(const std::string &name);
  [[nodiscard]] std::string GetString() const;
  [[nodiscard]] double GetMass() const;
  [[nodiscard]] ElementName GetElementName() const { return name_; }
  bool operator<(const Element &o) const { return GetString() < o.GetString(); }
  bool operator==(const Element &o) const { return name_ == o.name_; }
  bool operator!=(const Element &o) const { return name_ != o.name_; }

 private:
  ElementName name_{ElementName::X};
};

using Vector_d = std::array<double, 3>;
using Vector_i = std::array<int, 3>;

namespace cfg {

// A perfect cubic FCC supercell of n x n x n conventional cells, lattice ids in
// the reference's ReassignLatticeVector order (id = hx*2n^2 + hy*n + hz/2 in
// half-lattice units), atoms tracked as in Config::LatticeJump (Config.cpp:431-456).
class Config {
 public:
  Config() = default;
  // A copy is a new configuration for the predictors' upload cache (its own identity).
  Config(const Config &o);
  Config &operator=(const Config &o);
  Config(Config &&) = default;
  Config &operator=(Config &&) = default;
  // Config::ReadConfig (Config.cpp:554-649): AtomEye CFG, gzip when the name ends in ".gz".
  static Config ReadConfig(const std::string &filename);
  // Config::GenerateFCC for a cubic box of `n` cells filled with `element`.
  static Config GenerateFCC(int n, const Element &element);
  // Config::WriteConfig (Config.cpp:651-692).
  void WriteConfig(const std::string &filename) const;
  // Config::ReadMap (Config.cpp:814-885): lattice file (site count, basis, per lattice id its
  // relative position and 1-3NN lists), element file (one element per atom id), map file (the
  // lattice id of every atom id). The lattice ids must be in ReassignLatticeVector order (what
  // WriteLattice writes for a configuration read from a CFG file and reassigned).
  static Config ReadMap(const std::string &lattice_filename, const std::string &element_filename,
                        const std::string &map_filename);
  // Config::WriteLattice / WriteElement / WriteMap (Config.cpp:887-922).
  void WriteLattice(const std::string &filename) const;
  void WriteElement(const std::string &filename) const;
  void WriteMap(const std::string &filename) const;
  // Lattice ids are already in ReassignLatticeVector order.
  void ReassignLatticeVector() {}

  [[nodiscard]] size_t GetNumAtoms() const { return lattice_to_atom_.size(); }
  [[nodiscard]] size_t GetNumLattices() const { return lattice_to_atom_.size(); }
  [[nodiscard]] int GetEdge() const { return n_; }
  [[nodiscard]] Element GetElementAtLatticeId(size_t lattice_id) const { return atom_element_.at(lattice_to_atom_.at(lattice_id)); }
  [[nodiscard]] Element GetElementAtAtomId(size_t atom_id) const { return atom_element_.at(atom_id); }
  void SetElementAtLatticeId(size_t lattice_id, const Element &element);
  [[nodiscard]] size_t GetAtomIdFromLatticeId(size_t lattice_id) const { return lattice_to_atom_.at(lattice_id); }
  [[nodiscard]] size_t GetLatticeIdFromAtomId(size_t atom_id) const { return atom_to_lattice_.at(atom_id); }
  [[nodiscard]] Vector_d GetRelativePositionOfLattice(size_t lattice_id) const;
  [[nodiscard]] Vector_d GetUnwrappedCartesianPositionOfLattice(size_t lattice_id) const;  // Config.cpp:280-292
  [[nodiscard]] size_t GetVacancyLatticeId() const;   // first X in atom order (Config.cpp:298-310)
  [[nodiscard]] Element GetSolventElement() const;     // Config.cpp:411-422
  [[nodiscard]] double GetVacancyConcentration() const;  // Config.cpp:373-381
  [[nodiscard]] double GetSoluteConcentration(const Element &solvent) const;  // Config.cpp:383-391
  [[nodiscard]] double GetTotalSoluteMass() const;
  [[nodiscard]] std::vector<size_t> GetNeighborLatticeIdVector(size_t lattice_id, int shell) const;
  void LatticeJump(const std::pair<size_t, size_t> &lattice_id_jump_pair);

  // Species codes per lattice id in the alphabet `names` (element set + X, string order).
  [[nodiscard]] std::vector<int8_t> SpeciesCodes(const std::vector<std::string> &names) const;
  // Replaces the species per lattice id (atoms keep their ids and image shifts).
  void SetSpeciesCodes(const std::vector<int8_t> &codes, const std::vector<std::string> &names);
  // Incremented by every change; predictors re-upload a lattice only when it moved.
  [[nodiscard]] uint64_t Revision() const { return revision_; }
  [[nodiscard]] uint64_t Identity() const { return identity_; }

 private:
  int n_{0};
  std::vector<Element> atom_element_;    // per atom id
  std::vector<uint32_t> lattice_to_atom_;
  std::vector<uint32_t> atom_to_lattice_;
  std::vector<Vector_i> map_shift_;      // per atom id
  uint64_t revision_{0};
  uint64_t identity_{0};
  static uint64_t NextIdentity();
  friend class ConfigAccess;
};

// GenerateSoluteConfig (Config.cpp:1097-1143): a pure `solvent` box of n cells with the solutes
// placed one at a time on uniformly drawn sites that are not within 3NN of an earlier solute. The
// reference draws from a clock-seeded generator over an unordered set; here the draw is over the
// sorted available sites with mt19937_64(seed) (the same distribution, reproducible).
Config GenerateSoluteConfig(int n, const Element &solvent, const std::map<Element, size_t> &solute_atom_count,
                            uint64_t seed);

}  // namespace cfg

namespace pred {

namespace detail {
// One model + one device context per predictor, with the last uploaded lattice.
class Device {
 public:
  Device(const std::string &json_filename, const std::set<Element> &element_set);
  ~Device();
  Device(const Device &) = delete;
  Device &operator=(const Device &) = delete;
  // Makes the context hold `config` (uploads only when it changed).
  void Sync(const cfg::Config &config);
  lmc_ctx *ctx() const { return ctx_; }
  lmc_model *model() const { return model_; }
  const std::vector<std::string> &alphabet() const { return alphabet_; }
  std::mutex &mutex() { return mu_; }

 private:
  lmc_model *model_{nullptr};
  lmc_ctx *ctx_{nullptr};
  std::vector<std::string> alphabet_;
  uint64_t identity_{0}, revision_{~0ull};
  std::mutex mu_;
};
// Throws the reference's exception type for a non-zero status.
void Check(int status);
std::vector<std::string> ElementNames(const std::set<Element> &element_set);
}  // namespace detail

class VacancyMigrationPredictorQuartic {
 public:
  VacancyMigrationPredictorQuartic(const std::string &predictor_filename, const cfg::Config &reference_config,
                                   const std::set<Element> &element_set);
  virtual ~VacancyMigrationPredictorQuartic() = default;
  // {Ea, dE} of the jump first -> second (first holds the vacancy).
  [[nodiscard]] virtual std::pair<double, double> GetBarrierAndDiffFromLatticeIdPair(
      const cfg::Config &config, const std::pair<size_t, size_t> &lattice_id_jump_pair) const;
  // Batched form (GB300 extension): one launch for many pairs.
  void GetBarrierAndDiffFromLatticeIdPairs(const cfg::Config &config,
                                           const std::vector<std::pair<size_t, size_t>> &pairs,
                                           std::vector<double> *barriers, std::vector<double> *energy_changes) const;

 protected:
  VacancyMigrationPredictorQuartic(const std::string &predictor_filename, const std::set<Element> &element_set,
                                   int kind);
  std::shared_ptr<detail::Device> device_;
  int kind_;
};

// The reference memoises barriers in an LRU keyed by the 176 neighbourhood
// species; recomputing on the GPU is cheaper, so cache_size is accepted and unused.
class VacancyMigrationPredictorQuarticLru : public VacancyMigrationPredictorQuartic {
 public:
  VacancyMigrationPredictorQuarticLru(const std::string &predictor_filename, const cfg::Config &reference_config,
                                      const std::set<Element> &element_set, size_t cache_size);
};

class VacancyMigrationPredictorE0 : public VacancyMigrationPredictorQuartic {
 public:
  VacancyMigrationPredictorE0(const std::string &predictor_filename, const cfg::Config &reference_config,
                              const std::set<Element> &element_set);
};

class EnergyChangePredictorPairSite {
 public:
  EnergyChangePredictorPairSite(const std::string &predictor_filename, const cfg::Config &reference_config,
                                const std::set<Element> &element_set);
  [[nodiscard]] double GetDeFromLatticeIdPair(const cfg::Config &config,
                                              const std::pair<size_t, size_t> &lattice_id_jump_pair) const;

 private:
  std::shared_ptr<detail::Device> device_;
};

class EnergyPredictor {
 public:
  EnergyPredictor(const std::string &predictor_filename, const std::set<Element> &element_set);
  [[nodiscard]] double GetEnergy(const cfg::Config &config) const;
  // GetChemicalPotential (EnergyPredictor.cpp:196-214): the energy of one atom of each element
  // (and X) in a 15^3 solvent box relative to the pure box; 0 for the solvent.
  [[nodiscard]] std::map<Element, double> GetChemicalPotential(const Element &solvent_element) const;

 private:
  std::shared_ptr<detail::Device> device_;
};

// TimeTemperatureInterpolator (TimeTemperatureInterpolator.cpp:10-65).
class TimeTemperatureInterpolator {
 public:
  TimeTemperatureInterpolator() = default;
  explicit TimeTemperatureInterpolator(const std::string &time_temperature_filename);
  explicit TimeTemperatureInterpolator(const std::vector<std::pair<double, double>> &points);
  [[nodiscard]] double GetTemperature(double time) const;
  [[nodiscard]] const std::vector<std::pair<double, double>> &GetPoints() const { return points_; }

 private:
  void SortPoints();
  std::vector<std::pair<double, double>> points_;
};

}  // namespace pred

namespace mc {

// ThermodynamicAveraging (ThermodynamicAveraging.cpp:6-42).
class ThermodynamicAveraging {
 public:
  explicit ThermodynamicAveraging(size_t size) : size_(size) {}
  void AddEnergy(double value);
  [[nodiscard]] double GetThermodynamicAverage(double beta) const;

 private:
  size_t size_;
  std::deque<double> energy_list_;
  double sum_{0.0};
};

// KineticMcFirstOmp (KineticMcAbstract.cpp:12-190, KineticMcFirstOmp.cpp): the step
// loop runs in the persistent KMC kernel on the reference's mt19937_64 stream; the
// host replays the trace for kmc_log.txt and the config dumps.
class KineticMcFirstOmp {
 public:
  KineticMcFirstOmp(cfg::Config config, unsigned long long log_dump_steps, unsigned long long config_dump_steps,
                    unsigned long long maximum_steps, unsigned long long thermodynamic_averaging_steps,
                    unsigned long long restart_steps, double restart_energy, double restart_time, double temperature,
                    const std::set<Element> &element_set, const std::string &json_coefficients_filename,
                    const std::string &time_temperature_filename, bool is_rate_corrector, bool is_early_stop,
                    bool is_solute_disp);
  ~KineticMcFirstOmp();
  KineticMcFirstOmp(KineticMcFirstOmp &&) = default;
  void Simulate();
  // The reference seeds its generator from the clock (McAbstract.cpp:32); a fixed seed reproduces a run.
  void SetSeed(uint64_t seed) { seed_ = seed; }
  [[nodiscard]] const cfg::Config &GetConfig() const { return config_; }

 protected:
  bool chain_{false};  // second-order residence time (KineticMcChainOmpi)

 private:
  cfg::Config config_;
  unsigned long long log_dump_steps_, config_dump_steps_, maximum_steps_, steps_;
  double energy_, time_, temperature_;
  std::set<Element> element_set_;
  std::string json_coefficients_filename_;
  pred::TimeTemperatureInterpolator time_temperature_interpolator_;
  bool is_time_temperature_interpolator_, is_rate_corrector_, is_early_stop_, is_solute_disp_;
  uint64_t seed_;
};

// KineticMcChainOmpi (KineticMcChainOmpi.cpp:56-152, KineticMcAbstract.cpp:225-263): the
// second-order residence-time algorithm on one GPU (the reference runs 12 MPI ranks, one per
// first jump): per step the 12 x 12 jumps after each first jump, deterministic second-order
// time, one uniform draw for the selection. Same log and dumps as KineticMcFirstOmp; the early
// stop is not available with it here.
class KineticMcChainOmpi : public KineticMcFirstOmp {
 public:
  KineticMcChainOmpi(cfg::Config config, unsigned long long log_dump_steps, unsigned long long config_dump_steps,
                     unsigned long long maximum_steps, unsigned long long thermodynamic_averaging_steps,
                     unsigned long long restart_steps, double restart_energy, double restart_time, double temperature,
                     const std::set<Element> &element_set, const std::string &json_coefficients_filename,
                     const std::string &time_temperature_filename, bool is_rate_corrector, bool is_early_stop,
                     bool is_solute_disp);
};

// CanonicalMcOmp (CanonicalMcOmp.cpp:40-92, CanonicalMcAbstract.cpp:43-101): batches
// of non-overlapping pairs on the reference's mt19937_64 stream, batch size = the
// OpenMP thread count (OMP_NUM_THREADS, else the hardware threads).
class CanonicalMcOmp {
 public:
  CanonicalMcOmp(cfg::Config config, unsigned long long log_dump_steps, unsigned long long config_dump_steps,
                 unsigned long long maximum_steps, unsigned long long thermodynamic_averaging_steps,
                 unsigned long long restart_steps, double restart_energy, double temperature,
                 const std::set<Element> &element_set, const std::string &json_coefficients_filename);
  void Simulate();
  void SetSeed(uint64_t seed) { seed_ = seed; }
  void SetBatch(int batch) { batch_ = batch; }
  [[nodiscard]] const cfg::Config &GetConfig() const { return config_; }

 private:
  cfg::Config config_;
  unsigned long long log_dump_steps_, config_dump_steps_, maximum_steps_, thermodynamic_averaging_steps_, steps_;
  double energy_, temperature_;
  std::set<Element> element_set_;
  std::string json_coefficients_filename_;
  uint64_t seed_;
  int batch_;
};

// Parameter (Parameter.cpp:8-130): the reference's keys, plus `seed` (fixed
// mt19937_64 seed) and `cmc_batch` (pairs per CanonicalMcOmp batch).
// Seed of the reference's clock-seeded generators (McAbstract.cpp:32).
uint64_t ClockSeedValue();

// SimulatedAnnealing (SimulatedAnnealing.cpp:31-185): trial swaps with the adaptive temperature
// schedule on one warp of the GPU; sa_log.txt and lowest_energy.cfg.gz as the reference writes them.
// `seed` (an extra trailing argument; the reference seeds from the clock) fixes both the solute
// placement (mt19937_64(seed + 1)) and the annealing stream (mt19937_64(seed)).
class SimulatedAnnealing {
 public:
  SimulatedAnnealing(int factor, const Element &solvent_element, const std::map<Element, size_t> &solute_atom_count,
                     unsigned long long log_dump_steps, unsigned long long config_dump_steps,
                     unsigned long long maximum_steps, double initial_temperature,
                     const std::string &json_coefficients_filename, uint64_t seed);
  void Simulate();
  [[nodiscard]] const cfg::Config &GetConfig() const { return config_; }

 private:
  cfg::Config config_;
  Element solvent_;
  std::map<Element, size_t> solute_atom_count_;
  unsigned long long log_dump_steps_, maximum_steps_, steps_{0};
  double initial_temperature_;
  std::string json_coefficients_filename_;
  uint64_t seed_;
};

}  // namespace mc

namespace api {

struct Parameter {
  Parameter() = default;
  Parameter(int argc, char *argv[]);
  explicit Parameter(const std::string &param_filename);
  void ParseArgs(int argc, char *argv[]);
  void ReadParam(const std::string &param_filename);

  std::string parameters_filename;
  std::string method;
  std::string config_filename_, map_filename_, json_coefficients_filename_, time_temperature_filename_;
  std::string log_type_, config_type_;
  unsigned long long log_dump_steps_{0}, config_dump_steps_{0}, maximum_steps_{0},
      thermodynamic_averaging_steps_{0}, restart_steps_{0};
  double temperature_{0}, restart_energy_{0}, restart_time_{0};
  std::vector<std::string> element_set_;
  bool rate_corrector_{false}, early_stop_{false}, solute_disp_{false};
  bool has_seed_{false};
  uint64_t seed_{0};
  int cmc_batch_{0};
  // keys of the analysis (Traverse / ExitTime / SoluteCluster) and annealing schedules, kept for
  // callers that read them (Parameter.cpp:66-80,125-126)
  double decrement_temperature_{0}, escape_temperature_{0};
  unsigned long long initial_steps_{0}, increment_steps_{0}, early_stop_steps_{0};
  size_t smallest_cluster_criteria_{0}, solvent_bond_criteria_{0};
  // SimulatedAnnealing keys (Parameter.cpp:64-65,113-125)
  int factor_{0};
  std::string solvent_element_;
  std::vector<std::string> solute_element_set_;
  std::vector<size_t> solute_number_set_;
  double initial_temperature_{0};
};

// Run (Home.cpp:97-125) for the methods of this path: KineticMcFirstOmp, KineticMcChainOmpi,
// CanonicalMcOmp and SimulatedAnnealing.
void Run(const Parameter &parameter);

}  // namespace api
