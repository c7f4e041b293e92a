// Implementation of the C++ host mirror (lmc_host.hpp) over the C ABI.
#include "lmc_host.hpp"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <fstream>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <limits>
#include <sstream>
#include <stdexcept>
#include <thread>

#if __has_include(<zlib.h>)
#include <zlib.h>
#define LMC_HOST_ZLIB 1
#else
#define LMC_HOST_ZLIB 0
#endif

namespace {

constexpr double kLatticeConstant = 4.046;  // Constants.hpp:6 (Angstrom)

bool EndsWith(const std::string &s, const std::string &suffix) {
  return s.size() >= suffix.size() && s.compare(s.size() - suffix.size(), suffix.size(), suffix) == 0;
}

// Whole file as text, gunzipped when the name ends in ".gz".
std::string ReadText(const std::string &filename) {
  std::ifstream probe(filename, std::ios::binary);
  if (!probe) throw std::runtime_error("Cannot open " + filename);
  if (!EndsWith(filename, ".gz")) {
    std::ostringstream ss;
    ss << probe.rdbuf();
    return ss.str();
  }
#if LMC_HOST_ZLIB
  probe.close();
  gzFile f = gzopen(filename.c_str(), "rb");
  if (!f) throw std::runtime_error("Cannot open " + filename);
  std::string out;
  char buf[1 << 16];
  int got;
  while ((got = gzread(f, buf, sizeof(buf))) > 0) out.append(buf, static_cast<size_t>(got));
  gzclose(f);
  if (got < 0) throw std::runtime_error("Cannot read " + filename);
  return out;
#else
  throw std::runtime_error("Cannot open " + filename + ": built without zlib");
#endif
}

#if !LMC_HOST_ZLIB
uint32_t Crc32(const unsigned char *p, size_t n, uint32_t c = 0) {
  // CRC-32 (IEEE 802.3, reflected polynomial 0xEDB88320), bitwise
  c = ~c;
  for (size_t i = 0; i < n; ++i) {
    c ^= p[i];
    for (int k = 0; k < 8; ++k) c = (c >> 1) ^ (0xEDB88320u & (0u - (c & 1u)));
  }
  return ~c;
}
#endif

// Writes text, gzipped when the name ends in ".gz" (zlib when available, else a
// valid gzip stream of stored deflate blocks, RFC 1951/1952).
void WriteText(const std::string &filename, const std::string &text) {
  if (!EndsWith(filename, ".gz")) {
    std::ofstream ofs(filename, std::ios::binary);
    if (!ofs) throw std::runtime_error("Cannot open " + filename);
    ofs << text;
    return;
  }
#if LMC_HOST_ZLIB
  gzFile f = gzopen(filename.c_str(), "wb");
  if (!f) throw std::runtime_error("Cannot open " + filename);
  if (!text.empty() && gzwrite(f, text.data(), static_cast<unsigned>(text.size())) == 0) {
    gzclose(f);
    throw std::runtime_error("Cannot write " + filename);
  }
  gzclose(f);
#else
  std::ofstream ofs(filename, std::ios::binary);
  if (!ofs) throw std::runtime_error("Cannot open " + filename);
  const unsigned char header[10] = {0x1f, 0x8b, 8, 0, 0, 0, 0, 0, 0, 255};
  ofs.write(reinterpret_cast<const char *>(header), 10);
  const auto *p = reinterpret_cast<const unsigned char *>(text.data());
  size_t left = text.size(), off = 0;
  do {
    const size_t len = std::min<size_t>(left, 65535);
    const unsigned char b[5] = {static_cast<unsigned char>(left <= 65535 ? 1 : 0), static_cast<unsigned char>(len),
                                static_cast<unsigned char>(len >> 8), static_cast<unsigned char>(~len),
                                static_cast<unsigned char>(~len >> 8)};
    ofs.write(reinterpret_cast<const char *>(b), 5);
    ofs.write(reinterpret_cast<const char *>(p + off), static_cast<std::streamsize>(len));
    off += len;
    left -= len;
  } while (left > 0);
  const uint32_t crc = Crc32(p, text.size()), sz = static_cast<uint32_t>(text.size());
  const unsigned char t[8] = {static_cast<unsigned char>(crc), static_cast<unsigned char>(crc >> 8),
                              static_cast<unsigned char>(crc >> 16), static_cast<unsigned char>(crc >> 24),
                              static_cast<unsigned char>(sz), static_cast<unsigned char>(sz >> 8),
                              static_cast<unsigned char>(sz >> 16), static_cast<unsigned char>(sz >> 24)};
  ofs.write(reinterpret_cast<const char *>(t), 8);
#endif
}

// Vector_d stream output as the reference's operator<< (VectorMatrix.hpp:41-51),
// which switches the stream to fixed notation for everything that follows.
std::ostream &PutVector(std::ostream &os, const Vector_d &v) {
  os << std::fixed << v[0] << ' ' << v[1] << ' ' << v[2];
  return os;
}
std::ostream &PutVector(std::ostream &os, const Vector_i &v) {
  os << std::fixed << v[0] << ' ' << v[1] << ' ' << v[2];
  return os;
}

std::vector<std::string> Split(const std::string &s) {
  std::vector<std::string> out;
  std::istringstream is(s);
  std::string w;
  while (is >> w) out.push_back(w);
  return out;
}

}  // namespace

// ---------------------------------------------------------------------------
// Element
// ---------------------------------------------------------------------------
Element::Element(const std::string &name) {
  static const std::map<std::string, ElementName> kNames = {{"X", ElementName::X},   {"Al", ElementName::Al},
                                                            {"Mg", ElementName::Mg}, {"Zn", ElementName::Zn},
                                                            {"Cu", ElementName::Cu}, {"Sn", ElementName::Sn}};
  const auto it = kNames.find(name);
  if (it == kNames.end()) throw std::invalid_argument("Unexpected element " + name);
  name_ = it->second;
}

std::string Element::GetString() const {
  switch (name_) {
    case ElementName::X: return "X";
    case ElementName::Al: return "Al";
    case ElementName::Mg: return "Mg";
    case ElementName::Zn: return "Zn";
    case ElementName::Cu: return "Cu";
    case ElementName::Sn: return "Sn";
  }
  throw std::invalid_argument("Unexpected element");
}

double Element::GetMass() const {
  // atomic masses as the reference tabulates them (Element.hpp:71-87)
  switch (name_) {
    case ElementName::X: return 0.00;
    case ElementName::Al: return 26.98;
    case ElementName::Mg: return 24.31;
    case ElementName::Zn: return 65.38;
    case ElementName::Cu: return 63.55;
    case ElementName::Sn: return 118.71;
  }
  throw std::invalid_argument("Unexpected element");
}

// ---------------------------------------------------------------------------
// cfg::Config
// ---------------------------------------------------------------------------
namespace cfg {

uint64_t Config::NextIdentity() {
  static std::atomic<uint64_t> next{1};
  return next++;
}

Config::Config(const Config &o)
    : n_(o.n_),
      atom_element_(o.atom_element_),
      lattice_to_atom_(o.lattice_to_atom_),
      atom_to_lattice_(o.atom_to_lattice_),
      map_shift_(o.map_shift_),
      revision_(0),
      identity_(NextIdentity()) {}

Config &Config::operator=(const Config &o) {
  if (this != &o) {
    n_ = o.n_;
    atom_element_ = o.atom_element_;
    lattice_to_atom_ = o.lattice_to_atom_;
    atom_to_lattice_ = o.atom_to_lattice_;
    map_shift_ = o.map_shift_;
    revision_ = 0;
    identity_ = NextIdentity();
  }
  return *this;
}

Config Config::GenerateFCC(int n, const Element &element) {
  if (n < 6 || n > 1000) throw std::invalid_argument("supercell edge must be in [6, 1000]");
  Config c;
  c.n_ = n;
  const size_t N = 4ull * n * n * n;
  c.atom_element_.assign(N, element);
  c.lattice_to_atom_.resize(N);
  c.atom_to_lattice_.resize(N);
  for (size_t i = 0; i < N; ++i) c.lattice_to_atom_[i] = c.atom_to_lattice_[i] = static_cast<uint32_t>(i);
  c.map_shift_.assign(N, Vector_i{0, 0, 0});
  c.identity_ = NextIdentity();
  return c;
}

Config Config::ReadConfig(const std::string &filename) {
  std::istringstream fis(ReadText(filename));
  const auto skip_to = [&](char ch) { fis.ignore(std::numeric_limits<std::streamsize>::max(), ch); };
  // "Number of particles = %i"
  skip_to('=');
  size_t num_atoms = 0;
  fis >> num_atoms;
  skip_to('=');  // A = 1.0 Angstrom
  double basis[9];
  for (double &b : basis) {
    skip_to('=');
    fis >> b;
  }
  skip_to('\n');
  bool has_no_velocity = false;
  if (fis.peek() == '.') {
    has_no_velocity = true;
    skip_to('\n');
  }
  skip_to('=');
  size_t entry_count = 0;
  fis >> entry_count;
  skip_to('\n');
  while (fis.good()) {
    while (std::isspace(fis.peek()) && fis.peek() != '\n') fis.get();
    const int next = fis.peek();
    if (fis.eof()) break;
    if (std::isdigit(next) || next == '.' || next == '-') break;
    skip_to('\n');
  }
  if (!fis.good() || num_atoms == 0) throw std::runtime_error("Cannot read " + filename);
  // perfect cubic FCC: N = 4 n^3, diagonal basis
  const int n = static_cast<int>(std::llround(std::cbrt(static_cast<double>(num_atoms) / 4.0)));
  if (4ull * n * n * n != num_atoms) throw std::invalid_argument(filename + ": not a cubic FCC supercell");
  if (basis[1] != 0 || basis[2] != 0 || basis[3] != 0 || basis[5] != 0 || basis[6] != 0 || basis[7] != 0 ||
      basis[0] != basis[4] || basis[0] != basis[8])
    throw std::invalid_argument(filename + ": only cubic boxes are supported");
  Config c = GenerateFCC(n, Element(ElementName::X));
  std::vector<char> taken(num_atoms, 0);
  const int m = 2 * n;
  for (size_t atom = 0; atom < num_atoms; ++atom) {
    double mass;
    std::string type;
    Vector_d r{};
    Vector_i shift{0, 0, 0};
    fis >> mass >> type >> r[0] >> r[1] >> r[2];
    if (entry_count >= 6 && has_no_velocity) fis >> shift[0] >> shift[1] >> shift[2];
    if (!fis) throw std::runtime_error("Cannot read " + filename);
    skip_to('\n');
    int h[3];
    for (int d = 0; d < 3; ++d) {
      const double v = r[d] * m;
      const long long k = std::llround(v);
      if (std::fabs(v - static_cast<double>(k)) > 1e-3) throw std::invalid_argument(filename + ": off-lattice atom");
      h[d] = static_cast<int>(((k % m) + m) % m);
    }
    if ((h[0] + h[1] + h[2]) & 1) throw std::invalid_argument(filename + ": off-lattice atom");
    const size_t id = static_cast<size_t>(h[0]) * 2 * n * n + static_cast<size_t>(h[1]) * n + h[2] / 2;
    if (taken[id]) throw std::invalid_argument(filename + ": two atoms on one lattice site");
    taken[id] = 1;
    c.atom_element_[atom] = Element(type);
    c.lattice_to_atom_[id] = static_cast<uint32_t>(atom);
    c.atom_to_lattice_[atom] = static_cast<uint32_t>(id);
    c.map_shift_[atom] = shift;
  }
  return c;
}

void Config::WriteConfig(const std::string &filename) const {
  std::ostringstream fos;
  fos.precision(16);
  const double L = n_ * kLatticeConstant;
  fos << "Number of particles = " << GetNumAtoms() << '\n';
  fos << "A = 1.0 Angstrom (basic length-scale)\n";
  const double b[9] = {L, 0, 0, 0, L, 0, 0, 0, L};
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) fos << "H0(" << i + 1 << ',' << j + 1 << ") = " << b[3 * i + j] << " A\n";
  fos << ".NO_VELOCITY.\n";
  fos << "entry_count = 6\n";
  fos << "auxiliary[0] = ix\n";
  fos << "auxiliary[1] = iy\n";
  fos << "auxiliary[2] = iz\n";
  for (size_t atom = 0; atom < atom_element_.size(); ++atom) {
    fos << atom_element_[atom].GetMass() << '\n' << atom_element_[atom].GetString() << '\n';
    PutVector(fos, GetRelativePositionOfLattice(atom_to_lattice_[atom])) << ' ';
    PutVector(fos, map_shift_[atom]) << '\n';
  }
  WriteText(filename, fos.str());
}

Config Config::ReadMap(const std::string &lattice_filename, const std::string &element_filename,
                       const std::string &map_filename) {
  std::ifstream ifs_lattice(lattice_filename);
  if (!ifs_lattice.is_open()) throw std::runtime_error("Cannot open " + lattice_filename);
  size_t num_atoms = 0;
  ifs_lattice >> num_atoms;
  ifs_lattice.ignore(std::numeric_limits<std::streamsize>::max(), '\n');
  double basis[9];
  for (double &b : basis) ifs_lattice >> b;
  if (!ifs_lattice || num_atoms == 0) throw std::runtime_error("Cannot read " + lattice_filename);
  const int n = static_cast<int>(std::llround(std::cbrt(static_cast<double>(num_atoms) / 4.0)));
  if (4ull * n * n * n != num_atoms) throw std::invalid_argument(lattice_filename + ": not a cubic FCC supercell");
  if (basis[1] != 0 || basis[2] != 0 || basis[3] != 0 || basis[5] != 0 || basis[6] != 0 || basis[7] != 0 ||
      basis[0] != basis[4] || basis[0] != basis[8])
    throw std::invalid_argument(lattice_filename + ": only cubic boxes are supported");
  Config c = GenerateFCC(n, Element(ElementName::X));
  const int m = 2 * n;
  for (size_t lattice_id = 0; lattice_id < num_atoms; ++lattice_id) {
    Vector_d r{};
    ifs_lattice >> r[0] >> r[1] >> r[2];
    if (!ifs_lattice) throw std::runtime_error("Cannot read " + lattice_filename);
    ifs_lattice.ignore(std::numeric_limits<std::streamsize>::max(), '\n');  // the neighbour lists
    int h[3];
    for (int d = 0; d < 3; ++d) {
      const double v = r[d] * m;
      const long long k = std::llround(v);
      if (std::fabs(v - static_cast<double>(k)) > 1e-3) throw std::invalid_argument(lattice_filename + ": off-lattice site");
      h[d] = static_cast<int>(((k % m) + m) % m);
    }
    if ((h[0] + h[1] + h[2]) & 1) throw std::invalid_argument(lattice_filename + ": off-lattice site");
    const size_t id = static_cast<size_t>(h[0]) * 2 * n * n + static_cast<size_t>(h[1]) * n + h[2] / 2;
    if (id != lattice_id)
      throw std::invalid_argument(lattice_filename + ": lattice ids are not in ReassignLatticeVector order");
  }
  std::ifstream ifs_element(element_filename);
  if (!ifs_element.is_open()) throw std::runtime_error("Cannot open " + element_filename);
  std::string type;
  for (size_t atom = 0; atom < num_atoms; ++atom) {
    if (!(ifs_element >> type)) throw std::runtime_error("Cannot read " + element_filename);
    c.atom_element_[atom] = Element(type);
    ifs_element.ignore(std::numeric_limits<std::streamsize>::max(), '\n');
  }
  std::ifstream ifs_map(map_filename);
  if (!ifs_map.is_open()) throw std::runtime_error("Cannot open " + map_filename);
  constexpr uint32_t kUnset = std::numeric_limits<uint32_t>::max();
  c.lattice_to_atom_.assign(num_atoms, kUnset);
  c.atom_to_lattice_.assign(num_atoms, kUnset);
  for (size_t atom = 0; atom < num_atoms; ++atom) {
    size_t lattice_id = 0;
    if (!(ifs_map >> lattice_id)) throw std::runtime_error("Cannot read " + map_filename);
    if (lattice_id >= num_atoms)
      throw std::runtime_error("Lattice id out of bounds in map file: " + std::to_string(lattice_id));
    if (c.lattice_to_atom_[lattice_id] != kUnset)
      throw std::runtime_error("Duplicate lattice id in map file: " + std::to_string(lattice_id));
    c.lattice_to_atom_[lattice_id] = static_cast<uint32_t>(atom);
    c.atom_to_lattice_[atom] = static_cast<uint32_t>(lattice_id);
    ifs_map.ignore(std::numeric_limits<std::streamsize>::max(), '\n');
  }
  return c;
}

void Config::WriteLattice(const std::string &filename) const {
  std::ofstream ofs(filename);
  ofs.precision(16);
  const double L = kLatticeConstant * static_cast<double>(n_);
  ofs << GetNumAtoms() << " positions in total" << '\n';
  PutVector(ofs, Vector_d{L, 0, 0}) << '\n';
  PutVector(ofs, Vector_d{0, L, 0}) << '\n';
  PutVector(ofs, Vector_d{0, 0, L}) << std::endl;
  for (size_t id = 0; id < GetNumLattices(); ++id) {
    PutVector(ofs, GetRelativePositionOfLattice(id));
    ofs << " # ";
    for (int shell = 1; shell <= 3; ++shell)
      for (size_t nb : GetNeighborLatticeIdVector(id, shell)) ofs << nb << ' ';
    ofs << std::endl;
  }
}

void Config::WriteElement(const std::string &filename) const {
  std::ofstream ofs(filename);
  ofs.precision(16);
  for (const auto &e : atom_element_) ofs << e.GetString() << std::endl;
}

void Config::WriteMap(const std::string &filename) const {
  std::ofstream ofs(filename);
  ofs.precision(16);
  for (size_t atom = 0; atom < atom_to_lattice_.size(); ++atom) ofs << atom_to_lattice_[atom] << std::endl;
}

Vector_d Config::GetRelativePositionOfLattice(size_t id) const {
  const size_t plane = 2ull * n_ * n_;
  const int hx = static_cast<int>(id / plane);
  const size_t rem = id - static_cast<size_t>(hx) * plane;
  const int hy = static_cast<int>(rem / n_);
  const int k = static_cast<int>(rem - static_cast<size_t>(hy) * n_);
  const int hz = 2 * k + ((hx + hy) & 1);
  const double m = 2.0 * n_;
  return {hx / m, hy / m, hz / m};
}

Vector_d Config::GetUnwrappedCartesianPositionOfLattice(size_t lattice_id) const {
  const Vector_d r = GetRelativePositionOfLattice(lattice_id);
  const Vector_i &s = map_shift_.at(lattice_to_atom_.at(lattice_id));
  const double L = n_ * kLatticeConstant;
  return {(r[0] + s[0]) * L, (r[1] + s[1]) * L, (r[2] + s[2]) * L};
}

size_t Config::GetVacancyLatticeId() const {
  for (size_t atom = 0; atom < atom_element_.size(); ++atom)
    if (atom_element_[atom].GetElementName() == ElementName::X) return atom_to_lattice_[atom];
  throw std::runtime_error("No vacancy found");
}

Element Config::GetSolventElement() const {
  std::map<Element, size_t> count;
  for (const auto &e : atom_element_) ++count[e];
  Element solvent(ElementName::X);
  size_t best = 0;
  for (const auto &[e, c] : count)
    if (c > best) {
      best = c;
      solvent = e;
    }
  return solvent;
}

double Config::GetVacancyConcentration() const {
  size_t v = 0;
  for (const auto &e : atom_element_) v += e.GetElementName() == ElementName::X;
  return static_cast<double>(v) / static_cast<double>(GetNumAtoms());
}

double Config::GetSoluteConcentration(const Element &solvent) const {
  size_t s = 0;
  for (const auto &e : atom_element_) s += (e != solvent && e.GetElementName() != ElementName::X);
  return static_cast<double>(s) / static_cast<double>(GetNumAtoms());
}

double Config::GetTotalSoluteMass() const {
  const Element solvent = GetSolventElement();
  double m = 0.0;
  for (const auto &e : atom_element_)
    if (e != solvent) m += e.GetMass();
  return m;
}

std::vector<size_t> Config::GetNeighborLatticeIdVector(size_t lattice_id, int shell) const {
  if (shell < 1 || shell > 3) throw std::out_of_range("shell must be 1, 2 or 3");
  std::vector<int64_t> nb(42);
  pred::detail::Check(lmc_geom_neighbors(n_, static_cast<int64_t>(lattice_id), nb.data()));
  const int begin = shell == 1 ? 0 : (shell == 2 ? 12 : 18), end = shell == 1 ? 12 : (shell == 2 ? 18 : 42);
  return std::vector<size_t>(nb.begin() + begin, nb.begin() + end);
}

void Config::SetElementAtLatticeId(size_t lattice_id, const Element &element) {
  atom_element_.at(lattice_to_atom_.at(lattice_id)) = element;
  ++revision_;
}

void Config::LatticeJump(const std::pair<size_t, size_t> &jump) {
  const auto [lhs, rhs] = jump;
  const uint32_t a_lhs = lattice_to_atom_.at(lhs), a_rhs = lattice_to_atom_.at(rhs);
  const Vector_d pl = GetRelativePositionOfLattice(lhs), pr = GetRelativePositionOfLattice(rhs);
  Vector_i image{0, 0, 0};
  for (int d = 0; d < 3; ++d) {
    const double shift = pr[d] - pl[d];
    if (std::fabs(shift) > 0.5 + 1e-8) image[d] = static_cast<int>(std::floor(shift + 0.5));
  }
  for (int d = 0; d < 3; ++d) {
    map_shift_[a_lhs][d] -= image[d];
    map_shift_[a_rhs][d] += image[d];
  }
  atom_to_lattice_[a_lhs] = static_cast<uint32_t>(rhs);
  atom_to_lattice_[a_rhs] = static_cast<uint32_t>(lhs);
  lattice_to_atom_[lhs] = a_rhs;
  lattice_to_atom_[rhs] = a_lhs;
  ++revision_;
}

std::vector<int8_t> Config::SpeciesCodes(const std::vector<std::string> &names) const {
  std::map<ElementName, int8_t> code;
  for (size_t i = 0; i < names.size(); ++i) code[Element(names[i]).GetElementName()] = static_cast<int8_t>(i);
  std::vector<int8_t> out(GetNumLattices());
  for (size_t id = 0; id < out.size(); ++id) {
    const auto it = code.find(atom_element_[lattice_to_atom_[id]].GetElementName());
    if (it == code.end())
      throw std::invalid_argument("element " + atom_element_[lattice_to_atom_[id]].GetString() +
                                  " is not in the element set");
    out[id] = it->second;
  }
  return out;
}

void Config::SetSpeciesCodes(const std::vector<int8_t> &codes, const std::vector<std::string> &names) {
  if (codes.size() != GetNumLattices()) throw std::invalid_argument("species array size mismatch");
  for (size_t id = 0; id < codes.size(); ++id) atom_element_[lattice_to_atom_[id]] = Element(names.at(codes[id]));
  ++revision_;
}

Config GenerateSoluteConfig(int n, const Element &solvent, const std::map<Element, size_t> &solute_atom_count,
                            uint64_t seed) {
  Config config = Config::GenerateFCC(n, solvent);
  std::mt19937_64 generator(seed);
  std::set<size_t> available;
  for (size_t i = 0; i < config.GetNumLattices(); ++i) available.insert(i);
  for (const auto &[solute, count] : solute_atom_count) {
    for (size_t it = 0; it < count; ++it) {
      if (available.empty()) {
        std::cerr << "Size is too small. Cannot generate correct config.\n";
        return config;
      }
      std::uniform_int_distribution<size_t> dis(0, available.size() - 1);
      auto pos = available.begin();
      std::advance(pos, static_cast<long>(dis(generator)));
      const size_t site = *pos;
      config.SetElementAtLatticeId(site, solute);
      available.erase(site);
      for (int shell = 1; shell <= 3; ++shell)
        for (size_t nb : config.GetNeighborLatticeIdVector(site, shell)) available.erase(nb);
    }
  }
  return config;
}

}  // namespace cfg

// ---------------------------------------------------------------------------
// pred
// ---------------------------------------------------------------------------
namespace pred {
namespace detail {

void Check(int status) {
  if (status == LMC_OK) return;
  const std::string msg = lmc_last_error();
  switch (status) {
    case LMC_ERR_OUT_OF_RANGE: throw std::out_of_range(msg);
    case LMC_ERR_INVALID_ARGUMENT: throw std::invalid_argument(msg);
    default: throw std::runtime_error(msg);
  }
}

std::vector<std::string> ElementNames(const std::set<Element> &element_set) {
  std::vector<std::string> out;
  for (const auto &e : element_set) out.push_back(e.GetString());
  return out;
}

Device::Device(const std::string &json_filename, const std::set<Element> &element_set) {
  const auto names = ElementNames(element_set);
  std::vector<const char *> ptrs;
  for (const auto &s : names) ptrs.push_back(s.c_str());
  {
    std::ifstream probe(json_filename);
    if (!probe) throw std::runtime_error("Cannot open " + json_filename);
  }
  Check(lmc_model_load_json(json_filename.c_str(), ptrs.data(), static_cast<int>(ptrs.size()), &model_));
  char buf[256];
  Check(lmc_model_alphabet(model_, buf, sizeof(buf)));
  std::istringstream is(buf);
  std::string w;
  while (is >> w) alphabet_.push_back(w);
  const int st = lmc_ctx_create(model_, 0, &ctx_);
  if (st != LMC_OK) {
    lmc_model_destroy(model_);
    model_ = nullptr;
    Check(st);
  }
}

Device::~Device() {
  if (ctx_) lmc_ctx_destroy(ctx_);
  if (model_) lmc_model_destroy(model_);
}

void Device::Sync(const cfg::Config &config) {
  if (config.Identity() == identity_ && config.Revision() == revision_) return;
  const auto codes = config.SpeciesCodes(alphabet_);
  const int32_t n = config.GetEdge();
  Check(lmc_ctx_set_lattices(ctx_, 1, &n, codes.data()));
  identity_ = config.Identity();
  revision_ = config.Revision();
}

}  // namespace detail

VacancyMigrationPredictorQuartic::VacancyMigrationPredictorQuartic(const std::string &predictor_filename,
                                                                   const cfg::Config &reference_config,
                                                                   const std::set<Element> &element_set)
    : VacancyMigrationPredictorQuartic(predictor_filename, element_set, LMC_BARRIER_QUARTIC) {
  (void)reference_config;  // the neighbour tables are translation invariant and built on the device
}

VacancyMigrationPredictorQuartic::VacancyMigrationPredictorQuartic(const std::string &predictor_filename,
                                                                   const std::set<Element> &element_set, int kind)
    : device_(std::make_shared<detail::Device>(predictor_filename, element_set)), kind_(kind) {}

std::pair<double, double> VacancyMigrationPredictorQuartic::GetBarrierAndDiffFromLatticeIdPair(
    const cfg::Config &config, const std::pair<size_t, size_t> &lattice_id_jump_pair) const {
  std::vector<double> ea, de;
  GetBarrierAndDiffFromLatticeIdPairs(config, {lattice_id_jump_pair}, &ea, &de);
  return {ea[0], de[0]};
}

void VacancyMigrationPredictorQuartic::GetBarrierAndDiffFromLatticeIdPairs(
    const cfg::Config &config, const std::vector<std::pair<size_t, size_t>> &pairs, std::vector<double> *barriers,
    std::vector<double> *energy_changes) const {
  std::lock_guard<std::mutex> lock(device_->mutex());
  device_->Sync(config);
  const int m = static_cast<int>(pairs.size());
  std::vector<int64_t> p(2 * pairs.size());
  for (size_t i = 0; i < pairs.size(); ++i) {
    p[2 * i] = static_cast<int64_t>(pairs[i].first);
    p[2 * i + 1] = static_cast<int64_t>(pairs[i].second);
  }
  barriers->assign(pairs.size(), 0.0);
  energy_changes->assign(pairs.size(), 0.0);
  std::vector<double> aux0(pairs.size()), aux1(pairs.size());
  detail::Check(lmc_barrier_batch(device_->ctx(), 0, kind_, p.data(), m, barriers->data(), energy_changes->data(),
                                  aux0.data(), aux1.data()));
}

VacancyMigrationPredictorQuarticLru::VacancyMigrationPredictorQuarticLru(const std::string &predictor_filename,
                                                                         const cfg::Config &reference_config,
                                                                         const std::set<Element> &element_set,
                                                                         size_t cache_size)
    : VacancyMigrationPredictorQuartic(predictor_filename, reference_config, element_set) {
  (void)cache_size;
}

VacancyMigrationPredictorE0::VacancyMigrationPredictorE0(const std::string &predictor_filename,
                                                         const cfg::Config &reference_config,
                                                         const std::set<Element> &element_set)
    : VacancyMigrationPredictorQuartic(predictor_filename, element_set, LMC_BARRIER_E0) {
  (void)reference_config;
}

EnergyChangePredictorPairSite::EnergyChangePredictorPairSite(const std::string &predictor_filename,
                                                             const cfg::Config &reference_config,
                                                             const std::set<Element> &element_set)
    : device_(std::make_shared<detail::Device>(predictor_filename, element_set)) {
  (void)reference_config;
}

double EnergyChangePredictorPairSite::GetDeFromLatticeIdPair(const cfg::Config &config,
                                                             const std::pair<size_t, size_t> &pair) const {
  std::lock_guard<std::mutex> lock(device_->mutex());
  device_->Sync(config);
  const int64_t p[2] = {static_cast<int64_t>(pair.first), static_cast<int64_t>(pair.second)};
  double de = 0.0;
  detail::Check(lmc_de_pairs(device_->ctx(), 0, p, 1, &de));
  return de;
}

EnergyPredictor::EnergyPredictor(const std::string &predictor_filename, const std::set<Element> &element_set)
    : device_(std::make_shared<detail::Device>(predictor_filename, element_set)) {}

double EnergyPredictor::GetEnergy(const cfg::Config &config) const {
  std::lock_guard<std::mutex> lock(device_->mutex());
  device_->Sync(config);
  double e = 0.0;
  detail::Check(lmc_energy(device_->ctx(), 0, &e, nullptr));
  return e;
}

std::map<Element, double> EnergyPredictor::GetChemicalPotential(const Element &solvent_element) const {
  std::map<Element, double> potential;
  const double solvent_energy = GetEnergy(cfg::Config::GenerateFCC(15, solvent_element));
  potential[solvent_element] = 0;
  for (const auto &name : device_->alphabet()) {  // the element set and X
    const Element element(name);
    if (element == solvent_element) continue;
    cfg::Config config = cfg::Config::GenerateFCC(15, solvent_element);
    config.SetElementAtLatticeId(config.GetLatticeIdFromAtomId(0), element);
    potential[element] = GetEnergy(config) - solvent_energy;
  }
  return potential;
}

TimeTemperatureInterpolator::TimeTemperatureInterpolator(const std::string &filename) {
  if (filename.empty()) return;
  std::ifstream ifs(filename);
  if (!ifs.is_open()) throw std::runtime_error("Cannot open " + filename);
  // header lines until the first line that starts with '0' (TimeTemperatureInterpolator.cpp:18)
  while (ifs.good() && ifs.peek() != '0') ifs.ignore(std::numeric_limits<std::streamsize>::max(), '\n');
  double time, temperature;
  while (ifs >> time >> temperature) {
    points_.emplace_back(time, temperature);
    ifs.ignore(std::numeric_limits<std::streamsize>::max(), '\n');
  }
  SortPoints();
}

TimeTemperatureInterpolator::TimeTemperatureInterpolator(const std::vector<std::pair<double, double>> &points)
    : points_(points) {
  SortPoints();
}

void TimeTemperatureInterpolator::SortPoints() {
  std::sort(points_.begin(), points_.end());
  for (size_t i = 1; i < points_.size(); ++i)
    if (std::abs(points_[i].first - points_[i - 1].first) < 1.0e-12)
      throw std::range_error("2 adjacent x values are equal." + std::to_string(points_[i].first));
}

double TimeTemperatureInterpolator::GetTemperature(double time) const {
  const auto it = std::lower_bound(points_.cbegin(), points_.cend(), time,
                                   [](const std::pair<double, double> &p, double x) { return p.first < x; });
  if (it == points_.cend()) return (points_.cend() - 1)->second;
  if (it == points_.cbegin() && time <= points_.cbegin()->first) return points_.cbegin()->second;
  const double ux = it->first, uy = it->second, lx = (it - 1)->first, ly = (it - 1)->second;
  return ly + ((time - lx) / (ux - lx)) * (uy - ly);
}

}  // namespace pred

// ---------------------------------------------------------------------------
// mc
// ---------------------------------------------------------------------------
namespace mc {

namespace {
constexpr double kBoltzmann = 8.617333262145e-5;  // Constants.hpp:31

uint64_t ClockSeed() {
  return static_cast<uint64_t>(std::chrono::system_clock::now().time_since_epoch().count());
}
}  // namespace

uint64_t ClockSeedValue() { return ClockSeed(); }

namespace {

// Log cadence of McAbstract::Dump (KineticMcAbstract.cpp:82-90, CanonicalMcAbstract.cpp:72-79).
bool LogThisStep(unsigned long long steps, unsigned long long log_dump_steps) {
  unsigned long long every;
  if (steps > 10 * log_dump_steps) {
    every = log_dump_steps;
  } else {
    every = static_cast<unsigned long long>(
        std::pow(10, static_cast<unsigned long long>(std::log10(static_cast<double>(steps + 1)) - 1)));
    every = std::max(every, 1ull);
    every = std::min(every, log_dump_steps);
  }
  return every == 0 || steps % every == 0;
}
}  // namespace

void ThermodynamicAveraging::AddEnergy(double value) {
  if (size_ == 0) return;
  if (energy_list_.size() == size_) {
    sum_ -= energy_list_.front();
    energy_list_.pop_front();
  }
  energy_list_.push_back(value);
  sum_ += value;
}

double ThermodynamicAveraging::GetThermodynamicAverage(double beta) const {
  if (size_ == 0) return 0;
  const double average = energy_list_.empty() ? 0 : sum_ / static_cast<double>(energy_list_.size());
  double partition = 0.0, weighted = 0.0;
  for (double e : energy_list_) {
    e -= average;
    const double w = std::exp(-e * beta);
    weighted += e * w;
    partition += w;
  }
  return weighted / partition + average;
}

KineticMcFirstOmp::KineticMcFirstOmp(cfg::Config config, unsigned long long log_dump_steps,
                                     unsigned long long config_dump_steps, unsigned long long maximum_steps,
                                     unsigned long long thermodynamic_averaging_steps,
                                     unsigned long long restart_steps, double restart_energy, double restart_time,
                                     double temperature, const std::set<Element> &element_set,
                                     const std::string &json_coefficients_filename,
                                     const std::string &time_temperature_filename, bool is_rate_corrector,
                                     bool is_early_stop, bool is_solute_disp)
    : config_(std::move(config)),
      log_dump_steps_(log_dump_steps),
      config_dump_steps_(config_dump_steps),
      maximum_steps_(maximum_steps),
      steps_(restart_steps),
      energy_(restart_energy),
      time_(restart_time),
      temperature_(temperature),
      element_set_(element_set),
      json_coefficients_filename_(json_coefficients_filename),
      time_temperature_interpolator_(time_temperature_filename),
      is_time_temperature_interpolator_(!time_temperature_filename.empty()),
      is_rate_corrector_(is_rate_corrector),
      is_early_stop_(is_early_stop),
      is_solute_disp_(is_solute_disp),
      seed_(ClockSeed()) {
  (void)thermodynamic_averaging_steps;  // the KMC log has no averaged column
}

KineticMcFirstOmp::~KineticMcFirstOmp() = default;

KineticMcChainOmpi::KineticMcChainOmpi(cfg::Config config, unsigned long long log_dump_steps,
                                       unsigned long long config_dump_steps, unsigned long long maximum_steps,
                                       unsigned long long thermodynamic_averaging_steps,
                                       unsigned long long restart_steps, double restart_energy, double restart_time,
                                       double temperature, const std::set<Element> &element_set,
                                       const std::string &json_coefficients_filename,
                                       const std::string &time_temperature_filename, bool is_rate_corrector,
                                       bool is_early_stop, bool is_solute_disp)
    : KineticMcFirstOmp(std::move(config), log_dump_steps, config_dump_steps, maximum_steps,
                        thermodynamic_averaging_steps, restart_steps, restart_energy, restart_time, temperature,
                        element_set, json_coefficients_filename, time_temperature_filename, is_rate_corrector,
                        is_early_stop, is_solute_disp) {
  if (is_early_stop) throw std::invalid_argument("early_stop is not available with KineticMcChainOmpi here");
  chain_ = true;
}

void KineticMcFirstOmp::Simulate() {
  pred::detail::Device dev(json_coefficients_filename_, element_set_);
  dev.Sync(config_);
  std::vector<double> tt_time, tt_temp;
  for (const auto &[t, v] : time_temperature_interpolator_.GetPoints()) {
    tt_time.push_back(t);
    tt_temp.push_back(v);
  }
  lmc_kmc_options opt{};
  opt.rng = LMC_RNG_MT19937_64;
  opt.seed = seed_;
  opt.barrier_kind = LMC_BARRIER_QUARTIC;
  opt.rate_corrector = is_rate_corrector_ ? 1 : 0;
  opt.tt_time = is_time_temperature_interpolator_ ? tt_time.data() : nullptr;
  opt.tt_temp = is_time_temperature_interpolator_ ? tt_temp.data() : nullptr;
  opt.tt_len = is_time_temperature_interpolator_ ? static_cast<int>(tt_time.size()) : 0;
  opt.early_stop = is_early_stop_ ? 1 : 0;
  opt.chain = chain_ ? 1 : 0;
  pred::detail::Check(lmc_kmc_init(dev.ctx(), &temperature_, &opt));

  const bool restarted = steps_ > 0;
  std::ofstream ofs("kmc_log.txt", restarted ? std::ofstream::app : std::ofstream::out);
  ofs.precision(16);
  bool skip_first_dump = restarted;  // McAbstract: the first Dump after a restart is skipped
  const Element solvent = config_.GetSolventElement();
  const double total_solute_mass = config_.GetTotalSoluteMass();
  Vector_d solute_com{0, 0, 0};
  const double L = config_.GetEdge() * kLatticeConstant;
  size_t vacancy = config_.GetVacancyLatticeId();
  const unsigned long long cds = std::max(1ull, config_dump_steps_);
  const double time0 = time_, energy0 = energy_;
  const unsigned long long steps0 = steps_;
  constexpr unsigned long long kChunk = 1 << 16;
  std::vector<lmc_kmc_step> trace;
  bool finished = false;
  while (!finished && steps_ <= maximum_steps_) {
    // a chunk never spans a config dump or the last step: their Dump writes the lattice before the jump
    unsigned long long end = std::min(maximum_steps_ + 1, steps_ + kChunk);
    end = std::min(end, (steps_ / cds + 1) * cds);
    if (steps_ < maximum_steps_) end = std::min(end, maximum_steps_);
    const unsigned long long count = end - steps_;
    trace.assign(count, lmc_kmc_step{});
    pred::detail::Check(lmc_kmc_run(dev.ctx(), count, 0, trace.data(), nullptr));
    uint8_t escaped = 0;
    if (is_early_stop_) pred::detail::Check(lmc_kmc_get_escaped(dev.ctx(), &escaped));
    int64_t vac_dev = 0;
    uint64_t device_steps = 0;
    double t_dev = 0, e_dev = 0;
    pred::detail::Check(lmc_kmc_get_state(dev.ctx(), &vac_dev, &device_steps, &t_dev, &e_dev));
    const unsigned long long executed = device_steps - (steps_ - steps0);
    for (unsigned long long i = 0; i < executed; ++i) {
      const lmc_kmc_step &s = trace[i];
      if (static_cast<size_t>(s.vacancy) != vacancy) throw std::runtime_error("KMC trace out of step with the host");
      const double temp = is_time_temperature_interpolator_ ? time_temperature_interpolator_.GetTemperature(time_)
                                                             : temperature_;
      if (escaped && i + 1 == executed) {
        // IsEscaped (KineticMcAbstract.cpp:192-223), before this step's Dump and jump
        config_.WriteConfig("escaped.cfg.gz");
        std::cout << "t_exit: " << time_ << std::endl;
        std::cout << "steps: " << steps_ << std::endl;
        steps_ = maximum_steps_ + 1;
        finished = true;
      }
      // Dump (KineticMcAbstract.cpp:59-104): the state before this step's jump
      if (skip_first_dump) {
        skip_first_dump = false;
      } else {
        if (steps_ == 0) {
          ofs << "steps\ttime\ttemperature\tenergy\tEa\tdE\tselected\tvac1\tvac2\tvac3";
          if (is_solute_disp_) ofs << "\tsolute_com1\tsolute_com2\tsolute_com3";
          ofs << std::endl;
        }
        if (steps_ % cds == 0) config_.WriteConfig(std::to_string(steps_) + ".cfg.gz");
        if (steps_ == maximum_steps_) config_.WriteConfig("end.cfg.gz");
        if (LogThisStep(steps_, log_dump_steps_)) {
          ofs << steps_ << '\t' << time_ << '\t' << temp << '\t' << energy_ << '\t' << s.ea << '\t' << s.de << '\t'
              << config_.GetAtomIdFromLatticeId(static_cast<size_t>(s.target)) << '\t';
          PutVector(ofs, config_.GetUnwrappedCartesianPositionOfLattice(vacancy));
          if (is_solute_disp_) {
            ofs << '\t';
            PutVector(ofs, solute_com);
          }
          ofs << std::endl;
        }
      }
      // modify (KineticMcAbstract.cpp:154-182)
      const size_t target = static_cast<size_t>(s.target);
      if (is_solute_disp_) {
        const Element jumping = config_.GetElementAtLatticeId(target);
        if (jumping != solvent) {
          const Vector_d a = config_.GetRelativePositionOfLattice(vacancy),
                         b = config_.GetRelativePositionOfLattice(target);
          for (int d = 0; d < 3; ++d) {
            double dd = b[d] - a[d];
            dd -= std::round(dd);  // GetRelativeDistanceVectorLattice: minimum image
            solute_com[d] -= dd * L * (jumping.GetMass() / total_solute_mass);
          }
        }
      }
      time_ = time0 + s.time;
      energy_ = energy0 + s.energy;
      config_.LatticeJump({vacancy, target});
      vacancy = target;
      ++steps_;
    }
    if (executed < count) finished = true;
  }
}

CanonicalMcOmp::CanonicalMcOmp(cfg::Config config, unsigned long long log_dump_steps,
                               unsigned long long config_dump_steps, unsigned long long maximum_steps,
                               unsigned long long thermodynamic_averaging_steps, unsigned long long restart_steps,
                               double restart_energy, double temperature, const std::set<Element> &element_set,
                               const std::string &json_coefficients_filename)
    : config_(std::move(config)),
      log_dump_steps_(log_dump_steps),
      config_dump_steps_(config_dump_steps),
      maximum_steps_(maximum_steps),
      thermodynamic_averaging_steps_(thermodynamic_averaging_steps),
      steps_(restart_steps),
      energy_(restart_energy),
      temperature_(temperature),
      element_set_(element_set),
      json_coefficients_filename_(json_coefficients_filename),
      seed_(ClockSeed()),
      batch_(0) {}

void CanonicalMcOmp::Simulate() {
  pred::detail::Device dev(json_coefficients_filename_, element_set_);
  dev.Sync(config_);
  int batch = batch_;
  if (batch <= 0) {
    const char *env = std::getenv("OMP_NUM_THREADS");
    batch = env ? std::atoi(env) : static_cast<int>(std::thread::hardware_concurrency());
    batch = std::max(1, std::min(batch, 256));
  }
  // McAbstract: absolute energy from EnergyPredictor on the starting configuration
  double absolute0 = 0.0;
  pred::detail::Check(lmc_energy(dev.ctx(), 0, &absolute0, nullptr));
  const double energy0 = energy_;
  const bool restarted = steps_ > 0;
  std::ofstream ofs("cmc_log.txt", restarted ? std::ofstream::app : std::ofstream::out);
  ofs.precision(16);
  bool skip_first_dump = restarted;
  const double beta = 1.0 / kBoltzmann / temperature_;
  ThermodynamicAveraging averaging(thermodynamic_averaging_steps_);
  const unsigned long long cds = std::max(1ull, config_dump_steps_);
  constexpr unsigned long long kChunk = 1 << 20;
  std::vector<double> trace;
  std::vector<int8_t> species(config_.GetNumLattices());
  while (steps_ <= maximum_steps_) {
    const unsigned long long want = std::min(kChunk, maximum_steps_ + 1 - steps_);
    trace.assign(want + batch, 0.0);
    lmc_cmc_options opt{};
    opt.mode = LMC_CMC_REFERENCE_BATCH;
    opt.seed = seed_;
    opt.batch = batch;
    opt.energy_trace = trace.data();
    double e = energy_;
    uint64_t done = 0, accepted = 0;
    // the lattice is read back between chunks (whole batches): config dumps inside a
    // chunk are written from the lattice at the chunk start
    pred::detail::Check(lmc_ctx_get_lattices(dev.ctx(), species.data()));
    config_.SetSpeciesCodes(species, dev.alphabet());
    pred::detail::Check(lmc_cmc_run(dev.ctx(), 0, temperature_, want, &opt, &e, &done, &accepted));
    for (uint64_t i = 0; i < done; ++i) {
      // Simulate loop body (CanonicalMcOmp.cpp:82-90): AddEnergy, Dump, SelectEvent
      const double energy_before = trace[i];
      averaging.AddEnergy(energy_before);
      if (skip_first_dump) {
        skip_first_dump = false;
      } else {
        if (steps_ == 0) ofs << "steps\ttemperature\tenergy\taverage_energy\tabsolute_energy" << std::endl;
        if (steps_ % cds == 0) config_.WriteConfig(std::to_string(steps_) + ".cfg.gz");
        if (steps_ == maximum_steps_) config_.WriteConfig("end.cfg.gz");
        if (LogThisStep(steps_, log_dump_steps_))
          ofs << steps_ << '\t' << temperature_ << '\t' << energy_before << '\t'
              << averaging.GetThermodynamicAverage(beta) << '\t' << absolute0 + (energy_before - energy0)
              << std::endl;
      }
      ++steps_;
    }
    energy_ = e;
  }
  pred::detail::Check(lmc_ctx_get_lattices(dev.ctx(), species.data()));
  config_.SetSpeciesCodes(species, dev.alphabet());
}

SimulatedAnnealing::SimulatedAnnealing(int factor, const Element &solvent_element,
                                       const std::map<Element, size_t> &solute_atom_count,
                                       unsigned long long log_dump_steps, unsigned long long config_dump_steps,
                                       unsigned long long maximum_steps, double initial_temperature,
                                       const std::string &json_coefficients_filename, uint64_t seed)
    : config_(cfg::GenerateSoluteConfig(factor, solvent_element, solute_atom_count, seed + 1)),
      solvent_(solvent_element),
      solute_atom_count_(solute_atom_count),
      log_dump_steps_(log_dump_steps),
      maximum_steps_(maximum_steps),
      initial_temperature_(initial_temperature),
      json_coefficients_filename_(json_coefficients_filename),
      seed_(seed) {
  (void)config_dump_steps;  // the annealing log writes only lowest_energy.cfg.gz
}

void SimulatedAnnealing::Simulate() {
  std::set<Element> element_set{solvent_};
  for (const auto &kv : solute_atom_count_) element_set.insert(kv.first);
  // SimulatedAnnealing constructor (SimulatedAnnealing.cpp:59-72): the cluster's energy relative
  // to the same solutes dissolved in the solvent
  const pred::EnergyPredictor energy_predictor(json_coefficients_filename_, element_set);
  const auto chemical_potential = energy_predictor.GetChemicalPotential(solvent_);
  double energy_change_solution_to_pure_solvent = 0;
  for (const auto &[element, count] : solute_atom_count_)
    energy_change_solution_to_pure_solvent += chemical_potential.at(element) * static_cast<double>(count);
  const double absolute0 = energy_predictor.GetEnergy(config_);
  const double energy_change_cluster_to_pure_solvent =
      absolute0 - energy_predictor.GetEnergy(cfg::Config::GenerateFCC(config_.GetEdge(), solvent_));
  double energy = energy_change_cluster_to_pure_solvent - energy_change_solution_to_pure_solvent;
  std::cout << "initial_energy = " << energy << std::endl;
  double lowest = energy, absolute = absolute0;

  pred::detail::Device dev(json_coefficients_filename_, element_set);
  dev.Sync(config_);
  pred::detail::Check(lmc_sa_init(dev.ctx(), 0, seed_, maximum_steps_, initial_temperature_, energy));
  std::ofstream ofs("sa_log.txt");
  ofs.precision(16);
  constexpr double kEps = 1e-4;  // kEpsilon (VectorMatrix.hpp:65)
  constexpr unsigned long long kChunk = 1 << 16;
  std::vector<lmc_sa_step> trace;
  steps_ = 0;
  while (steps_ <= maximum_steps_) {
    const unsigned long long count = std::min(kChunk, maximum_steps_ + 1 - steps_);
    trace.assign(count, lmc_sa_step{});
    pred::detail::Check(lmc_sa_run(dev.ctx(), count, trace.data()));
    for (const lmc_sa_step &s : trace) {
      // Dump (SimulatedAnnealing.cpp:78-97): the state before this step's move
      if (steps_ == 0) ofs << "steps\ttemperature\tenergy\tlowest_energy\tabsolute_energy" << std::endl;
      if (energy < lowest - kEps) {
        lowest = energy;
        config_.WriteConfig("lowest_energy.cfg.gz");
        ofs << steps_ << '\t' << s.temperature << '\t' << energy << '\t' << lowest << '\t' << absolute << std::endl;
      }
      if (steps_ % std::max(1ull, log_dump_steps_) == 0)
        ofs << steps_ << '\t' << s.temperature << '\t' << energy << '\t' << lowest << '\t' << absolute << std::endl;
      if (s.accepted) {
        config_.LatticeJump({static_cast<size_t>(s.site1), static_cast<size_t>(s.site2)});
        energy += s.de;
        absolute += s.de;
      }
      ++steps_;
    }
  }
}

}  // namespace mc

// ---------------------------------------------------------------------------
// api
// ---------------------------------------------------------------------------
namespace api {

Parameter::Parameter(int argc, char *argv[]) {
  ParseArgs(argc, argv);
  ReadParam(parameters_filename);
}

Parameter::Parameter(const std::string &param_filename) { ReadParam(param_filename); }

void Parameter::ParseArgs(int argc, char *argv[]) {
  for (int i = 0; i < argc; ++i)
    if ((!std::strcmp(argv[i], "--p") || !std::strcmp(argv[i], "-p")) && i + 1 < argc)
      parameters_filename = std::string(argv[++i]);
}

void Parameter::ReadParam(const std::string &param_filename) {
  if (param_filename.empty()) return;
  std::ifstream ifs(param_filename);
  if (!ifs.is_open()) throw std::runtime_error("Cannot open " + param_filename);
  std::string line;
  const auto flag = [](const std::string &v) { return v == "true"; };
  while (std::getline(ifs, line)) {
    if (line.empty() || line[0] == '#') continue;
    const auto segs = Split(line);
    if (segs.size() < 2) continue;
    const std::string &k = segs[0], &v = segs[1];
    if (k == "simulation_method") method = v;
    else if (k == "config_filename") config_filename_ = v;
    else if (k == "map_filename") map_filename_ = v;
    else if (k == "json_coefficients_filename") json_coefficients_filename_ = v;
    else if (k == "time_temperature_filename") time_temperature_filename_ = v;
    else if (k == "log_type") log_type_ = v;
    else if (k == "config_type") config_type_ = v;
    else if (k == "log_dump_steps") log_dump_steps_ = std::stoull(v);
    else if (k == "config_dump_steps") config_dump_steps_ = std::stoull(v);
    else if (k == "maximum_steps") maximum_steps_ = std::stoull(v);
    else if (k == "thermodynamic_averaging_steps") thermodynamic_averaging_steps_ = std::stoull(v);
    else if (k == "temperature") temperature_ = std::stod(v);
    else if (k == "element_set") element_set_.assign(segs.begin() + 1, segs.end());
    else if (k == "restart_steps") restart_steps_ = std::stoull(v);
    else if (k == "rate_corrector") rate_corrector_ = flag(v);
    else if (k == "early_stop") early_stop_ = flag(v);
    else if (k == "solute_disp") solute_disp_ = flag(v);
    else if (k == "restart_energy") restart_energy_ = std::stod(v);
    else if (k == "restart_time") restart_time_ = std::stod(v);
    else if (k == "seed") {
      seed_ = std::stoull(v);
      has_seed_ = true;
    } else if (k == "cmc_batch") cmc_batch_ = std::stoi(v);
    else if (k == "factor") factor_ = std::stoi(v);
    else if (k == "solvent_element") solvent_element_ = v;
    else if (k == "solute_element_set") solute_element_set_.assign(segs.begin() + 1, segs.end());
    else if (k == "solute_number_set") {
      solute_number_set_.clear();
      for (size_t q = 1; q < segs.size(); ++q) solute_number_set_.push_back(std::stoull(segs[q]));
    } else if (k == "initial_temperature") initial_temperature_ = std::stod(v);
    else if (k == "decrement_temperature") decrement_temperature_ = std::stod(v);
    else if (k == "escape_temperature") escape_temperature_ = std::stod(v);
    else if (k == "initial_steps") initial_steps_ = std::stoull(v);
    else if (k == "increment_steps") increment_steps_ = std::stoull(v);
    else if (k == "early_stop_steps") early_stop_steps_ = std::stoull(v);
    else if (k == "smallest_cluster_criteria") smallest_cluster_criteria_ = std::stoul(v);
    else if (k == "solvent_bond_criteria") solvent_bond_criteria_ = std::stoul(v);
    // the remaining keys of the reference's grammar (vacancy_trajectory) are commented out there
  }
}

void Run(const Parameter &p) {
  std::set<Element> element_set;
  for (const auto &e : p.element_set_) element_set.insert(Element(e));
  if (p.method == "SimulatedAnnealing") {
    // BuildSimulatedAnnealingFromParameter (Home.cpp:223-240)
    std::map<Element, size_t> solute_atom_count;
    for (size_t i = 0; i < p.solute_element_set_.size() && i < p.solute_number_set_.size(); ++i)
      solute_atom_count.emplace(Element(p.solute_element_set_[i]), p.solute_number_set_[i]);
    mc::SimulatedAnnealing sa(p.factor_, Element(p.solvent_element_), solute_atom_count, p.log_dump_steps_,
                              p.config_dump_steps_, p.maximum_steps_, p.initial_temperature_,
                              p.json_coefficients_filename_, p.has_seed_ ? p.seed_ : mc::ClockSeedValue());
    sa.Simulate();
    return;
  }
  if (p.method != "KineticMcFirstOmp" && p.method != "KineticMcChainOmpi" && p.method != "CanonicalMcOmp") {
    std::cout << "No such method: " << p.method << std::endl;
    return;
  }
  // Home.cpp:165-170: a CFG file (reassigned), or the map files lattice.txt / element.txt / map_filename
  cfg::Config config;
  if (p.map_filename_.empty()) {
    config = cfg::Config::ReadConfig(p.config_filename_);
    config.ReassignLatticeVector();
  } else {
    config = cfg::Config::ReadMap("lattice.txt", "element.txt", p.map_filename_);
  }
  if (p.method == "KineticMcFirstOmp") {
    std::cout << "Finish config reading. Start KMC." << std::endl;
    mc::KineticMcFirstOmp kmc(config, p.log_dump_steps_, p.config_dump_steps_, p.maximum_steps_,
                              p.thermodynamic_averaging_steps_, p.restart_steps_, p.restart_energy_, p.restart_time_,
                              p.temperature_, element_set, p.json_coefficients_filename_,
                              p.time_temperature_filename_, p.rate_corrector_, p.early_stop_, p.solute_disp_);
    if (p.has_seed_) kmc.SetSeed(p.seed_);
    kmc.Simulate();
  } else if (p.method == "KineticMcChainOmpi") {
    std::cout << "Finish config reading. Start KMC." << std::endl;
    mc::KineticMcChainOmpi kmc(config, p.log_dump_steps_, p.config_dump_steps_, p.maximum_steps_,
                               p.thermodynamic_averaging_steps_, p.restart_steps_, p.restart_energy_,
                               p.restart_time_, p.temperature_, element_set, p.json_coefficients_filename_,
                               p.time_temperature_filename_, p.rate_corrector_, p.early_stop_, p.solute_disp_);
    if (p.has_seed_) kmc.SetSeed(p.seed_);
    kmc.Simulate();
  } else {
    std::cout << "Finish config reading. Start CMC." << std::endl;
    mc::CanonicalMcOmp cmc(config, p.log_dump_steps_, p.config_dump_steps_, p.maximum_steps_,
                           p.thermodynamic_averaging_steps_, p.restart_steps_, p.restart_energy_, p.temperature_,
                           element_set, p.json_coefficients_filename_);
    if (p.has_seed_) cmc.SetSeed(p.seed_);
    if (p.cmc_batch_ > 0) cmc.SetBatch(p.cmc_batch_);
    cmc.Simulate();
  }
}

}  // namespace api
