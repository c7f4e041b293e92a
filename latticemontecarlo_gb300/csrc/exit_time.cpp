// ansys::ExitTime's per-cluster quantities over the GPU's barrier lists:
// the Markov-chain escape time of a vacancy from a cluster and its shell
// (ExitTime::BuildMarkovChain, lmc/ansys/src/ExitTime.cpp:165-216), the
// neighbour-shell size, the mean and spread of the barriers inside, into, on
// and off the cluster (ExitTime::GetAverageBarriers, ExitTime.cpp:311-399) and
// the effective binding energy (ExitTime.cpp:118-122).
//
// The barriers come from lmc_site_jump_energetics (one GPU warp per site, the
// lattice's vacancy filled with the solvent and the vacancy placed on the
// site, as ExitTime::GetJumpEnergetics does, ExitTime.cpp:217-310) for the
// union of every cluster and its first-neighbour shell. The linear system of
// each chain, (I - Q) x = tau with Q the transient-to-transient jump
// probabilities and tau the mean residence times, is solved on the host by LU
// with partial pivoting; clusters are spread over the host's threads.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <limits>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/lmc_gb300.h"
#include "abi_common.hpp"
#include "geometry.hpp"

using lmc::abi::Guard;
using lmc::abi::LmcError;
using lmc::abi::Require;

namespace {

constexpr double kBoltzmannEv = 8.617333262145e-5;  // lmc/cfg/include/Constants.hpp:31
constexpr double kPrefactorHz = 1e13;               // lmc/cfg/include/Constants.hpp:32
constexpr int64_t kMaxTransient = 4096;             // dense LU: 4096^2 doubles = 128 MiB per thread

// Solves a x = b in place (a: m x m row-major, overwritten; b -> x). Returns false if singular.
bool LuSolve(std::vector<double> &a, std::vector<double> &b, int64_t m) {
  for (int64_t k = 0; k < m; ++k) {
    int64_t p = k;
    double best = std::fabs(a[k * m + k]);
    for (int64_t i = k + 1; i < m; ++i) {
      const double v = std::fabs(a[i * m + k]);
      if (v > best) {
        best = v;
        p = i;
      }
    }
    if (!(best > 0.0)) return false;
    if (p != k) {
      for (int64_t j = 0; j < m; ++j) std::swap(a[k * m + j], a[p * m + j]);
      std::swap(b[k], b[p]);
    }
    const double inv = 1.0 / a[k * m + k];
    for (int64_t i = k + 1; i < m; ++i) {
      const double f = a[i * m + k] * inv;
      if (f == 0.0) continue;
      a[i * m + k] = f;
      const double *rk = &a[k * m];
      double *ri = &a[i * m];
      for (int64_t j = k + 1; j < m; ++j) ri[j] -= f * rk[j];
      b[i] -= f * b[k];
    }
  }
  for (int64_t k = m - 1; k >= 0; --k) {
    double s = b[k];
    for (int64_t j = k + 1; j < m; ++j) s -= a[k * m + j] * b[j];
    b[k] = s / a[k * m + k];
  }
  return true;
}

struct SiteJumps {
  std::unordered_map<int64_t, int64_t> row;  // site -> row of the arrays below
  std::vector<double> ea, de;                // [rows][12]
  std::vector<int64_t> nb;                   // [rows][12] adjacency-list order
};

// Mean and population standard deviation (NaN for an empty list), as GetAverageBarriers.
void MeanStd(const std::vector<double> &v, double *mean, double *sd) {
  if (v.empty()) {
    *mean = *sd = std::nan("");
    return;
  }
  double s = 0.0;
  for (double x : v) s += x;
  const double mu = s / static_cast<double>(v.size());
  double q = 0.0;
  for (double x : v) q += (x - mu) * (x - mu);
  *mean = mu;
  *sd = std::sqrt(q / static_cast<double>(v.size()));
}

// One cluster: returns false when its chain exceeds kMaxTransient states or is singular.
bool OneCluster(const lmc::Fcc &fcc, const SiteJumps &sj, const int64_t *members, int64_t count,
                const double *profile, double beta, double *escape, int64_t *neighbor_size, double *barriers8) {
  std::vector<int64_t> in(members, members + count);
  std::sort(in.begin(), in.end());
  std::vector<int64_t> all = in;
  for (int64_t s : in)
    for (int64_t j : lmc::SortedNeighbors(fcc, s, 1)) all.push_back(j);
  std::sort(all.begin(), all.end());
  all.erase(std::unique(all.begin(), all.end()), all.end());
  const int64_t m = static_cast<int64_t>(all.size());
  *neighbor_size = m - static_cast<int64_t>(in.size());
  auto index_of = [&](int64_t site) -> int64_t {
    const auto it = std::lower_bound(all.begin(), all.end(), site);
    return (it != all.end() && *it == site) ? it - all.begin() : -1;
  };
  auto in_cluster = [&](int64_t site) { return std::binary_search(in.begin(), in.end(), site); };
  // GetAverageBarriers: Ea - dE / 2 of every jump out of a site of the cluster or its shell
  std::vector<double> lists[4];  // in, to, on, off
  for (int64_t l : all) {
    const int64_t r = sj.row.at(l);
    const bool l_in = in_cluster(l);
    for (int q = 0; q < 12; ++q) {
      const int64_t nbq = sj.nb[r * 12 + q];
      const bool nb_in = in_cluster(nbq), nb_nn = index_of(nbq) >= 0;
      int cat = -1;
      if (l_in && nb_in) cat = 0;
      else if (l_in && !nb_in && nb_nn) cat = 1;
      else if (!l_in && !nb_in && nb_nn) cat = 2;
      else if (!l_in && !nb_nn) cat = 3;
      if (cat >= 0) lists[cat].push_back(sj.ea[r * 12 + q] - sj.de[r * 12 + q] / 2);
    }
  }
  for (int c = 0; c < 4; ++c) MeanStd(lists[c], &barriers8[c], &barriers8[4 + c]);
  if (m > kMaxTransient) return false;
  // BuildMarkovChain: start in state i with probability ~ exp(-profile_i beta); from i the 12
  // jumps with rates 1e13 exp(-Ea beta); jumps leaving the set are absorbing
  std::vector<double> a(static_cast<size_t>(m * m), 0.0), tau(m), p(m);
  double psum = 0.0;
  for (int64_t i = 0; i < m; ++i) {
    const int64_t r = sj.row.at(all[i]);
    p[i] = std::exp(-profile[all[i]] * beta);
    psum += p[i];
    double rates[12], total = 0.0;
    for (int q = 0; q < 12; ++q) {
      rates[q] = kPrefactorHz * std::exp(-sj.ea[r * 12 + q] * beta);
      total += rates[q];
    }
    tau[i] = 1.0 / total;
    a[i * m + i] = 1.0;
    for (int q = 0; q < 12; ++q) {
      const int64_t j = index_of(sj.nb[r * 12 + q]);
      if (j >= 0) a[i * m + j] -= rates[q] / total;
    }
  }
  if (!LuSolve(a, tau, m)) return false;
  double t = 0.0;
  for (int64_t i = 0; i < m; ++i) t += p[i] / psum * tau[i];
  *escape = t;
  return true;
}

}  // namespace

int lmc_exit_time_clusters(lmc_ctx *ctx, int replica, int solvent_code, double escape_temperature,
                           const int64_t *offsets, const int64_t *members, int64_t num_clusters,
                           const double *profile_energy, double *markov_escape_time, int64_t *neighbor_size,
                           double *barriers, double *effective_binding_energy) {
  return Guard([&] {
    Require(ctx && offsets && profile_energy && num_clusters >= 0 && (members || num_clusters == 0),
            LMC_ERR_INVALID_ARGUMENT, "bad argument");
    Require(escape_temperature > 0, LMC_ERR_INVALID_ARGUMENT, "escape_temperature must be > 0");
    if (num_clusters == 0) return;
    const int64_t off = lmc_ctx_replica_offset(ctx, replica);
    Require(off >= 0, LMC_ERR_OUT_OF_RANGE, "replica out of range");
    const int64_t next_off =
        lmc_ctx_replica_offset(ctx, replica + 1) >= 0 ? lmc_ctx_replica_offset(ctx, replica + 1) : lmc_ctx_total_sites(ctx);
    const int n = static_cast<int>(std::llround(std::cbrt(static_cast<double>(next_off - off) / 4.0)));
    Require(4LL * n * n * n == next_off - off, LMC_ERR_INVALID_ARGUMENT, "replica is not a cubic supercell");
    const lmc::Fcc fcc{n};
    const int64_t nsites = fcc.NumSites();
    Require(offsets[0] == 0, LMC_ERR_INVALID_ARGUMENT, "offsets[0] must be 0");
    for (int64_t c = 0; c < num_clusters; ++c)
      Require(offsets[c + 1] > offsets[c], LMC_ERR_INVALID_ARGUMENT, "empty cluster");
    for (int64_t k = 0; k < offsets[num_clusters]; ++k)
      Require(members[k] >= 0 && members[k] < nsites, LMC_ERR_OUT_OF_RANGE, "cluster site out of range");
    // the union of the clusters and their first-neighbour shells: the sites whose 12 barriers the
    // chains and the averages read (GetJumpEnergetics' lattice_id_set_plus_nn)
    std::vector<int64_t> sites;
    for (int64_t k = 0; k < offsets[num_clusters]; ++k) {
      sites.push_back(members[k]);
      for (int64_t j : lmc::SortedNeighbors(fcc, members[k], 1)) sites.push_back(j);
    }
    std::sort(sites.begin(), sites.end());
    sites.erase(std::unique(sites.begin(), sites.end()), sites.end());
    const int64_t m = static_cast<int64_t>(sites.size());
    SiteJumps sj;
    sj.ea.resize(12 * m);
    sj.de.resize(12 * m);
    sj.nb.resize(12 * m);
    const int rc = lmc_site_jump_energetics(ctx, replica, LMC_BARRIER_QUARTIC, solvent_code, escape_temperature,
                                            sites.data(), m, sj.ea.data(), sj.de.data(), sj.nb.data(), nullptr,
                                            nullptr);
    if (rc != LMC_OK) throw LmcError(rc, lmc_last_error());
    sj.row.reserve(2 * m);
    for (int64_t i = 0; i < m; ++i) sj.row.emplace(sites[i], i);
    const double beta = 1.0 / kBoltzmannEv / escape_temperature;
    std::vector<double> esc(num_clusters, std::nan("")), bar(8 * num_clusters, std::nan(""));
    std::vector<int64_t> nsz(num_clusters, 0);
    std::vector<char> ok(num_clusters, 1);
    std::atomic<int64_t> next{0};
    auto work = [&] {
      for (int64_t c; (c = next.fetch_add(1)) < num_clusters;)
        ok[c] = OneCluster(fcc, sj, members + offsets[c], offsets[c + 1] - offsets[c], profile_energy, beta,
                           &esc[c], &nsz[c], &bar[8 * c]);
    };
    const unsigned threads = std::max(1u, std::min(std::thread::hardware_concurrency(), 32u));
    std::vector<std::thread> pool;
    for (unsigned t = 1; t < threads && t < num_clusters; ++t) pool.emplace_back(work);
    work();
    for (auto &th : pool) th.join();
    for (int64_t c = 0; c < num_clusters; ++c)
      Require(ok[c], LMC_ERR_UNSUPPORTED,
              "cluster " + std::to_string(c) + ": more than " + std::to_string(kMaxTransient) +
                  " sites with its shell, or a chain without escape");
    for (int64_t c = 0; c < num_clusters; ++c) {
      if (markov_escape_time) markov_escape_time[c] = esc[c];
      if (neighbor_size) neighbor_size[c] = nsz[c];
      if (barriers) std::copy(&bar[8 * c], &bar[8 * c] + 8, barriers + 8 * c);
      // ExitTime.cpp:121: -ln(t 1e13) / beta + the mean barrier of the jumps off the shell
      if (effective_binding_energy)
        effective_binding_energy[c] = -std::log(esc[c] * kPrefactorHz) / beta + bar[8 * c + 3];
    }
  });
}
