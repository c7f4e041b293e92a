"""Seeded synthetic inputs: FCC species lattices and coefficient files.

The reference ships no coefficient file, configuration or benchmark dataset,
so every workload here is generated from a seed with numpy's PCG64
(``np.random.default_rng(seed)``), which gives identical values on x86-64 and
aarch64.

Coefficients follow the layout the reference's predictors read
(lmc/pred/src/VacancyMigrationPredictorQuartic.cpp:38-63,
lmc/pred/src/VacancyMigrationPredictorE0.cpp:22-40):

* ``"Base": {"theta": [...]}`` -- cluster-expansion ECIs in ElementCluster
  order; pair ECIs (labels 1-3) and first-shell triplets (label 4) drawn from
  N(0, 0.02) eV, all other entries 0.
* one block per element with the Quartic keys (mu_x_mmm, sigma_x_mmm,
  mu_x_mm2, sigma_x_mm2, U_mmm, U_mm2, theta_D, theta_Ks, mu_D, mu_Ks, sigma_D,
  sigma_Ks) and the E0 keys (theta_e0, mu_e0, sigma_e0): mu_x ~ U(0, 1),
  sigma_x ~ U(0.5, 1.5), U ~ N(0, 1/sqrt(F)) with k rows, theta scaled so the
  barrier spread over environments of the given composition is about
  ``ea_std`` eV, and mu_D / mu_Ks / mu_e0 set so a pure-solvent environment
  has D = 2.86 and Ea = ``ea0`` eV (Ea(dE=0) = Ks D^2 / 64).
"""
from __future__ import annotations

import math

import numpy as np

from .api import Model

DEFAULT_K = 64


def alphabet(elements) -> list[str]:
    return sorted(set(elements) | {"X"})


def theta_labels(elements) -> list[int]:
    """Cluster label of every "Base".theta entry (ElementCluster map order)."""
    alpha = alphabet(elements)
    x = alpha.index("X")
    keys = set()
    for c1 in range(len(alpha)):
        keys.add((1, 0, (c1,)))
    for c1 in range(len(alpha)):
        for c2 in range(len(alpha)):
            if c2 == x:
                continue
            for label in (1, 2, 3):
                keys.add((2, label, tuple(sorted((c1, c2)))))
            for c3 in range(len(alpha)):
                if c3 == x:
                    continue
                for label in (4, 5, 6, 7):
                    keys.add((3, label, tuple(sorted((c1, c2, c3)))))
    return [k[1] for k in sorted(keys)]


def make_lattice(n: int, fractions: dict, vacancies: int, seed: int, elements) -> np.ndarray:
    """Species codes of an n^3 FCC supercell in lattice-id order: i.i.d. draws
    from `fractions` (element -> fraction), then exactly `vacancies` X sites at
    seeded uniform positions."""
    rng = np.random.default_rng(seed)
    alpha = alphabet(elements)
    names = list(fractions)
    p = np.asarray([fractions[k] for k in names], np.float64)
    p = p / p.sum()
    nsites = 4 * n ** 3
    idx = rng.choice(len(names), size=nsites, p=p)
    codes = np.asarray([alpha.index(nm) for nm in names], np.int8)
    sp = codes[idx].astype(np.int8)
    if vacancies:
        pos = rng.choice(nsites, size=vacancies, replace=False)
        sp[pos] = alpha.index("X")
    return sp


def _nn1_pairs(n: int, count: int, rng) -> np.ndarray:
    """Random (site, 1NN neighbour) pairs of an n^3 supercell (closed-form ids)."""
    plane = 2 * n * n
    sites = rng.integers(0, 4 * n ** 3, size=count)
    hx, r = sites // plane, sites % plane
    hy, k = r // n, r % n
    hz = 2 * k + ((hx + hy) & 1)
    dirs = np.array([(x, y, z) for x in (-1, 0, 1) for y in (-1, 0, 1) for z in (-1, 0, 1)
                     if (x * x + y * y + z * z) == 2])
    d = dirs[rng.integers(0, 12, size=count)]
    m = 2 * n
    jx, jy, jz = (hx + d[:, 0]) % m, (hy + d[:, 1]) % m, (hz + d[:, 2]) % m
    j = jx * plane + jy * n + jz // 2
    return np.stack([sites, j], axis=1).astype(np.int64)


def make_coefficients(elements, seed: int, k: int = DEFAULT_K, pair_eci_std: float = 0.02,
                      ea0: float = 0.6, ea_std: float = 0.05, d0: float = 2.86,
                      calib_fractions: dict | None = None, calib_samples: int = 256,
                      calibrate: bool = True, theta_scale: float = 0.02) -> dict:
    """Coefficient dict for `elements`. With calibrate=False the theta vectors
    are N(0, theta_scale) and mu_D / mu_Ks / mu_e0 take their nominal values,
    so the result depends on numpy alone (used for pinned test fixtures)."""
    elements = sorted(set(elements))
    rng = np.random.default_rng(seed)
    model = Model.create(elements)
    if not calibrate:
        return _plain_coefficients(model, elements, rng, k, pair_eci_std, ea0, d0, theta_scale)
    labels = np.asarray(theta_labels(elements))
    theta = np.zeros(model.num_theta)
    mask = (labels >= 1) & (labels <= 4)
    theta[mask] = rng.normal(0.0, pair_eci_std, size=int(mask.sum()))
    sizes_mmm = model.orbit_sizes(0).astype(np.float64)
    sizes_mm2 = model.orbit_sizes(1).astype(np.float64)
    # calibration environments: random lattice of the requested composition, no vacancy
    solvent = "Al" if "Al" in elements else elements[0]
    if calib_fractions is None:
        calib_fractions = {e: (0.96 if e == solvent else 0.04 / max(1, len(elements) - 1)) for e in elements}
    n_cal = 10
    sp = make_lattice(n_cal, calib_fractions, 0, seed + 1, elements)
    pure = np.full_like(sp, model.code(solvent))
    pairs = _nn1_pairs(n_cal, calib_samples, rng)
    feats_mmm, feats_mm2 = [], []
    for a, b in pairs:
        _, _, mm, mf, mb = model.host_encode_pair(n_cal, sp, int(a), int(b))
        feats_mmm.append(mm / sizes_mmm)
        feats_mm2.append((mf + mb) / sizes_mm2)
    # site 0 and site n are first neighbours (half-lattice offset (0, 1, 1))
    _, _, mm, mf, mb = model.host_encode_pair(n_cal, pure, 0, n_cal)
    x_mmm = np.asarray(feats_mmm)
    x_mm2 = np.asarray(feats_mm2)
    coeffs = {"Base": {"theta": theta.tolist()}}
    for el in elements:
        f_mmm, f_mm2 = model.f_mmm, model.f_mm2
        mu_mmm = rng.uniform(0.0, 1.0, f_mmm)
        sg_mmm = rng.uniform(0.5, 1.5, f_mmm)
        mu_mm2 = rng.uniform(0.0, 1.0, f_mm2)
        sg_mm2 = rng.uniform(0.5, 1.5, f_mm2)
        u_mmm = rng.normal(0.0, 1.0 / math.sqrt(f_mmm), (k, f_mmm))
        u_mm2 = rng.normal(0.0, 1.0 / math.sqrt(f_mm2), (k, f_mm2))
        th_d = rng.normal(0.0, 1.0, k)
        th_ks = rng.normal(0.0, 1.0, k)
        th_e0 = rng.normal(0.0, 1.0, k)

        def lin(x, mu, sg, u, th):
            return ((x - mu) / sg) @ u.T @ th

        l_d, l_ks, l_e0 = lin(x_mmm, mu_mmm, sg_mmm, u_mmm, th_d), lin(x_mm2, mu_mm2, sg_mm2, u_mm2, th_ks), \
            lin(x_mmm, mu_mmm, sg_mmm, u_mmm, th_e0)
        # log Ea(dE=0) = log Ks + 2 log D - log 64: scale theta so its spread is ea_std / ea0
        spread = float(np.std(2.0 * l_d + l_ks))
        s = (ea_std / ea0) / spread if spread > 0 else 1.0
        spread_e0 = float(np.std(l_e0))
        s_e0 = (ea_std / ea0) / spread_e0 if spread_e0 > 0 else 1.0
        th_d, th_ks, th_e0 = th_d * s, th_ks * s, th_e0 * s_e0
        x_pure_mmm = mm / sizes_mmm
        x_pure_mm2 = (mf + mb) / sizes_mm2
        p_d = float(lin(x_pure_mmm, mu_mmm, sg_mmm, u_mmm, th_d))
        p_ks = float(lin(x_pure_mm2, mu_mm2, sg_mm2, u_mm2, th_ks))
        p_e0 = float(lin(x_pure_mmm, mu_mmm, sg_mmm, u_mmm, th_e0))
        coeffs[el] = {
            "mu_x_mmm": mu_mmm.tolist(), "sigma_x_mmm": sg_mmm.tolist(),
            "mu_x_mm2": mu_mm2.tolist(), "sigma_x_mm2": sg_mm2.tolist(),
            "U_mmm": u_mmm.tolist(), "U_mm2": u_mm2.tolist(),
            "theta_D": th_d.tolist(), "theta_Ks": th_ks.tolist(),
            "mu_D": math.log(d0) - p_d, "sigma_D": 1.0,
            "mu_Ks": math.log(64.0 * ea0 / d0 ** 2) - p_ks, "sigma_Ks": 1.0,
            "theta_e0": th_e0.tolist(), "mu_e0": math.log(ea0) - p_e0, "sigma_e0": 1.0,
        }
    return coeffs


def _plain_coefficients(model, elements, rng, k, pair_eci_std, ea0, d0, theta_scale) -> dict:
    labels = np.asarray(theta_labels(elements))
    theta = np.zeros(model.num_theta)
    mask = (labels >= 1) & (labels <= 4)
    theta[mask] = rng.normal(0.0, pair_eci_std, size=int(mask.sum()))
    coeffs = {"Base": {"theta": theta.tolist()}}
    for el in elements:
        f_mmm, f_mm2 = model.f_mmm, model.f_mm2
        coeffs[el] = {
            "mu_x_mmm": rng.uniform(0.0, 1.0, f_mmm).tolist(), "sigma_x_mmm": rng.uniform(0.5, 1.5, f_mmm).tolist(),
            "mu_x_mm2": rng.uniform(0.0, 1.0, f_mm2).tolist(), "sigma_x_mm2": rng.uniform(0.5, 1.5, f_mm2).tolist(),
            "U_mmm": rng.normal(0.0, 1.0 / math.sqrt(f_mmm), (k, f_mmm)).tolist(),
            "U_mm2": rng.normal(0.0, 1.0 / math.sqrt(f_mm2), (k, f_mm2)).tolist(),
            "theta_D": rng.normal(0.0, theta_scale, k).tolist(), "theta_Ks": rng.normal(0.0, theta_scale, k).tolist(),
            "mu_D": math.log(d0), "sigma_D": 1.0, "mu_Ks": math.log(64.0 * ea0 / d0 ** 2), "sigma_Ks": 1.0,
            "theta_e0": rng.normal(0.0, theta_scale, k).tolist(), "mu_e0": math.log(ea0), "sigma_e0": 1.0,
        }
    return coeffs


# Workloads of the benchmark configurations (sizes and compositions).
KMC_SINGLE = dict(n=10, fractions={"Al": 0.96, "Mg": 0.02, "Zn": 0.02}, vacancies=1, T=400.0, steps=100_000,
                  elements=("Al", "Mg", "Zn"))
CMC_SINGLE = dict(n=30, fractions={"Al": 0.94, "Mg": 0.02, "Zn": 0.02, "Cu": 0.02}, T=500.0, sweeps=1000,
                  elements=("Al", "Cu", "Mg", "Zn"))
KMC_BATCHED = dict(replicas=4096, n_range=(8, 24), fractions={"Al": 0.96, "Mg": 0.02, "Zn": 0.02},
                   T_range=(350.0, 550.0), steps=10_000, elements=("Al", "Mg", "Zn"))
LARGE = dict(n=64, fractions={"Al": 0.93, "Mg": 0.03, "Zn": 0.03, "Cu": 0.01}, vacancies=64,
             elements=("Al", "Cu", "Mg", "Zn"))


def batched_replicas(seed: int, replicas: int, n_range=(8, 24), fractions=None, T_range=(350.0, 550.0),
                     elements=("Al", "Mg", "Zn")):
    """Edges n_r ~ U{n_lo..n_hi}, temperatures ~ U(T_lo, T_hi), one vacancy each.
    Returns (ns int32, species int8 concatenated, temperatures float64)."""
    rng = np.random.default_rng(seed)
    fractions = fractions or KMC_BATCHED["fractions"]
    ns = rng.integers(n_range[0], n_range[1] + 1, size=replicas).astype(np.int32)
    temps = rng.uniform(T_range[0], T_range[1], size=replicas)
    parts = [make_lattice(int(n), fractions, 1, seed * 100003 + r, elements) for r, n in enumerate(ns)]
    return ns, np.concatenate(parts), temps
