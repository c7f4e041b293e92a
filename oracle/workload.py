"""TEST ORACLE inputs: the benchmark's seeded synthetic workloads rebuilt from
numpy and the oracle alone.

Test infrastructure only: bench.py's CPU legs (``--impl reference`` and the
``cpu_baseline`` of the GPU arm) use it so that the timed CPU code never loads
the product library. It restates, value for value, the product's generator of
synthetic inputs (lattices from numpy's PCG64, calibrated coefficient blocks),
with the oracle's restated encoder (orc_encode) in place of the product's; a CPU
test checks that both give identical lattices and coefficients.

The coefficient layout is the one the reference's predictors read
(lmc/pred/src/VacancyMigrationPredictorQuartic.cpp:38-63,
lmc/pred/src/VacancyMigrationPredictorE0.cpp:22-40).
"""
from __future__ import annotations

import math

import numpy as np

from . import oracle as O

# benchmark configurations (sizes and compositions)
KMC_BATCHED = dict(replicas=4096, n_range=(8, 24), fractions={"Al": 0.96, "Mg": 0.02, "Zn": 0.02},
                   T_range=(350.0, 550.0), steps=10_000, elements=("Al", "Mg", "Zn"))
CMC_SINGLE = dict(n=30, fractions={"Al": 0.94, "Mg": 0.02, "Zn": 0.02, "Cu": 0.02}, T=500.0, sweeps=1000,
                  elements=("Al", "Cu", "Mg", "Zn"))


def alphabet(elements) -> list[str]:
    return sorted(set(elements) | {"X"})


def theta_labels(elements) -> list[int]:
    """Cluster label of every "Base".theta entry: ElementCluster order (size, label, sorted codes;
    ElementCluster.hpp:40-50) over the clusters InitializeClusterHashMap enumerates
    (EnergyUtility.cpp:314-343)."""
    alpha = alphabet(elements)
    x = alpha.index("X")
    keys = {(1, 0, (c,)) for c in range(len(alpha))}
    for c1 in range(len(alpha)):
        for c2 in range(len(alpha)):
            if c2 == x:
                continue
            keys.update((2, lab, tuple(sorted((c1, c2)))) for lab in (1, 2, 3))
            for c3 in range(len(alpha)):
                if c3 != x:
                    keys.update((3, lab, tuple(sorted((c1, c2, c3)))) for lab in (4, 5, 6, 7))
    return [k[1] for k in sorted(keys)]


def make_lattice(n: int, fractions: dict, vacancies: int, seed: int, elements) -> np.ndarray:
    """Species codes of an n^3 FCC supercell in lattice-id order: i.i.d. draws from `fractions`, then
    exactly `vacancies` X sites at seeded uniform positions."""
    rng = np.random.default_rng(seed)
    alpha = alphabet(elements)
    names = list(fractions)
    p = np.asarray([fractions[k] for k in names], np.float64)
    p = p / p.sum()
    nsites = 4 * n ** 3
    sp = np.asarray([alpha.index(nm) for nm in names], np.int8)[rng.choice(len(names), size=nsites, p=p)]
    if vacancies:
        sp[rng.choice(nsites, size=vacancies, replace=False)] = alpha.index("X")
    return sp


def batched_edges_and_temperatures(seed: int, replicas: int, n_range=(8, 24), T_range=(350.0, 550.0)):
    rng = np.random.default_rng(seed)
    ns = rng.integers(n_range[0], n_range[1] + 1, size=replicas).astype(np.int32)
    temps = rng.uniform(T_range[0], T_range[1], size=replicas)
    return ns, temps


def batched_replica_lattice(seed: int, r: int, n: int, fractions=None, elements=("Al", "Mg", "Zn")) -> np.ndarray:
    """Replica r's lattice of the batched workload (one vacancy, its own seed)."""
    return make_lattice(int(n), fractions or KMC_BATCHED["fractions"], 1, seed * 100003 + r, elements)


def _nn1_pairs(n: int, count: int, rng) -> np.ndarray:
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
    return np.stack([sites, jx * plane + jy * n + jz // 2], axis=1).astype(np.int64)


class _Encoder:
    """The oracle's encoder with an all-zero theta (the encodings do not depend on coefficients)."""

    def __init__(self, elements, lat: O.Lattice):
        import ctypes as C
        names = (C.c_char_p * len(elements))(*[e.encode() for e in elements])
        h = O.lib().orc_model_create(names, len(elements))
        nt = O.lib().orc_model_num_theta(h)
        O.lib().orc_model_destroy(h)
        self.model = O.Model(elements, {"Base": {"theta": [0.0] * nt}}, lat)
        self.lat = lat
        e = len(elements)
        self.sizes = [self._orbit_sizes(lat.mapping(w), e) for w in (2, 3)]

    @staticmethod
    def _orbit_sizes(records, e):
        """Per feature, the size of its orbit (list length e, e^2 or e(e+1)/2 per orbit,
        GetOneHotParametersFromMap, EnergyUtility.cpp:753-792)."""
        out = []
        groups = records[:, 0]
        for g in range(int(groups.max()) + 1):
            r = records[groups == g]
            size, sym = int(r[0, 1]), int(r[0, 2])
            width = e if size == 1 else (e * (e + 1) // 2 if sym else e * e)
            out += [len(r)] * width
        return np.asarray(out, np.float64)

    def encode(self, sp, a, b):
        return O.encode(self.model, self.lat, sp, int(a), int(b))


def make_coefficients(elements, seed: int, k: int = 64, pair_eci_std: float = 0.02, ea0: float = 0.6,
                      ea_std: float = 0.05, d0: float = 2.86, calib_samples: int = 256) -> dict:
    """The benchmark's calibrated coefficient dict for `elements` and `seed`: pair ECIs (labels 1-3)
    and first-shell triplets (label 4) ~ N(0, pair_eci_std); per migrating element mu_x ~ U(0, 1),
    sigma_x ~ U(0.5, 1.5), U ~ N(0, 1/sqrt(F)) with k rows, theta scaled so the barrier spread over
    random environments of the 0.96-solvent composition is ea_std, and mu_D / mu_Ks / mu_e0 set so
    a pure-solvent environment has D = d0 and Ea = ea0 (Ea(dE=0) = Ks D^2 / 64)."""
    elements = sorted(set(elements))
    rng = np.random.default_rng(seed)
    labels = np.asarray(theta_labels(elements))
    theta = np.zeros(labels.size)
    mask = (labels >= 1) & (labels <= 4)
    theta[mask] = rng.normal(0.0, pair_eci_std, size=int(mask.sum()))
    solvent = "Al" if "Al" in elements else elements[0]
    calib_fractions = {e: (0.96 if e == solvent else 0.04 / max(1, len(elements) - 1)) for e in elements}
    n_cal = 10
    lat = O.Lattice(n_cal)
    enc = _Encoder(elements, lat)
    sizes_mmm, sizes_mm2 = enc.sizes
    sp = make_lattice(n_cal, calib_fractions, 0, seed + 1, elements)
    pure = np.full_like(sp, alphabet(elements).index(solvent))
    pairs = _nn1_pairs(n_cal, calib_samples, rng)
    feats_mmm, feats_mm2 = [], []
    for a, b in pairs:
        _, _, mm, mf, mb = enc.encode(sp, a, b)
        feats_mmm.append(mm / sizes_mmm)
        feats_mm2.append((mf + mb) / sizes_mm2)
    _, _, mm, mf, mb = enc.encode(pure, 0, n_cal)  # sites 0 and n are first neighbours
    x_mmm, x_mm2 = np.asarray(feats_mmm), np.asarray(feats_mm2)
    f_mmm, f_mm2 = sizes_mmm.size, sizes_mm2.size
    coeffs = {"Base": {"theta": theta.tolist()}}
    for el in elements:
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

        l_d = lin(x_mmm, mu_mmm, sg_mmm, u_mmm, th_d)
        l_ks = lin(x_mm2, mu_mm2, sg_mm2, u_mm2, th_ks)
        l_e0 = lin(x_mmm, mu_mmm, sg_mmm, u_mmm, th_e0)
        spread = float(np.std(2.0 * l_d + l_ks))
        s = (ea_std / ea0) / spread if spread > 0 else 1.0
        spread_e0 = float(np.std(l_e0))
        s_e0 = (ea_std / ea0) / spread_e0 if spread_e0 > 0 else 1.0
        th_d, th_ks, th_e0 = th_d * s, th_ks * s, th_e0 * s_e0
        x_pure_mmm, x_pure_mm2 = mm / sizes_mmm, (mf + mb) / sizes_mm2
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
