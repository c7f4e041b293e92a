"""ExitTime's per-cluster analysis (ExitTime::GetExitTimeInfo, lmc/ansys/src/ExitTime.cpp:53-128)
through lmc_exit_time_clusters against a restatement on the oracle: every barrier of the clusters
and their first-neighbour shells from the oracle's Quartic predictor on the lattice with its
vacancy filled by the solvent and the vacancy moved to the site (GetJumpEnergetics,
ExitTime.cpp:217-310), the Markov chain's escape time solved densely with numpy
(BuildMarkovChain, ExitTime.cpp:165-216), the barrier averages (GetAverageBarriers,
ExitTime.cpp:311-399) and the effective binding energy (ExitTime.cpp:121)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

EL = ("Al", "Cu", "Mg", "Zn")
KB, NU = 8.617333262145e-5, 1e13


def _oracle_cluster(oracle_mod, m, lat, this, cluster, profile, beta):
    x = sorted(set(EL) | {"X"}).index("X")
    s = set(int(v) for v in cluster)
    t = set(s)
    for v in s:
        t.update(int(j) for j in lat.neighbors(v)[:12])
    states = sorted(t)
    index = {v: i for i, v in enumerate(states)}
    ea, de, nb = {}, {}, {}
    for v in states:  # GetJumpEnergetics: the vacancy placed on v
        keep = this[v]
        this[v] = x
        nb[v] = [int(j) for j in lat.neighbors(v)[:12]]
        q = [oracle_mod.quartic(m, lat, this, v, j) for j in nb[v]]
        this[v] = keep
        ea[v], de[v] = np.array([r[0] for r in q]), np.array([r[1] for r in q])
    k = len(states)
    a, tau = np.eye(k), np.zeros(k)
    p = np.array([np.exp(-profile[v] * beta) for v in states])
    lists = [[], [], [], []]
    for v in states:
        rates = NU * np.exp(-ea[v] * beta)
        tau[index[v]] = 1.0 / rates.sum()
        for q, j in enumerate(nb[v]):
            if j in index:
                a[index[v], index[j]] -= rates[q] / rates.sum()
            cat = (0 if (v in s and j in s) else 1 if (v in s and j not in s and j in t)
                   else 2 if (v not in s and j not in s and j in t) else 3 if (v not in s and j not in t) else -1)
            if cat >= 0:
                lists[cat].append(ea[v][q] - de[v][q] / 2)
    escape = float(p / p.sum() @ np.linalg.solve(a, tau))
    bars = [np.mean(x) if x else np.nan for x in lists] + [np.std(x) if x else np.nan for x in lists]
    return escape, len(t) - len(s), np.array(bars)


def test_exit_time_clusters_against_oracle(native, oracle_mod):
    from latticemontecarlo_gb300 import api
    from latticemontecarlo_gb300 import synthetic as S
    coeffs = S.make_coefficients(EL, 11)
    n = 10
    sp = S.make_lattice(n, {"Al": 0.86, "Cu": 0.04, "Mg": 0.05, "Zn": 0.05}, 1, 77, EL)
    alpha = S.alphabet(EL)
    al, x = alpha.index("Al"), alpha.index("X")
    ctx = api.Context(api.Model.from_coefficients(coeffs, list(EL)))
    ctx.set_lattices([n], sp)
    mu = ctx.chemical_potential(al)
    _, profile = ctx.exit_time_energies(al, mu)
    clusters, _ = ctx.solute_clusters(al, 2, 3)
    assert len(clusters) >= 10
    T = 600.0
    got = ctx.exit_time_clusters(clusters, al, T, profile)
    lat = oracle_mod.Lattice(n)
    m = oracle_mod.Model(EL, coeffs, lat)
    this = sp.copy()
    this[this == x] = al  # ExitTime's this_config: the vacancy filled with the solvent
    beta = 1.0 / KB / T
    for c in list(range(6)) + list(range(len(clusters) - 4, len(clusters))):
        esc, nsize, bars = _oracle_cluster(oracle_mod, m, lat, this, clusters[c], profile, beta)
        assert got["neighbor_size"][c] == nsize
        np.testing.assert_allclose(got["markov_escape_time"][c], esc, rtol=1e-6)
        np.testing.assert_allclose(got["barriers"][c], bars, rtol=0, atol=1e-8, equal_nan=True)
        eff = -np.log(esc * NU) / beta + bars[3]
        np.testing.assert_allclose(got["effective_binding_energy"][c], eff, rtol=0, atol=1e-7)
    assert np.all(got["markov_escape_time"] > 0)
