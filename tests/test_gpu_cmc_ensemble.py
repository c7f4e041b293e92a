"""The throughput CMC (LMC_CMC_THROUGHPUT: every round, random-priority
non-overlapping pairs more than 3NN apart, dE on the unchanged lattice) is a
different Markov chain from CanonicalMcOmp's batch order (LMC_CMC_REFERENCE_BATCH,
bit-identical to the reference). Both must sample the same canonical ensemble:
on a case whose ECIs give 40 % acceptance at 500 K (the golden cases'
STRONG_ECI_SCALE), the equilibrium mean energy and the 1NN Warren-Cowley
parameters of the solute pairs agree within their statistical errors (8
independent chains per mode, error bars from the spread of the chains' means)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

EL = ("Al", "Cu", "Mg", "Zn")
N_EDGE, T, SEEDS = 10, 500.0, 8
BURN, BLOCKS, SWEEPS_PER_BLOCK = 60, 30, 10
NSIGMA = 4.0


def _first_neighbours(native, n):
    nb = np.zeros(42, np.int64)
    out = np.zeros((4 * n ** 3, 12), np.int64)
    for s in range(out.shape[0]):
        native.check(native.lib.lmc_geom_neighbors(n, s, nb.ctypes.data_as(C.POINTER(C.c_int64))))
        out[s] = nb[:12]
    return out


def _warren_cowley(sp, nb, codes):
    """alpha_ij = 1 - P(a 1NN of an i site is j) / c_j for the solute codes."""
    c = np.bincount(sp, minlength=8) / sp.size
    neigh = sp[nb]
    out = []
    for a in codes:
        rows = neigh[sp == a]
        for b in codes:
            out.append(1.0 - np.mean(rows == b) / c[b])
    return np.asarray(out)


def _chains(native, api, coeffs, sp0, nb, mode):
    solutes = [sorted(set(EL) | {"X"}).index(e) for e in ("Cu", "Mg", "Zn")]
    energies, alphas = [], []
    for seed in range(SEEDS):
        ctx = api.Context(api.Model.from_coefficients(coeffs, list(EL)))
        ctx.set_lattices([N_EDGE], sp0)
        e, _ = ctx.energy()
        kw = dict(mode=mode, seed=1000 + seed, batch=16)
        e, _, _ = ctx.cmc_run(T, BURN * sp0.size, energy=e, **kw)
        es, al, acc_all, done_all = [], [], 0, 0
        for b in range(BLOCKS):
            e, done, acc = ctx.cmc_run(T, SWEEPS_PER_BLOCK * sp0.size, energy=e, **kw)
            acc_all += acc
            done_all += done
            census, _ = ctx.energy()
            assert abs(census - e) < 1e-8  # the accumulated dE equals the census difference
            es.append(census)
            al.append(_warren_cowley(ctx.get_lattices(), nb, solutes))
        assert 0.3 < acc_all / done_all < 0.6
        energies.append(np.mean(es))
        alphas.append(np.mean(al, axis=0))
    return np.asarray(energies), np.asarray(alphas)


def test_throughput_cmc_samples_the_reference_ensemble(native, golden):
    from latticemontecarlo_gb300 import api
    from latticemontecarlo_gb300 import synthetic as S
    G, _ = golden
    coeffs = G.scaled_eci(S.make_coefficients(EL, 4321), G.STRONG_ECI_SCALE)
    sp0 = S.make_lattice(N_EDGE, {"Al": 0.94, "Cu": 0.02, "Mg": 0.02, "Zn": 0.02}, 0, 5, EL)
    nb = _first_neighbours(native, N_EDGE)
    ctx = api.Context(api.Model.from_coefficients(coeffs, list(EL)))
    ctx.set_lattices([N_EDGE], sp0)
    e_random, _ = ctx.energy()
    e_ref, a_ref = _chains(native, api, coeffs, sp0, nb, native.LMC_CMC_REFERENCE_BATCH)
    e_tp, a_tp = _chains(native, api, coeffs, sp0, nb, native.LMC_CMC_THROUGHPUT)

    def se(x):
        return np.std(x, axis=0, ddof=1) / np.sqrt(len(x))

    # the ensemble is far from the random start, so the comparison has power
    assert e_ref.mean() < e_random - 20 * se(e_ref)
    d_e = abs(e_tp.mean() - e_ref.mean())
    s_e = np.hypot(se(e_tp), se(e_ref))
    assert d_e < NSIGMA * s_e, (e_tp.mean(), e_ref.mean(), s_e)
    d_a = np.abs(a_tp.mean(axis=0) - a_ref.mean(axis=0))
    s_a = np.hypot(se(a_tp), se(a_ref))
    assert np.all(d_a < NSIGMA * s_a + 1e-3), (a_tp.mean(axis=0), a_ref.mean(axis=0), s_a)
