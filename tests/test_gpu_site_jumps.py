"""Vacancy placed on every site (ansys::ExitTime::GetJumpEnergetics and
GetBarrierListAndExitTime): the 12 jump barriers, energy changes and neighbour
ids per site against the oracle's pinned predictor on the same modified lattice
(own vacancy -> solvent, site -> vacancy), and the mean barrier and exit time
from the sorted barriers."""
import numpy as np
import pytest

from latticemontecarlo_gb300 import synthetic as S

pytestmark = pytest.mark.gpu

EL = ("Al", "Mg", "Zn")


@pytest.mark.parametrize("kind", [0, 1])
def test_site_jumps_against_oracle(native, oracle_mod, kind):
    from latticemontecarlo_gb300 import api
    coeffs = S.make_coefficients(EL, 23)
    n = 8
    sp = S.make_lattice(n, {"Al": 0.85, "Mg": 0.08, "Zn": 0.07}, 1, 6, EL)
    alpha = S.alphabet(EL)
    al, x = alpha.index("Al"), alpha.index("X")
    vac = int(np.flatnonzero(sp == x)[0])
    ctx = api.Context(api.Model.from_coefficients(coeffs, list(EL)))
    ctx.set_lattices([n], sp)
    T = 600.0
    ea, de, nb, avg, ext = ctx.site_jump_energetics(al, T, kind=kind)
    assert ea.shape == (sp.size, 12) and np.all(np.isfinite(ea)) and np.all(ext > 0)
    lat = oracle_mod.Lattice(n)
    m = oracle_mod.Model(EL, coeffs, lat)
    rng = np.random.default_rng(2)
    nbv = lat.neighbors(vac)[:12]
    picks = sorted(set(rng.choice(sp.size, 40, replace=False).tolist()) | {vac, int(nbv[0]), int(nbv[5])})
    beta = 1.0 / 8.617333262145e-5 / T
    for s in picks:
        mod = sp.copy()
        mod[vac] = al
        mod[s] = x
        ids = lat.neighbors(s)[:12]
        assert np.array_equal(nb[s], ids)
        for j, t in enumerate(ids):
            q = (oracle_mod.quartic if kind == 0 else oracle_mod.e0)(m, lat, mod, s, int(t))
            np.testing.assert_allclose(ea[s, j], q[0], rtol=1e-9)
            np.testing.assert_allclose(de[s, j], q[1], rtol=0, atol=1e-12)
        b = np.sort(ea[s])
        np.testing.assert_allclose(avg[s], b.sum() / 12, rtol=1e-14)
        np.testing.assert_allclose(ext[s], 1.0 / np.exp(-b * beta).sum() / 1e13, rtol=1e-12)
    # a site list gives the same rows
    sub = np.array(picks[:7], np.int64)
    ea2, de2, nb2, avg2, ext2 = ctx.site_jump_energetics(al, T, sites=sub, kind=kind)
    assert np.array_equal(ea2, ea[sub]) and np.array_equal(nb2, nb[sub]) and np.array_equal(ext2, ext[sub])
