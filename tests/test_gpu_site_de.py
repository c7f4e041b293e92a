"""Single-site substitution energies and ExitTime's binding / profile energies through the C ABI.

* lmc_site_de_batch (GetDeFromLatticeIdSite) against the reference's own values
  (tests/golden/site_de_quaternary.npz) within the folded-weight tolerance.
* The fill option equals running on a lattice with that site changed, bit for bit.
* Context.exit_time_energies (lmc_exit_time_energies, one warp per site) against a restatement of
  ExitTime::GetBindingEnergy / GetProfileEnergy (ExitTime.cpp:401-511) over the oracle's site dE,
  and bit for bit against the same lists composed from lmc_site_de_batch queries."""
import numpy as np
import pytest

from latticemontecarlo_gb300 import synthetic as S

pytestmark = pytest.mark.gpu

DE_ATOL = 1e-12


def _ctx(elements, coeffs, n, species):
    from latticemontecarlo_gb300 import api
    ctx = api.Context(api.Model.from_coefficients(coeffs, list(elements)))
    ctx.set_lattices([n], species)
    return ctx


def test_site_de_golden(native):
    from tests.golden.make_golden import site_de_lattice
    elements, coeffs, n, sp, vac = site_de_lattice()
    g = np.load("tests/golden/site_de_quaternary.npz")
    q = g["queries"]
    ctx = _ctx(elements, coeffs, n, sp)
    de = ctx.site_de(q[:, 0], q[:, 2], q[:, 1])
    np.testing.assert_allclose(de, g["de"], rtol=0, atol=DE_ATOL)


def test_fill_equals_changed_lattice(native):
    el = ("Al", "Cu", "Mg", "Zn")
    coeffs = S.make_coefficients(el, 8)
    sp = S.make_lattice(10, {"Al": 0.8, "Cu": 0.05, "Mg": 0.08, "Zn": 0.07}, 1, 8, el)
    alpha = S.alphabet(el)
    x, al = alpha.index("X"), alpha.index("Al")
    vac = int(np.flatnonzero(sp == x)[0])
    rng = np.random.default_rng(3)
    sites = np.concatenate([rng.choice(sp.size, 500, replace=False), [vac]])
    to = rng.integers(0, len(alpha), sites.size)
    with_fill = _ctx(el, coeffs, 10, sp).site_de(sites, to, None, vac, al)
    filled = sp.copy()
    filled[vac] = al
    plain = _ctx(el, coeffs, 10, filled).site_de(sites, to)
    assert np.array_equal(with_fill, plain)


def test_exit_time_energies_against_oracle(native, oracle_mod):
    el = ("Al", "Mg", "Zn")
    coeffs = S.make_coefficients(el, 12)
    n = 8
    sp = S.make_lattice(n, {"Al": 0.82, "Mg": 0.09, "Zn": 0.09}, 1, 12, el)
    alpha = S.alphabet(el)
    x, al = alpha.index("X"), alpha.index("Al")
    ctx = _ctx(el, coeffs, n, sp)
    mu = ctx.chemical_potential(al)
    binding, profile = ctx.exit_time_energies(al, mu)
    lat = oracle_mod.Lattice(n)
    m = oracle_mod.Model(el, coeffs, lat)
    vac = int(np.flatnonzero(sp == x)[0])
    this = sp.copy()
    this[vac] = al
    rng = np.random.default_rng(1)
    for i in list(rng.choice(sp.size, 60, replace=False)) + [vac]:
        i = int(i)
        for c in (c for c in range(len(alpha)) if c != x):
            t = this.copy()
            t[i] = c
            want = oracle_mod.site_de(m, lat, t, i, x) - (mu[x] - mu[c])
            np.testing.assert_allclose(binding[alpha[c]][i], want, rtol=0, atol=DE_ATOL)
        if i == vac:
            cand = []
            for c in (c for c in range(len(alpha)) if c != x):
                t = this.copy()
                t[i] = c
                cand.append(oracle_mod.site_de(m, lat, t, i, x) + mu[c] - mu[x])
            want = max(cand)
        else:
            want = oracle_mod.site_de(m, lat, this, i, x) + mu[this[i]] - mu[x]
        np.testing.assert_allclose(profile[i], want, rtol=0, atol=DE_ATOL)


def test_site_de_checks_arguments(native):
    from latticemontecarlo_gb300 import _native as N
    el = ("Al", "Mg", "Zn")
    sp = S.make_lattice(8, {"Al": 0.9, "Mg": 0.05, "Zn": 0.05}, 1, 2, el)
    ctx = _ctx(el, S.make_coefficients(el, 1), 8, sp)
    with pytest.raises(N.LmcError) as e:
        ctx.site_de([sp.size], [0])
    assert e.value.code == N.LMC_ERR_OUT_OF_RANGE
    with pytest.raises(N.LmcError) as e:
        ctx.site_de([0], [9])
    assert e.value.code == N.LMC_ERR_INVALID_ARGUMENT


@pytest.mark.parametrize("vacancies", [1, 3])
def test_exit_time_energies_equal_site_de_queries(native, vacancies):
    el = ("Al", "Cu", "Mg", "Zn")
    coeffs = S.make_coefficients(el, 21)
    n = 10
    sp = S.make_lattice(n, {"Al": 0.8, "Cu": 0.05, "Mg": 0.08, "Zn": 0.07}, vacancies, 21, el)
    alpha = S.alphabet(el)
    x, al = alpha.index("X"), alpha.index("Al")
    ctx = _ctx(el, coeffs, n, sp)
    mu = ctx.chemical_potential(al)
    binding, profile = ctx.exit_time_energies(al, mu)
    vac = int(np.flatnonzero(sp == x)[0])
    idx = np.arange(sp.size)
    elems = [c for c in range(len(alpha)) if c != x]
    best = np.full(sp.size, -np.inf)
    for c in elems:
        de = ctx.site_de(idx, x, np.full(sp.size, c, np.int8), vac, al)
        assert np.array_equal(binding[alpha[c]], de - (mu[x] - mu[c]))
        best = np.maximum(best, de + mu[c] - mu[x])
    own = sp.copy()
    own[vac] = al
    want = ctx.site_de(idx, x, None, vac, al) + mu[own] - mu[x]
    want[vac] = best[vac]
    assert np.array_equal(profile, want)

