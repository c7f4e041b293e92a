"""Solute clusters (ansys::SoluteCluster) through the C ABI.

* Cluster lists (union-find on the GPU, the reference's small-cluster and
  solvent-shell rules on the host) equal the oracle's restatement for several
  criteria, lattices with vacancies included.
* Formation energies (GetEnergyOfCluster on the GPU, one block per cluster)
  equal the reference's own values (tests/golden/clusters_quaternary.npz) and
  the oracle's; the chemical potentials from the GPU census equal the
  reference's.
* The n = 64 lattice (2^20 sites): every cluster list equals the oracle's."""
import numpy as np
import pytest

from latticemontecarlo_gb300 import synthetic as S

from tests.golden.make_golden import CLUSTER_BOND, CLUSTER_SMALLEST, case_inputs

pytestmark = pytest.mark.gpu


def _ctx(elements, coeffs, n, species):
    from latticemontecarlo_gb300 import api
    ctx = api.Context(api.Model.from_coefficients(coeffs, list(elements)))
    ctx.set_lattices([n], species)
    return ctx


def test_golden_formation_energies(native):
    elements, coeffs, n, species = case_inputs("clusters_quaternary")
    g = np.load("tests/golden/clusters_quaternary.npz")
    solvent = S.alphabet(elements).index("Al")
    ctx = _ctx(elements, coeffs, n, species)
    mu = ctx.chemical_potential(solvent)
    np.testing.assert_allclose(mu, g["mu"], rtol=1e-12, atol=1e-15)
    clusters, ef = ctx.solute_clusters(solvent, CLUSTER_SMALLEST, CLUSTER_BOND, chemical_potential=g["mu"])
    off, mem, ref = g["offsets"], g["members"], g["energies"]
    assert len(clusters) == 79
    for k, c in enumerate(clusters):
        assert np.array_equal(c, mem[off[k]:off[k + 1]]), k
        want = (ref[k, 1] - ref[k, 2]) - sum(g["mu"][species[i]] for i in c)
        np.testing.assert_allclose(ef[k], want, rtol=1e-12, atol=1e-15, err_msg=f"cluster {k}")


@pytest.mark.parametrize("smallest,bond,seed", [(1, 12, 3), (2, 3, 4), (3, 2, 5), (1, 0, 6)])
def test_clusters_against_oracle(native, oracle_mod, smallest, bond, seed):
    el = ("Al", "Cu", "Mg", "Zn")
    coeffs = S.make_coefficients(el, seed)
    n = 10
    sp = S.make_lattice(n, {"Al": 0.80, "Cu": 0.05, "Mg": 0.08, "Zn": 0.07}, 3, seed, el)
    solvent = S.alphabet(el).index("Al")
    lat = oracle_mod.Lattice(n)
    m = oracle_mod.Model(el, coeffs, lat)
    m.set_vacancy_zero(True)  # clusters holding two vacancies count nothing, as on the GPU
    ctx = _ctx(el, coeffs, n, sp)
    mu = ctx.chemical_potential(solvent)
    got, ef = ctx.solute_clusters(solvent, smallest, bond, chemical_potential=mu)
    want = oracle_mod.solute_clusters(lat, sp, solvent, smallest, bond)
    assert len(got) == len(want) > 3
    for k, (a, b) in enumerate(zip(got, want)):
        assert np.array_equal(a, b), k
        e = (oracle_mod.cluster_energy(m, lat, sp, solvent, b, 1) - oracle_mod.cluster_energy(m, lat, sp, solvent, b, 2)
             - sum(mu[sp[i]] for i in b))
        np.testing.assert_allclose(ef[k], e, rtol=1e-12, atol=1e-15, err_msg=f"cluster {k}")
    # without chemical potentials: the same lists, no energies
    again, ef2 = ctx.solute_clusters(solvent, smallest, bond)
    assert all(np.array_equal(a, b) for a, b in zip(again, got)) and np.all(np.isnan(ef2))


def test_large_lattice_clusters(native, oracle_mod):
    L = S.LARGE
    el = L["elements"]
    coeffs = S.make_coefficients(el, 31)
    sp = S.make_lattice(L["n"], L["fractions"], L["vacancies"], 31, el)
    solvent = S.alphabet(el).index("Al")
    ctx = _ctx(el, coeffs, L["n"], sp)
    got, _ = ctx.solute_clusters(solvent, 2, 3)
    want = oracle_mod.solute_clusters(oracle_mod.Lattice(L["n"]), sp, solvent, 2, 3)
    assert len(got) == len(want) > 1000
    assert all(np.array_equal(a, b) for a, b in zip(got, want))


def test_solvent_code_checked(native):
    from latticemontecarlo_gb300 import _native as N
    el = ("Al", "Mg", "Zn")
    sp = S.make_lattice(8, {"Al": 0.9, "Mg": 0.05, "Zn": 0.05}, 1, 2, el)
    ctx = _ctx(el, S.make_coefficients(el, 1), 8, sp)
    with pytest.raises(N.LmcError) as e:
        ctx.solute_clusters(S.alphabet(el).index("X"))
    assert e.value.code == N.LMC_ERR_INVALID_ARGUMENT
