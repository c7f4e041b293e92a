"""Simulated annealing (SimulatedAnnealing.cpp:78-185) on the GPU against the
oracle's restatement on the reference's mt19937_64 stream: the same trial pairs,
acceptances, dE, energies and temperature schedule (windowed cool-down, reheats,
baseline decay), the same final lattice; a run split over two launches equals one."""
import numpy as np
import pytest

from latticemontecarlo_gb300 import synthetic as S

pytestmark = pytest.mark.gpu

EL = ("Al", "Mg", "Zn")


# eci_scale 800: "Base".theta scaled so |dE| ~ kT (STRONG_ECI_SCALE of the golden cases), so the
# Metropolis test rejects often and the reheat / cool-down schedule sees real energy changes
@pytest.mark.parametrize("T0,fractions,eci_scale", [(800.0, {"Al": 0.9, "Mg": 0.05, "Zn": 0.05}, 1.0),
                                                    (150.0, {"Al": 0.8, "Mg": 0.1, "Zn": 0.1}, 1.0),
                                                    (600.0, {"Al": 0.9, "Mg": 0.05, "Zn": 0.05}, 800.0)])
def test_sa_against_oracle(native, oracle_mod, golden, T0, fractions, eci_scale):
    from latticemontecarlo_gb300 import api
    G, _ = golden
    coeffs = G.scaled_eci(S.make_coefficients(EL, 9), eci_scale)
    n = 8
    sp = S.make_lattice(n, fractions, 0, 3, EL)
    lat = oracle_mod.Lattice(n)
    m = oracle_mod.Model(EL, coeffs, lat)
    max_steps, seed, e0 = 3000, 21, -0.5
    ref_sp = sp.copy()
    ref, ref_state = oracle_mod.sa(m, lat, ref_sp, T0, seed, max_steps, max_steps + 1, e0)
    ctx = api.Context(api.Model.from_coefficients(coeffs, list(EL)))
    ctx.set_lattices([n], sp)
    ctx.sa_init(T0, max_steps, seed=seed, energy=e0)
    tr = np.concatenate([ctx.sa_run(1400, trace=True), ctx.sa_run(max_steps + 1 - 1400, trace=True)])
    assert np.array_equal(tr["site1"], ref[:, 0].astype(np.int64))
    assert np.array_equal(tr["site2"], ref[:, 1].astype(np.int64))
    assert np.array_equal(tr["accepted"], ref[:, 2].astype(np.int32))
    np.testing.assert_allclose(tr["de"], ref[:, 3], rtol=0, atol=1e-12)
    np.testing.assert_allclose(tr["energy"], ref[:, 4], rtol=0, atol=1e-10)
    np.testing.assert_allclose(tr["temperature"], ref[:, 5], rtol=1e-12)
    steps, T, e, lowest = ctx.sa_state()
    assert steps == max_steps + 1
    np.testing.assert_allclose([T, e, lowest], ref_state[1:], rtol=1e-12, atol=1e-10)
    assert np.array_equal(ctx.get_lattices(), ref_sp)
    assert 0.05 < tr["accepted"].mean() < 0.999 and T < T0
    if eci_scale > 1:
        assert tr["accepted"].mean() < 0.7


def test_sa_single_species_rejected(native):
    from latticemontecarlo_gb300 import api
    coeffs = S.make_coefficients(EL, 9)
    sp = S.make_lattice(8, {"Al": 1.0}, 0, 3, EL)
    ctx = api.Context(api.Model.from_coefficients(coeffs, list(EL)))
    ctx.set_lattices([8], sp)
    with pytest.raises(native.LmcError):
        ctx.sa_init(500.0, 100)
