"""Second-order "chain" KMC (KineticMcChainOmpi, KineticMcChainOmpi.cpp:56-152)
against the oracle's restatement: the reference's mt19937_64 stream on one
lattice, and the Philox production streams of a batch of uneven lattices.
Selected events identical; barriers, rates, times and energies within the
parity tolerances. Also: sparse and dense evaluations identical, and a run split
over two launches equal to one launch (the previous-site state carries over)."""
import numpy as np
import pytest

from latticemontecarlo_gb300 import synthetic as S

pytestmark = pytest.mark.gpu

EA_RTOL = 1e-9
DE_ATOL = 1e-12
TIME_RTOL = 1e-9
EL = ("Al", "Mg", "Zn")
FRAC = {"Al": 0.85, "Mg": 0.08, "Zn": 0.07}


def _compare(tr, ref):
    assert np.array_equal(tr["vacancy"], ref[:, 0].astype(np.int64))
    assert np.array_equal(tr["target"], ref[:, 1].astype(np.int64))
    assert np.array_equal(tr["selected"], ref[:, 2].astype(np.int32))
    np.testing.assert_allclose(tr["ea"], ref[:, 3], rtol=EA_RTOL)
    np.testing.assert_allclose(tr["de"], ref[:, 4], rtol=0, atol=DE_ATOL)
    np.testing.assert_allclose(tr["total_rate"], ref[:, 5], rtol=1e-9)
    np.testing.assert_allclose(tr["time"], ref[:, 6], rtol=TIME_RTOL)
    np.testing.assert_allclose(tr["energy"], ref[:, 7], rtol=0, atol=1e-10)


@pytest.mark.parametrize("eci_scale", [1.0, 800.0])
def test_chain_reference_stream(native, oracle_mod, golden, eci_scale):
    """eci_scale 800: "Base".theta scaled so |dE| ~ kT (the golden cases' STRONG_ECI_SCALE)."""
    from latticemontecarlo_gb300 import api
    G, _ = golden
    coeffs = G.scaled_eci(S.make_coefficients(EL, 17), eci_scale)
    n = 8
    sp = S.make_lattice(n, FRAC, 1, 4, EL)
    lat = oracle_mod.Lattice(n)
    m = oracle_mod.Model(EL, coeffs, lat)
    steps, T, seed = 80, 450.0, 123
    ref = oracle_mod.kmc_chain(m, lat, sp.copy(), T, seed, steps, rng=0)
    ctx = api.Context(api.Model.from_coefficients(coeffs, list(EL)))
    ctx.set_lattices([n], sp)
    ctx.kmc_init([T], seed=seed, rng=native.LMC_RNG_MT19937_64, chain=True)
    tr, _ = ctx.kmc_run(steps, trace_replica=0)
    _compare(tr, ref)


def test_chain_batched_philox(native, oracle_mod):
    from latticemontecarlo_gb300 import api
    coeffs = S.make_coefficients(EL, 5)
    ns, sp, temps = S.batched_replicas(12, 6, n_range=(8, 10), fractions=FRAC)
    ctx = api.Context(api.Model.from_coefficients(coeffs, list(EL)))
    ctx.set_lattices(ns, sp)
    seed, steps, r = 31, 60, 3
    ctx.kmc_init(temps, seed=seed, rng=native.LMC_RNG_PHILOX, chain=True)
    tr, _ = ctx.kmc_run(steps, trace_replica=r)
    offs = np.concatenate([[0], np.cumsum(4 * ns.astype(np.int64) ** 3)])
    lat = oracle_mod.Lattice(int(ns[r]))
    m = oracle_mod.Model(EL, coeffs, lat)
    spr = sp[offs[r]:offs[r + 1]].copy()
    ref = oracle_mod.kmc_chain(m, lat, spr, float(temps[r]), seed, steps, rng=1, replica=r)
    _compare(tr, ref)
    assert np.array_equal(ctx.get_lattices()[offs[r]:offs[r + 1]], spr)


def test_chain_sparse_equals_dense_and_split_launches(native):
    from latticemontecarlo_gb300 import api
    coeffs = S.make_coefficients(EL, 8)
    ns, sp, temps = S.batched_replicas(3, 10, n_range=(8, 11), fractions=FRAC)
    out = []
    for evaluation, split in ((0, False), (1, False), (0, True)):
        ctx = api.Context(api.Model.from_coefficients(coeffs, list(EL)))
        ctx.set_lattices(ns, sp)
        ctx.kmc_init(temps, seed=2, rng=native.LMC_RNG_PHILOX, chain=True, evaluation=evaluation)
        if split:
            ctx.kmc_run(70)
            ctx.kmc_run(50)
        else:
            ctx.kmc_run(120)
        out.append((ctx.get_lattices(),) + tuple(ctx.kmc_state()))
    for other in out[1:]:
        for a, b in zip(out[0], other):
            assert np.array_equal(a, b)
