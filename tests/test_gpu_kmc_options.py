"""KMC options beyond the default Quartic / constant-temperature run, each
against the oracle on the reference's mt19937_64 stream:

* E0 barriers (VacancyMigrationPredictorE0, Ea = max(0, e0 + dE/2));
* a time-temperature schedule (TimeTemperatureInterpolator, T updated at the
  start of every step) together with the RateCorrector time factor;
* the host stop flag (a persistent launch ends early with LMC_ERR_STOPPED and
  resumes where it stopped).

Event sequences must be identical; barriers, energies and times within the
tolerances of the parity tests."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

EA_RTOL = 1e-9
DE_ATOL = 1e-12
TIME_RTOL = 1e-9


def _compare(tr, ref):
    assert np.array_equal(tr["vacancy"], ref[:, 0].astype(np.int64))
    assert np.array_equal(tr["target"], ref[:, 1].astype(np.int64))
    assert np.array_equal(tr["selected"], ref[:, 2].astype(np.int32))
    np.testing.assert_allclose(tr["ea"], ref[:, 3], rtol=EA_RTOL)
    np.testing.assert_allclose(tr["de"], ref[:, 4], rtol=0, atol=DE_ATOL)
    np.testing.assert_allclose(tr["total_rate"], ref[:, 5], rtol=1e-8)
    np.testing.assert_allclose(tr["time"], ref[:, 6], rtol=TIME_RTOL)
    np.testing.assert_allclose(tr["energy"], ref[:, 7], rtol=0, atol=1e-10)


def _setup(native, golden, oracle_mod):
    from latticemontecarlo_gb300 import api
    G, _ = golden
    el, coeffs, n, sp = G.case_inputs("kmc_ternary")
    ctx = api.Context(api.Model.from_coefficients(coeffs, list(el)))
    ctx.set_lattices([n], sp)
    lat = oracle_mod.Lattice(n)
    m = oracle_mod.Model(el, coeffs, lat)
    return G, ctx, lat, m, sp


def test_kmc_e0_barriers(native, golden, oracle_mod):
    G, ctx, lat, m, sp = _setup(native, golden, oracle_mod)
    steps = 400
    ref, _ = oracle_mod.kmc(m, lat, sp.copy(), G.KMC_T, G.KMC_SEED, steps, kind=1)
    ctx.kmc_init([G.KMC_T], seed=G.KMC_SEED, rng=native.LMC_RNG_MT19937_64, kind=native.LMC_BARRIER_E0)
    tr, _ = ctx.kmc_run(steps, trace_replica=0)
    _compare(tr, ref)


@pytest.mark.parametrize("evaluation", [0, 1])
def test_kmc_temperature_schedule_and_rate_corrector(native, golden, oracle_mod, evaluation):
    G, ctx, lat, m, sp = _setup(native, golden, oracle_mod)
    steps = 400
    tt = (np.array([0.0, 2e-5, 1e-4]), np.array([350.0, 550.0, 450.0]))
    ref, _ = oracle_mod.kmc(m, lat, sp.copy(), G.KMC_T, G.KMC_SEED, steps, tt=tt, rate_corrector=True)
    assert ref[-1, 6] > tt[0][1]  # the run crosses the first breakpoint of the schedule
    ctx.kmc_init([G.KMC_T], seed=G.KMC_SEED, rng=native.LMC_RNG_MT19937_64, rate_corrector=True, tt=tt,
                 evaluation=evaluation)
    tr, _ = ctx.kmc_run(steps, trace_replica=0)
    _compare(tr, ref)


def test_kmc_stop_flag(native, golden, oracle_mod):
    G, ctx, lat, m, sp = _setup(native, golden, oracle_mod)
    ctx.kmc_init([G.KMC_T], seed=G.KMC_SEED, rng=native.LMC_RNG_MT19937_64)
    ctx.request_stop(1)
    with pytest.raises(native.LmcError) as e:
        ctx.kmc_run(500)
    assert e.value.code == native.LMC_ERR_STOPPED
    vac, steps, time, energy = ctx.kmc_state()
    assert steps[0] == 0 and time[0] == 0.0
    ctx.request_stop(0)
    tr, _ = ctx.kmc_run(120, trace_replica=0)
    ref, _ = oracle_mod.kmc(m, lat, sp.copy(), G.KMC_T, G.KMC_SEED, 120)
    _compare(tr, ref)
    assert ctx.kmc_state()[1][0] == 120


@pytest.mark.parametrize("evaluation", [0, 1])
def test_kmc_early_stop(native, golden, oracle_mod, evaluation):
    """IsEscaped: with seed 103 the oracle's trajectory escapes at step 193 (the
    vacancy's 1-3NN shells hold only the solvent); the GPU run stops there too
    and later launches leave the replica untouched."""
    G, ctx, lat, m, sp = _setup(native, golden, oracle_mod)
    ref, _ = oracle_mod.kmc(m, lat, sp.copy(), G.KMC_T, 103, 500, early_stop=True)
    assert 0 < len(ref) < 500
    ctx.kmc_init([G.KMC_T], seed=103, rng=native.LMC_RNG_MT19937_64, early_stop=True, evaluation=evaluation)
    tr, _ = ctx.kmc_run(500, trace_replica=0)
    _compare(tr[:len(ref)], ref)
    assert ctx.kmc_state()[1][0] == len(ref) and ctx.kmc_escaped()[0]
    before = ctx.get_lattices().copy()
    ctx.kmc_run(50)
    assert ctx.kmc_state()[1][0] == len(ref)
    assert np.array_equal(ctx.get_lattices(), before)
