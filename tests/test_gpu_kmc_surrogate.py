"""Surrogate-assisted multi-vacancy KMC (lmc_kmc_multi_surrogate_run) on a four-species
lattice with the composition of the large-lattice workload (Al/Mg/Zn/Cu .93/.03/.03/.01),
smaller for the test:

* with threshold 0 every jump takes the plain predictor, and the run is the plain
  multi-vacancy run of the same seed event for event (slots, targets, selections,
  barriers, times, energies) with the same final lattice: the step loop, the
  re-evaluation lists, the selection and the energy sums are those of
  lmc_kmc_multi_run;
* with the 10 meV spread threshold and a trained ensemble: the barriers the run used
  for its selected events against the plain predictor's barriers of the same events
  (recorded by the run), the summed energy changes against the census difference,
  composition and vacancy conservation, and a fallback share strictly between 0 and 1."""
import numpy as np
import pytest

from latticemontecarlo_gb300 import synthetic as S

pytestmark = pytest.mark.gpu

EL = ("Al", "Cu", "Mg", "Zn")
FRAC = {"Al": 0.93, "Cu": 0.01, "Mg": 0.03, "Zn": 0.03}


def _setup(api, N, n, vacancies, seed):
    coeffs = S.make_coefficients(EL, 31)
    sp = S.make_lattice(n, FRAC, vacancies, seed, EL)
    ctx = api.Context(api.Model.from_coefficients(coeffs, list(EL)))
    ctx.set_lattices([n], sp)
    ctx.set_surrogate_encoding(N.LMC_FEATURES_SOLUTE)
    return ctx, sp


def _net(api, ctx, samples, epochs):
    nin = api.surrogate_feature_count(ctx)
    assert nin == 192
    x, ea, _, _ = api.surrogate_dataset(ctx, 1, samples, 0.0, 0.15, nin)
    net = api.Surrogate(nin, 128, 2, seed=3)
    net.set_label_scale(float(ea.mean()), float(ea.std()))
    net.train(x, ea, batch=2048, epochs=epochs, lr=3e-3, seed=4)
    return net


def test_threshold_zero_is_the_plain_trajectory(native):
    pytest.importorskip("torch")
    from latticemontecarlo_gb300 import api
    N = native
    n, vac, seed, steps = 14, 12, 5, 1500
    plain, sp = _setup(api, N, n, vac, seed)
    plain.kmc_multi_init([500.0], seed=9, evaluation=N.LMC_EVAL_DENSE)
    ref = plain.kmc_multi_run(steps, trace_replica=0)
    ref_state = plain.kmc_multi_state()
    ref_lat = plain.get_lattices()

    ctx, _ = _setup(api, N, n, vac, seed)
    net = _net(api, ctx, 1 << 16, 1)
    ctx.kmc_multi_init([500.0], seed=9)
    tr, plain_ea, nfb = ctx.kmc_multi_surrogate_run(net, steps, threshold_ev=0.0, trace=True)
    state = ctx.kmc_multi_state()
    assert nfb >= 12 * vac
    for f in ("vacancy", "target", "selected", "slot"):
        assert np.array_equal(tr[f], ref[f]), f
    for f in ("ea", "de", "total_rate", "time", "energy"):
        np.testing.assert_array_equal(tr[f], ref[f], err_msg=f)
    np.testing.assert_array_equal(plain_ea, ref["ea"])
    assert np.array_equal(ctx.get_lattices(), ref_lat)
    for a, b in zip(state[1:], ref_state[1:]):
        np.testing.assert_array_equal(a, b)


def test_surrogate_assisted_run(native):
    pytest.importorskip("torch")
    from latticemontecarlo_gb300 import api
    N = native
    n, vac, seed, steps = 16, 24, 6, 4000
    ctx, sp = _setup(api, N, n, vac, seed)
    net = _net(api, ctx, 1 << 19, 20)
    e0, _ = ctx.energy()
    ctx.kmc_multi_init([500.0], seed=11)
    tr, plain_ea, nfb = ctx.kmc_multi_surrogate_run(net, steps, threshold_ev=0.010, trace=True)
    off, vacs, st, time, energy = ctx.kmc_multi_state()
    final = ctx.get_lattices()
    x = S.alphabet(EL).index("X")
    assert st[0] == steps and time[0] > 0 and np.all(np.diff(tr["time"]) > 0)
    assert np.array_equal(np.bincount(sp, minlength=len(EL) + 1), np.bincount(final, minlength=len(EL) + 1))
    assert sorted(vacs.tolist()) == sorted(np.flatnonzero(final == x).tolist())
    # the energy changes are the plain predictor's: their sum is the census difference
    e1, _ = ctx.energy()
    np.testing.assert_allclose(e1 - e0, energy[0], rtol=0, atol=1e-8)
    np.testing.assert_allclose(tr["energy"][-1], energy[0], rtol=0, atol=1e-12)
    # barriers used for the selected events against the plain predictor's
    err = np.abs(tr["ea"] - plain_ea)
    assert np.all(np.isfinite(plain_ea)) and float(err.mean()) < 0.005, float(err.mean())
    # evaluated jumps: every slot at the start, then the re-evaluated slots' 12 each step
    assert 0 < nfb < 12 * vac + 12 * steps * vac
    # a second run continues the clock and the Philox stream
    tr2, _, _ = ctx.kmc_multi_surrogate_run(net, 100, threshold_ev=0.010, trace=True)
    assert tr2["time"][0] > tr["time"][-1]
