"""FP32 barriers and rates of the production KMC streams (LMC_RATES_FP32, the
default on Philox streams): barriers and energy changes within 1e-6 relative of
the reference predictor (the oracle, FP64) on the benchmark's own replicas, and
trajectories that agree with the FP64-rate kernel except where a draw falls
within the rates' rounding of an event boundary."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

F32_RTOL = 1e-6


def _bench_replicas(count):
    from latticemontecarlo_gb300 import synthetic as S
    cfg = S.KMC_BATCHED
    coeffs = S.make_coefficients(cfg["elements"], 1234)
    ns, sp, temps = S.batched_replicas(1234, count, cfg["n_range"], cfg["fractions"], cfg["T_range"],
                                       cfg["elements"])
    return cfg["elements"], coeffs, ns, sp, temps


def test_fp32_barriers_against_oracle_on_bench_replicas(native, oracle_mod):
    """Every event of four traced replicas of the 4096-replica workload over 150 steps: the FP32
    barrier and energy change of each of the 12 jumps against the oracle's FP64 predictor."""
    from latticemontecarlo_gb300 import api
    el, coeffs, ns, sp, temps = _bench_replicas(4096)
    offs = np.concatenate([[0], np.cumsum(4 * ns.astype(np.int64) ** 3)])
    x = sorted(set(el) | {"X"}).index("X")
    worst = 0.0
    for r in (0, 1000, 2047, 4095):
        ctx = api.Context(api.Model.from_coefficients(coeffs, list(el)))
        ctx.set_lattices(ns, sp)
        ctx.kmc_init(temps, seed=1234, rng=native.LMC_RNG_PHILOX)
        steps = 150
        tr, ev = ctx.kmc_run(steps, trace_replica=r, events=True)
        n = int(ns[r])
        lat = oracle_mod.Lattice(n)
        m = oracle_mod.Model(el, coeffs, lat)
        cur = sp[offs[r]:offs[r + 1]].copy()
        for s in range(steps):
            vac, tgt = int(tr["vacancy"][s]), int(tr["target"][s])
            assert cur[vac] == x
            for k in range(12):
                q = oracle_mod.quartic(m, lat, cur, vac, int(ev[s, k, 0]))
                worst = max(worst, abs(ev[s, k, 1] - q[0]) / q[0])
                np.testing.assert_allclose(ev[s, k, 1], q[0], rtol=F32_RTOL)
                np.testing.assert_allclose(ev[s, k, 2], q[1], rtol=F32_RTOL, atol=1e-12)
            cur[vac], cur[tgt] = cur[tgt], x
        assert np.array_equal(ctx.get_lattices()[offs[r]:offs[r + 1]], cur)
    assert worst < F32_RTOL


def test_fp32_and_fp64_rates_agree_on_bench_replicas(native):
    """The 4096 replicas for 200 steps with FP32 and with FP64 rates (same Philox streams): the
    trajectories are the same except where a draw falls within the rates' rounding of an event
    boundary, which happens on a handful of replicas at most; where they agree the clock agrees
    to the FP32 rates' precision and the energies (exact fixed point vs FP64 sums) to rounding."""
    from latticemontecarlo_gb300 import api
    el, coeffs, ns, sp, temps = _bench_replicas(4096)
    out = []
    for rates in (native.LMC_RATES_FP32, native.LMC_RATES_FP64):
        ctx = api.Context(api.Model.from_coefficients(coeffs, list(el)))
        ctx.set_lattices(ns, sp)
        ctx.kmc_init(temps, seed=77, rng=native.LMC_RNG_PHILOX, rates=rates)
        ctx.kmc_run(200)
        out.append((ctx.get_lattices(), ctx.kmc_state()))
    (l32, (v32, s32, t32, e32)), (l64, (v64, s64, t64, e64)) = out
    assert np.all(s32 == 200) and np.all(s64 == 200)
    offs = np.concatenate([[0], np.cumsum(4 * ns.astype(np.int64) ** 3)])
    same_lattice = np.array([np.array_equal(l32[offs[r]:offs[r + 1]], l64[offs[r]:offs[r + 1]])
                             for r in range(ns.size)])
    rel_t = np.abs(t32 - t64) / t64
    # a trajectory that took another path (and possibly came back) shows in its clock
    same = same_lattice & (v32 == v64) & (rel_t < 1e-5)
    assert same.sum() >= 4096 - 8, f"{4096 - same.sum()} trajectories differ"
    assert np.median(rel_t[same]) < 1e-6, np.median(rel_t[same])
    np.testing.assert_allclose(e32[same], e64[same], rtol=0, atol=1e-9)
