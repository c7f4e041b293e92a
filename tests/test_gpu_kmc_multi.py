"""Multi-vacancy KMC (every vacancy of a lattice tracked, one event per step
chosen among all of them) through the C ABI.

* Against the oracle's restatement (orc_kmc_multi, which re-evaluates every
  slot every step, so the kernel's re-evaluation of only the affected slots is
  checked too): slots, vacancies, targets and selections identical; barriers,
  rates, times and energies within the parity tolerances. Lattices include
  vacancies on 1NN and 3NN sites of one another (environments with a second
  vacancy, where clusters with two vacancies count nothing).
* With one vacancy per lattice the kernel reproduces the single-vacancy kernel's
  Philox trajectories; sparse and dense evaluations give identical results.
* The large-lattice workload (n = 64, 2^20 sites, 64 vacancies, Al/Mg/Zn/Cu
  .93/.03/.03/.01): composition conserved, vacancies where the state says,
  summed energy changes equal to the census difference."""
import numpy as np
import pytest

from latticemontecarlo_gb300 import synthetic as S

pytestmark = pytest.mark.gpu

EA_RTOL = 1e-9
DE_ATOL = 1e-12
TIME_RTOL = 1e-9
EL = ("Al", "Mg", "Zn")
FRAC = {"Al": 0.85, "Mg": 0.08, "Zn": 0.07}


def _lattice(oracle_mod, n, vacancies, seed, adjacent):
    sp = S.make_lattice(n, FRAC, vacancies, seed, EL)
    x = S.alphabet(EL).index("X")
    if adjacent:
        lat = oracle_mod.Lattice(n)
        v0 = int(np.flatnonzero(sp == x)[0])
        nb = lat.neighbors(v0)
        for j in (int(nb[3]), int(nb[30])):
            if sp[j] != x:
                other = int(np.flatnonzero((sp != x) & (np.arange(sp.size) != v0))[-1])
                sp[j], sp[other] = x, sp[j]
    return sp


def test_multi_vacancy_against_oracle(native, oracle_mod):
    from latticemontecarlo_gb300 import api
    coeffs = S.make_coefficients(EL, 13)
    specs = [(8, 6, 21, True), (9, 3, 22, False), (10, 1, 23, False)]
    parts = [_lattice(oracle_mod, n, v, s, a) for n, v, s, a in specs]
    ns = np.array([p[0] for p in specs], np.int32)
    temps = np.array([420.0, 480.0, 520.0])
    ctx = api.Context(api.Model.from_coefficients(coeffs, list(EL)))
    ctx.set_lattices(ns, np.concatenate(parts))
    seed = 77
    ctx.kmc_multi_init(temps, seed=seed)
    tr1 = ctx.kmc_multi_run(90, trace_replica=0)
    tr2 = ctx.kmc_multi_run(60, trace_replica=0)  # a second launch continues the streams and slots
    trace = np.concatenate([tr1, tr2])
    off, vac, steps, time, energy = ctx.kmc_multi_state()
    final = ctx.get_lattices()
    assert np.all(steps == 150)
    x = S.alphabet(EL).index("X")
    offs = np.concatenate([[0], np.cumsum(4 * ns.astype(np.int64) ** 3)])
    for r, (n, v, _, _) in enumerate(specs):
        sp = parts[r].copy()
        lat = oracle_mod.Lattice(n)
        m = oracle_mod.Model(EL, coeffs, lat)
        ref, ref_vac, t, e = oracle_mod.kmc_multi(m, lat, sp, float(temps[r]), seed, np.flatnonzero(sp == x), 150,
                                                  replica=r)
        assert np.array_equal(final[offs[r]:offs[r + 1]], sp), f"lattice {r}"
        assert np.array_equal(vac[off[r]:off[r + 1]], ref_vac)
        np.testing.assert_allclose(time[r], t, rtol=TIME_RTOL)
        np.testing.assert_allclose(energy[r], e, rtol=0, atol=1e-10)
        if r == 0:
            assert np.array_equal(trace["slot"], ref[:, 0].astype(np.int32))
            assert np.array_equal(trace["vacancy"], ref[:, 1].astype(np.int64))
            assert np.array_equal(trace["target"], ref[:, 2].astype(np.int64))
            assert np.array_equal(trace["selected"], ref[:, 3].astype(np.int32))
            np.testing.assert_allclose(trace["ea"], ref[:, 4], rtol=EA_RTOL)
            np.testing.assert_allclose(trace["de"], ref[:, 5], rtol=0, atol=DE_ATOL)
            np.testing.assert_allclose(trace["total_rate"], ref[:, 6], rtol=1e-12)
            np.testing.assert_allclose(trace["time"], ref[:, 7], rtol=TIME_RTOL)
            np.testing.assert_allclose(trace["energy"], ref[:, 8], rtol=0, atol=1e-10)
            assert len(set(trace["slot"].tolist())) > 1


def test_single_vacancy_equals_kmc_kernel(native):
    from latticemontecarlo_gb300 import api
    coeffs = S.make_coefficients(EL, 2)
    ns, sp, temps = S.batched_replicas(6, 40, n_range=(8, 12), fractions=FRAC)
    single = api.Context(api.Model.from_coefficients(coeffs, list(EL)))
    single.set_lattices(ns, sp)
    single.kmc_init(temps, seed=5, rng=native.LMC_RNG_PHILOX, rates=native.LMC_RATES_FP64)
    single.kmc_run(200)
    multi = api.Context(api.Model.from_coefficients(coeffs, list(EL)))
    multi.set_lattices(ns, sp)
    multi.kmc_multi_init(temps, seed=5)
    multi.kmc_multi_run(200)
    assert np.array_equal(single.get_lattices(), multi.get_lattices())
    v1, s1, t1, e1 = single.kmc_state()
    off, v2, s2, t2, e2 = multi.kmc_multi_state()
    assert np.array_equal(v1, v2) and np.array_equal(s1, s2)
    assert np.array_equal(e1, e2)
    np.testing.assert_allclose(t1, t2, rtol=1e-13)


def test_sparse_equals_dense(native, oracle_mod):
    from latticemontecarlo_gb300 import api
    coeffs = S.make_coefficients(EL, 4)
    parts = [_lattice(oracle_mod, 10, 12, 40 + r, r == 0) for r in range(4)]
    ns = np.full(4, 10, np.int32)
    out = []
    for evaluation in (native.LMC_EVAL_SPARSE, native.LMC_EVAL_DENSE):
        ctx = api.Context(api.Model.from_coefficients(coeffs, list(EL)))
        ctx.set_lattices(ns, np.concatenate(parts))
        ctx.kmc_multi_init([450.0] * 4, seed=9, evaluation=evaluation)
        tr = ctx.kmc_multi_run(300, trace_replica=0)
        out.append((ctx.get_lattices(), ctx.kmc_multi_state(), tr))
    (l0, s0, t0), (l1, s1, t1) = out
    assert np.array_equal(l0, l1) and np.array_equal(t0, t1)
    for a, b in zip(s0, s1):
        assert np.array_equal(a, b)


def test_lattice_without_vacancy_rejected(native):
    from latticemontecarlo_gb300 import api
    coeffs = S.make_coefficients(EL, 2)
    sp = S.make_lattice(8, FRAC, 0, 1, EL)
    ctx = api.Context(api.Model.from_coefficients(coeffs, list(EL)))
    ctx.set_lattices([8], sp)
    with pytest.raises(native.LmcError) as e:
        ctx.kmc_multi_init([400.0], seed=1)
    assert e.value.code == native.LMC_ERR_UNSUPPORTED


def test_large_lattice_64_vacancies(native):
    from latticemontecarlo_gb300 import api
    L = S.LARGE
    el = L["elements"]
    coeffs = S.make_coefficients(el, 31)
    sp = S.make_lattice(L["n"], L["fractions"], L["vacancies"], 31, el)
    ctx = api.Context(api.Model.from_coefficients(coeffs, list(el)))
    ctx.set_lattices([L["n"]], sp)
    e0, _ = ctx.energy()
    ctx.kmc_multi_init([500.0], seed=3)
    ctx.kmc_multi_run(3000)
    off, vac, steps, time, energy = ctx.kmc_multi_state()
    final = ctx.get_lattices()
    x = S.alphabet(el).index("X")
    assert off[-1] == L["vacancies"] and steps[0] == 3000 and time[0] > 0
    assert np.array_equal(np.bincount(sp, minlength=len(el) + 1), np.bincount(final, minlength=len(el) + 1))
    assert sorted(vac.tolist()) == sorted(np.flatnonzero(final == x).tolist())
    e1, _ = ctx.energy()
    np.testing.assert_allclose(e1 - e0, energy[0], rtol=0, atol=1e-8)


def test_fp32_rates_large_lattice(native):
    """LMC_RATES_FP32 on the large-lattice workload: conservation, vacancies where the state says,
    and the exact fixed-point energy sum equal to the census difference."""
    from latticemontecarlo_gb300 import api
    L = S.LARGE
    el = L["elements"]
    coeffs = S.make_coefficients(el, 31)
    sp = S.make_lattice(L["n"], L["fractions"], L["vacancies"], 31, el)
    ctx = api.Context(api.Model.from_coefficients(coeffs, list(el)))
    ctx.set_lattices([L["n"]], sp)
    e0, _ = ctx.energy()
    ctx.kmc_multi_init([500.0], seed=3, rates=native.LMC_RATES_FP32)
    tr = ctx.kmc_multi_run(3000, trace_replica=0)
    off, vac, steps, time, energy = ctx.kmc_multi_state()
    final = ctx.get_lattices()
    x = S.alphabet(el).index("X")
    assert steps[0] == 3000 and time[0] > 0 and np.all(np.diff(tr["time"]) > 0)
    assert np.array_equal(np.bincount(sp, minlength=len(el) + 1), np.bincount(final, minlength=len(el) + 1))
    assert sorted(vac.tolist()) == sorted(np.flatnonzero(final == x).tolist())
    e1, _ = ctx.energy()
    np.testing.assert_allclose(e1 - e0, energy[0], rtol=0, atol=1e-8)
    np.testing.assert_allclose(tr["energy"][-1], energy[0], rtol=0, atol=1e-12)


def test_fp32_and_fp64_rates_agree(native):
    """The same lattices and Philox streams with FP32 and FP64 barriers and rates: the trajectories
    agree except where a draw falls within the rates' rounding of an event boundary (a lattice or
    two at most); on the common steps the barriers agree within 1e-6 relative, the clock to the
    FP32 rates' precision and the energies (exact fixed point against FP64 sums) to rounding."""
    from latticemontecarlo_gb300 import api
    coeffs = S.make_coefficients(EL, 41)
    R, n, vac = 8, 16, 8
    sp = np.concatenate([S.make_lattice(n, FRAC, vac, 100 + r, EL) for r in range(R)])
    out = []
    for rates in (native.LMC_RATES_FP32, native.LMC_RATES_FP64):
        ctx = api.Context(api.Model.from_coefficients(coeffs, list(EL)))
        ctx.set_lattices([n] * R, sp)
        ctx.kmc_multi_init([480.0] * R, seed=19, rates=rates)
        tr = ctx.kmc_multi_run(400, trace_replica=0)
        out.append((tr, ctx.get_lattices(), ctx.kmc_multi_state()))
    (t32, l32, s32), (t64, l64, s64) = out
    size = 4 * n ** 3
    same = np.array([np.array_equal(l32[r * size:(r + 1) * size], l64[r * size:(r + 1) * size]) for r in range(R)])
    rel_t = np.abs(s32[3] - s64[3]) / s64[3]
    same &= rel_t < 3e-5
    assert same.sum() >= R - 2, f"{R - same.sum()} trajectories differ"
    assert np.median(rel_t[same]) < 3e-6
    np.testing.assert_allclose(s32[4][same], s64[4][same], rtol=0, atol=1e-9)
    # replica 0's events up to the first difference
    diff = np.flatnonzero((t32["slot"] != t64["slot"]) | (t32["target"] != t64["target"]))
    k = int(diff[0]) if diff.size else t32.size
    assert k >= 100
    np.testing.assert_allclose(t32["ea"][:k], t64["ea"][:k], rtol=1e-6)
    np.testing.assert_allclose(t32["de"][:k], t64["de"][:k], rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(t32["total_rate"][:k], t64["total_rate"][:k], rtol=3e-5)
