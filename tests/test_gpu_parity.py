"""GPU parity: every kernel through the C ABI against the reference's golden
vectors and the oracle, at fixture sizes and (through size-independent
properties) at the benchmark sizes.

Tolerances. Integer encodings, census counts, selected events and lattices
are compared exactly. Barriers and energy changes are computed from exact
int64 fixed-point cluster sums and an FP64 epilogue; the reference computes
them in FP64 with a different operation order, so they are compared with
EA_RTOL / DE_ATOL below (far inside the 1e-6 relative bar of the task)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

EA_RTOL = 1e-9      # barrier, relative
DE_ATOL = 1e-12     # energy change, eV
TIME_RTOL = 1e-9    # simulated time, relative
F32_RTOL = 1e-6     # FP32 barriers, energy changes and rates of the production KMC streams (the task's bar)


@pytest.fixture(scope="module")
def api(native):
    from latticemontecarlo_gb300 import api
    return api


def ctx_for(api, G, name):
    el, coeffs, n, sp = G.case_inputs(name)
    m = api.Model.from_coefficients(coeffs, list(el))
    ctx = api.Context(m)
    ctx.set_lattices([n], sp)
    return ctx, el, coeffs, n, sp


@pytest.mark.parametrize("name", ["pred_ternary", "pred_quaternary"])
def test_barriers_and_encodings(api, golden, name):
    G, load = golden
    fx = load(name)
    ctx, el, coeffs, n, sp = ctx_for(api, G, name)
    jumps = fx["pair"][fx["jump_ok"].astype(bool)]
    ea, de, d, ks = ctx.barrier_batch(jumps, kind=0)
    ref = fx["quartic"]
    np.testing.assert_allclose(ea, ref[:, 0], rtol=EA_RTOL)
    np.testing.assert_allclose(de, ref[:, 1], rtol=0, atol=DE_ATOL)
    np.testing.assert_allclose(d, ref[:, 2], rtol=EA_RTOL)
    np.testing.assert_allclose(ks, ref[:, 3], rtol=EA_RTOL)
    ea0, de0, e0v, _ = ctx.barrier_batch(jumps, kind=1)
    np.testing.assert_allclose(ea0, fx["e0"][:, 0], rtol=EA_RTOL, atol=1e-15)
    np.testing.assert_allclose(de0, fx["e0"][:, 1], rtol=0, atol=DE_ATOL)
    cs, ce, mm, mf, mb = ctx.encode_batch(jumps)
    assert np.array_equal(cs, fx["state_start"]) and np.array_equal(ce, fx["state_end"])
    assert np.array_equal(mm, fx["enc_mmm"])
    assert np.array_equal(mf, fx["enc_mm2_fwd"]) and np.array_equal(mb, fx["enc_mm2_bwd"])


@pytest.mark.parametrize("name", ["pred_ternary", "pred_quaternary"])
def test_pair_swap_de_and_census(api, golden, name):
    G, load = golden
    fx = load(name)
    ctx, el, coeffs, n, sp = ctx_for(api, G, name)
    de = ctx.de_pairs(fx["pair"])
    np.testing.assert_allclose(de, fx["pairsite"], rtol=0, atol=DE_ATOL)
    e, counts = ctx.energy()
    from latticemontecarlo_gb300 import synthetic as S
    bonds = np.asarray([256, 3072, 1536, 6144, 12288, 6144, 12288, 6144], float)
    assert np.array_equal(counts / bonds[np.asarray(S.theta_labels(el))], fx["census_encode"])
    assert e == fx["energy"]


def test_barrier_errors(api, golden):
    from latticemontecarlo_gb300 import LmcError
    G, load = golden
    ctx, el, coeffs, n, sp = ctx_for(api, G, "pred_ternary")
    with pytest.raises(LmcError) as e:
        ctx.barrier_batch([[0, 1]])  # second neighbours
    assert e.value.code == 2 and "Neighbor not found" in str(e.value)
    with pytest.raises(LmcError):
        ctx.barrier_batch([[0, 4 * n ** 3]])


@pytest.mark.parametrize("warps,evaluation", [(1, 0), (3, 0), (12, 0), (1, 1), (12, 1)])
def test_kmc_reference_stream(api, golden, warps, evaluation):
    """mt19937_64 stream: the event sequence equals the reference's (sparse and dense evaluation)."""
    G, load = golden
    fx = load("kmc_ternary")
    ctx, el, coeffs, n, sp = ctx_for(api, G, "kmc_ternary")
    ctx.kmc_init([G.KMC_T], seed=G.KMC_SEED, rng=0, warps_per_replica=warps, replicas_per_block=1,
                 evaluation=evaluation)
    tr, ev = ctx.kmc_run(G.KMC_STEPS, trace_replica=0, events=True)
    ref = fx["steps"]  # steps vacancy target selected Ea dE total time energy
    assert np.array_equal(tr["vacancy"], ref[:, 1].astype(np.int64))
    assert np.array_equal(tr["target"], ref[:, 2].astype(np.int64))
    assert np.array_equal(tr["selected"], ref[:, 3].astype(np.int32))
    np.testing.assert_allclose(tr["ea"], ref[:, 4], rtol=EA_RTOL)
    np.testing.assert_allclose(tr["de"], ref[:, 5], rtol=0, atol=DE_ATOL)
    np.testing.assert_allclose(tr["total_rate"], ref[:, 6], rtol=1e-8)
    np.testing.assert_allclose(tr["time"], ref[:, 7], rtol=TIME_RTOL)
    np.testing.assert_allclose(tr["energy"], ref[:, 8], rtol=0, atol=1e-10)
    d = G.KMC_DETAIL
    assert np.array_equal(ev[:d, :, 0], fx["events"][:, :, 0])
    np.testing.assert_allclose(ev[:d, :, 1], fx["events"][:, :, 1], rtol=EA_RTOL)
    np.testing.assert_allclose(ev[:d, :, 2], fx["events"][:, :, 2], rtol=0, atol=DE_ATOL)
    vac, steps, time, energy = ctx.kmc_state()
    assert steps[0] == G.KMC_STEPS and vac[0] == int(ref[-1, 2])


def test_cmc_reference_batch(api, golden):
    """CanonicalMcOmp batch semantics on the reference's RNG stream."""
    G, load = golden
    fx = load("cmc_quaternary")
    ctx, el, coeffs, n, sp = ctx_for(api, G, "cmc_quaternary")
    e, done, acc = ctx.cmc_run(G.CMC_T, G.CMC_STEPS + 1, mode=0, seed=G.CMC_SEED, batch=G.CMC_BATCH)
    assert done == int(fx["final_steps"])
    assert np.array_equal(ctx.get_lattices(), fx["final_species"])
    np.testing.assert_allclose(e, fx["final_energy"][0], rtol=0, atol=1e-10)


@pytest.mark.parametrize("name", ["kmc_config1", "kmc_config1_strong"])
@pytest.mark.parametrize("warps,evaluation", [(1, 1), (12, 0)])
def test_kmc_baseline_config_stream(api, golden, name, warps, evaluation):
    """The benchmark's one-trajectory KMC configuration (n = 10, Al/Mg/Zn .96/.02/.02, 400 K) for
    its full 1e5 steps on the reference's mt19937_64 stream: the event selected at every step is
    the reference's (plain coefficients, and ECIs scaled so |dE| ~ kT), sparse and dense evaluation."""
    G, load = golden
    fx = load(name)
    kind, el, *_, T, rseed, steps = G.BASELINE_CASES[name]
    _, coeffs, n, sp = G.baseline_inputs(name)
    ctx = api.Context(api.Model.from_coefficients(coeffs, list(el)))
    ctx.set_lattices([n], sp)
    ctx.kmc_init([T], seed=rseed, rng=0, warps_per_replica=warps, replicas_per_block=1, evaluation=evaluation)
    tr, _ = ctx.kmc_run(steps, trace_replica=0)
    first_diff = np.flatnonzero(tr["target"] != fx["target"])
    assert first_diff.size == 0, f"first differing step {first_diff[:1]}"
    assert np.array_equal(tr["selected"], fx["selected"].astype(np.int32))
    k = fx["sample_steps"]
    ref = fx["sample"]  # Ea dE total time energy
    np.testing.assert_allclose(tr["ea"][k], ref[:, 0], rtol=EA_RTOL)
    np.testing.assert_allclose(tr["de"][k], ref[:, 1], rtol=0, atol=DE_ATOL * 1e3 * abs(ref[:, 1]).max())
    np.testing.assert_allclose(tr["total_rate"][k], ref[:, 2], rtol=1e-8)
    np.testing.assert_allclose(tr["time"][k], ref[:, 3], rtol=TIME_RTOL)
    np.testing.assert_allclose(tr["energy"][k], ref[:, 4], rtol=0, atol=1e-8)
    vac, nsteps, time, energy = ctx.kmc_state()
    assert nsteps[0] == steps and vac[0] == int(fx["final_vacancy"])


def test_cmc_baseline_config_reference_batch(api, golden):
    """CanonicalMcOmp at the benchmark's CMC size (n = 30, 108000 sites, Al/Mg/Zn/Cu .94/.02/.02/.02,
    500 K, batch 16) with ECIs scaled for 40-50 % acceptance, 1.2e5 attempts on the reference's
    mt19937_64 stream: the final lattice is the reference's, and the Metropolis test rejects often."""
    G, load = golden
    name = "cmc_config2_strong"
    fx = load(name)
    kind, el, *_, T, rseed, steps = G.BASELINE_CASES[name]
    _, coeffs, n, sp = G.baseline_inputs(name)
    ctx = api.Context(api.Model.from_coefficients(coeffs, list(el)))
    ctx.set_lattices([n], sp)
    e, done, acc = ctx.cmc_run(T, steps + 1, mode=0, seed=rseed, batch=G.BASELINE_CMC_BATCH)
    assert done == int(fx["final_steps"])
    assert np.array_equal(ctx.get_lattices(), fx["final_species"])
    np.testing.assert_allclose(e, fx["final_energy"][0], rtol=0, atol=1e-9)
    assert 0.3 < acc / done < 0.7, acc / done


def _replay_check(api, oracle_mod, G, el, coeffs, ns, species, replica, trace, ev, every=7,
                  tol=(EA_RTOL, DE_ATOL, 0.0)):
    """Replays a traced replica on the host and checks the traced events of
    every `every`-th step against the oracle's barriers for that lattice
    (tol: barrier rtol, energy-change atol, energy-change rtol)."""
    n = int(ns[replica])
    off = int(np.concatenate([[0], np.cumsum(4 * ns.astype(np.int64) ** 3)])[replica])
    sp = species[off: off + 4 * n ** 3].copy()
    lat = oracle_mod.Lattice(n)
    m = oracle_mod.Model(el, coeffs, lat)
    x = sorted(set(el) | {"X"}).index("X")
    for s in range(len(trace)):
        vac, tgt = int(trace["vacancy"][s]), int(trace["target"][s])
        assert sp[vac] == x
        if s % every == 0:
            for k in range(12):
                j = int(ev[s, k, 0])
                q = oracle_mod.quartic(m, lat, sp, vac, j)
                np.testing.assert_allclose(ev[s, k, 1], q[0], rtol=tol[0])
                np.testing.assert_allclose(ev[s, k, 2], q[1], rtol=tol[2], atol=tol[1])
        sp[vac], sp[tgt] = sp[tgt], x
    return sp


@pytest.mark.parametrize("rates", [0, 1])
def test_batched_kmc_against_oracle(api, golden, oracle_mod, rates):
    """Uneven replicas in one persistent launch (Philox streams): every traced
    event matches the oracle (FP64 rates: EA_RTOL; FP32 rates: 1e-6 relative),
    lattices stay consistent, energies match the census."""
    from latticemontecarlo_gb300 import synthetic as S
    G, load = golden
    el = ("Al", "Mg", "Zn")
    coeffs = S.make_coefficients(el, 3)
    ns, sp, temps = S.batched_replicas(9, 64, n_range=(8, 12), fractions={"Al": 0.8, "Mg": 0.1, "Zn": 0.1})
    ctx = api.Context(api.Model.from_coefficients(coeffs, list(el)))
    ctx.set_lattices(ns, sp)
    e_before = np.array([ctx.energy(r)[0] for r in range(ns.size)])
    ctx.kmc_init(temps, seed=99, rng=1, rates=rates)
    steps = 300
    tr, ev = ctx.kmc_run(steps, trace_replica=37, events=True)
    final = ctx.get_lattices()
    vac, nsteps, time, energy = ctx.kmc_state()
    assert np.all(nsteps == steps) and np.all(time > 0)
    # species conserved per replica, one vacancy at the recorded site
    offs = np.concatenate([[0], np.cumsum(4 * ns.astype(np.int64) ** 3)])
    x = 2
    for r in range(ns.size):
        a, b = sp[offs[r]:offs[r + 1]], final[offs[r]:offs[r + 1]]
        assert np.array_equal(np.bincount(a, minlength=4), np.bincount(b, minlength=4))
        assert b[vac[r]] == x
    e_after = np.array([ctx.energy(r)[0] for r in range(ns.size)])
    np.testing.assert_allclose(e_after - e_before, energy, rtol=0, atol=1e-9)
    tol = (EA_RTOL, DE_ATOL, 0.0) if rates == 1 else (F32_RTOL, 1e-12, F32_RTOL)
    replay = _replay_check(api, oracle_mod, G, el, coeffs, ns, sp, 37, tr, ev, tol=tol)
    assert np.array_equal(replay, final[offs[37]:offs[38]])


def test_cmc_throughput_properties(api, golden):
    """Priority-resolved parallel swaps: composition conserved, the reported
    energy change equals the census difference, acceptance is Metropolis-like."""
    from latticemontecarlo_gb300 import synthetic as S
    G, load = golden
    el = ("Al", "Cu", "Mg", "Zn")
    coeffs = S.make_coefficients(el, 11)
    n = 12
    sp = S.make_lattice(n, {"Al": 0.94, "Cu": 0.02, "Mg": 0.02, "Zn": 0.02}, 0, 5, el)
    ctx = api.Context(api.Model.from_coefficients(coeffs, list(el)))
    ctx.set_lattices([n], sp)
    e0, _ = ctx.energy()
    e, done, acc = ctx.cmc_run(500.0, 20 * sp.size, mode=1, seed=4)
    assert done >= 20 * sp.size and 0 < acc < done
    # rounds counted; the survivors of a round are disjoint pairs of sites
    rounds = ctx.cmc_rounds()
    assert 0 < rounds and done / rounds <= sp.size / 2
    out = ctx.get_lattices()
    assert np.array_equal(np.bincount(out, minlength=5), np.bincount(sp, minlength=5))
    e1, _ = ctx.energy()
    np.testing.assert_allclose(e1 - e0, e, rtol=0, atol=1e-9)


def test_census_full_size(api, oracle_mod):
    """EnergyPredictor census at the large-lattice size (n = 64, 2^20 sites): exact counts."""
    from latticemontecarlo_gb300 import synthetic as S
    el = ("Al", "Cu", "Mg", "Zn")
    coeffs = S.make_coefficients(el, 11, calibrate=False)
    sp = S.make_lattice(64, {"Al": 0.93, "Cu": 0.01, "Mg": 0.03, "Zn": 0.03}, 64, 8, el)
    ctx = api.Context(api.Model.from_coefficients(coeffs, list(el)))
    ctx.set_lattices([64], sp)
    e, counts = ctx.energy()
    lat = oracle_mod.Lattice(64)
    m = oracle_mod.Model(el, coeffs, lat)
    e_ref, c_ref = oracle_mod.energy(m, lat, sp)
    assert np.array_equal(counts, c_ref)
    assert e == e_ref


@pytest.mark.parametrize("base_fraction,warps", [(0.96, 1), (0.85, 1), (0.85, 2), (0.78, 1), (0.55, 1)])
def test_sparse_equals_dense_bitwise(api, base_fraction, warps):
    """The sparse evaluation (single-site plus pair corrections to the all-base
    sums) and the dense cluster sums give identical trajectories (exact int64
    sums). At 0.85 most clusters near a solute hold several solutes; near 0.78
    the neighbourhood's solute count crosses the sparse limit from step to step
    (both paths in one trajectory); at 0.55 every step takes the dense path."""
    from latticemontecarlo_gb300 import synthetic as S
    el = ("Al", "Cu", "Mg", "Zn")
    coeffs = S.make_coefficients(el, 21)
    rest = (1.0 - base_fraction) / 3
    ns, sp, temps = S.batched_replicas(5, 24, n_range=(8, 11),
                                       fractions={"Al": base_fraction, "Cu": rest, "Mg": rest, "Zn": rest},
                                       elements=el)
    out = []
    for evaluation in (0, 1):
        ctx = api.Context(api.Model.from_coefficients(coeffs, list(el)))
        ctx.set_lattices(ns, sp)
        ctx.kmc_init(temps, seed=17, rng=1, evaluation=evaluation, warps_per_replica=warps)
        tr, ev = ctx.kmc_run(400, trace_replica=3, events=True)
        out.append((ctx.get_lattices(), ctx.kmc_state(), tr, ev))
    (l0, s0, t0, e0), (l1, s1, t1, e1) = out
    assert np.array_equal(l0, l1)
    for a, b in zip(s0, s1):
        assert np.array_equal(a, b)
    assert np.array_equal(t0, t1) and np.array_equal(e0, e1)


@pytest.mark.parametrize("base_fraction", [0.96, 0.9])
def test_barrier_batch_sparse_equals_dense(api, oracle_mod, base_fraction):
    """lmc_barrier_batch's sparse path (runs of jumps that share a vacancy, evaluated once with the
    solvent-relative sums) gives the dense per-pair results bit for bit: the 12 jumps of every
    vacancy of a vacancy grid, a vacancy whose 1-3NN shells are all solute (more non-solvent sites
    than the sparse lists hold: its run falls back to the dense pairs), jumps asked singly and in a
    shuffled order, and pairs whose first site is not a vacancy; a vacancy with a second vacancy in
    its environments raises on both."""
    from latticemontecarlo_gb300 import synthetic as S
    el = ("Al", "Mg", "Zn")
    coeffs = S.make_coefficients(el, 8)
    n = 16
    rest = (1.0 - base_fraction) / 2
    sp = S.make_lattice(n, {"Al": base_fraction, "Mg": rest, "Zn": rest}, 0, 12, el)
    x = S.alphabet(el).index("X")
    m2 = 2 * n
    grid = [(a, b, c) for a in range(0, m2, 8) for b in range(0, m2, 8) for c in range(0, m2, 8)]
    vac = np.array([a * 2 * n * n + b * n + c // 2 for a, b, c in grid])
    sp[vac] = x
    sp[vac[0] + 1] = x  # a second vacancy inside vac[0]'s environments
    lat = oracle_mod.Lattice(n)
    sp[lat.neighbors(int(vac[1]))] = S.alphabet(el).index("Mg")  # a solute-rich neighbourhood
    ctx = api.Context(api.Model.from_coefficients(coeffs, list(el)))
    ctx.set_lattices([n], sp)
    grouped = np.array([[v, j] for v in vac[1:] for j in lat.neighbors(int(v))[:12]], np.int64)
    rng = np.random.default_rng(3)
    shuffled = grouped[rng.permutation(len(grouped))[:200]]
    others = []
    while len(others) < 40:  # non-vacancy first sites whose environments hold no vacancy
        a = int(rng.choice(np.flatnonzero(sp != x)))
        b = int(lat.neighbors(a)[rng.integers(12)])
        if sp[b] != x and not any(np.any(sp[v] == x) for v in lat.pair_lists(a, b)):
            others.append([a, b])
    pairs = np.concatenate([grouped, shuffled, np.array(others, np.int64)])
    out = []
    for evaluation in (0, 1):
        ctx.set_barrier_evaluation(evaluation)
        out.append(ctx.barrier_batch(pairs))
    for a, b in zip(out[0], out[1]):
        assert np.array_equal(a, b)
    bad = np.array([[vac[0], j] for j in lat.neighbors(int(vac[0]))[:12]], np.int64)
    for evaluation in (0, 1):
        ctx.set_barrier_evaluation(evaluation)
        with pytest.raises(Exception):  # X inside an environment, as the reference's encoder throws
            ctx.barrier_batch(bad)


def test_invalid_species_rejected(api, golden):
    from latticemontecarlo_gb300 import LmcError
    G, load = golden
    el, coeffs, n, sp = G.case_inputs("pred_ternary")
    ctx = api.Context(api.Model.from_coefficients(coeffs, list(el)))
    bad = sp.copy()
    bad[17] = 9
    with pytest.raises(LmcError) as e:
        ctx.set_lattices([n], bad)
    assert "species code out of range" in str(e.value)
