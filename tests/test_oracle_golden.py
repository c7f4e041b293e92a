"""The oracle restatement (oracle/lmc_oracle.c) against vectors produced by
the reference's own sources (tests/golden/, made by make_golden.py)."""
import ctypes as C

import numpy as np
import pytest


@pytest.mark.parametrize("n", [6, 8, 10])
def test_lattice_ids_and_neighbours(oracle_mod, golden, n):
    G, load = golden
    gz = load("geometry")
    lat = oracle_mod.Lattice(n)
    nn = np.stack([lat.neighbors(i) for i in range(lat.num_sites)])
    assert np.array_equal(nn, gz[f"n{n}_nn"])
    pos = np.stack([lat.position(i) for i in range(lat.num_sites)])
    assert np.array_equal(pos, gz[f"n{n}_pos"])


@pytest.mark.parametrize("n", [6, 8, 10])
def test_sorted_pair_and_site_lists(oracle_mod, golden, n):
    G, load = golden
    gz = load("geometry")
    lat = oracle_mod.Lattice(n)
    for k, (a, b) in enumerate(gz[f"n{n}_pairs"]):
        st, mm, m2 = lat.pair_lists(int(a), int(b))
        assert np.array_equal(st, gz[f"n{n}_state"][k])
        assert np.array_equal(mm, gz[f"n{n}_mmm"][k])
        assert np.array_equal(m2, gz[f"n{n}_mm2"][k])
    assert np.array_equal(lat.site_list(0), gz[f"n{n}_site0"])


def _canon(records):
    """orbit -> sorted list of index tuples (order inside an orbit is unspecified)."""
    out = {}
    for r in records:
        out.setdefault(int(r[0]), []).append(tuple(int(x) for x in r[1:] if x != -2))
    return {k: sorted(v) for k, v in out.items()}


@pytest.mark.parametrize("which,key", [(0, "map_state"), (1, "map_site"), (2, "map_mmm"), (3, "map_mm2")])
def test_cluster_mappings(oracle_mod, golden, which, key):
    G, load = golden
    gz = load("geometry")
    lat = oracle_mod.Lattice(10)
    got = lat.mapping(which)
    recs = []
    for g, size, sym, i0, i1, i2 in got:
        idx = [i0, i1, i2][:size]
        if which >= 2 and sym:
            idx = [-1] + idx
        recs.append([g] + idx)
    assert _canon(recs) == _canon(gz[key])


@pytest.mark.parametrize("name", ["pred_ternary", "pred_quaternary"])
def test_predictors(oracle_mod, golden, name):
    G, load = golden
    el, coeffs, n, sp = G.case_inputs(name)
    fx = load(name)
    lat = oracle_mod.Lattice(n)
    m = oracle_mod.Model(el, coeffs, lat)
    qi = 0
    for k, (a, b) in enumerate(fx["pair"]):
        a, b = int(a), int(b)
        if fx["jump_ok"][k]:
            q = oracle_mod.quartic(m, lat, sp, a, b)
            assert np.array_equal(q, fx["quartic"][qi][:4])
            cs, ce, mm, mf, mb = oracle_mod.encode(m, lat, sp, a, b)
            assert np.array_equal(cs, fx["state_start"][qi]) and np.array_equal(ce, fx["state_end"][qi])
            assert np.array_equal(mm, fx["enc_mmm"][qi])
            assert np.array_equal(mf, fx["enc_mm2_fwd"][qi]) and np.array_equal(mb, fx["enc_mm2_bwd"][qi])
            assert np.array_equal(oracle_mod.e0(m, lat, sp, a, b)[:2], fx["e0"][qi])
            qi += 1
        assert oracle_mod.pair_site_de(m, lat, sp, a, b) == fx["pairsite"][k]
    assert qi >= 48
    e, counts = oracle_mod.energy(m, lat, sp)
    assert e == fx["energy"]
    bonds = np.asarray([256, 3072, 1536, 6144, 12288, 6144, 12288, 6144], float)
    from latticemontecarlo_gb300 import synthetic as S
    labels = np.asarray(S.theta_labels(el))
    assert np.array_equal(counts / bonds[labels], fx["census_encode"])


def _feature_orbit_sizes(records, e: int) -> np.ndarray:
    """Per one-hot feature, the size of its orbit, from the reference's own MMM / MM2 mapping
    (GetOneHotParametersFromMap, EnergyUtility.cpp:753-792): an orbit of singlets has e features,
    of ordered pairs e^2, of symmetric pairs (flag -1) e(e+1)/2; each feature is the orbit's summed
    one-hot vector divided by the number of clusters in the orbit."""
    sizes = []
    for o in range(int(records[:, 0].max()) + 1):
        r = records[records[:, 0] == o]
        if r[0, 1] == -1:
            width = e * (e + 1) // 2
        else:
            width = e ** int(np.sum(r[0, 1:] >= 0))
        sizes += [len(r)] * width
    return np.asarray(sizes, float)


@pytest.mark.parametrize("name", ["pred_ternary", "pred_quaternary"])
def test_onehot_vectors_are_the_references(golden, name):
    """The integer one-hot numerators the GPU tests compare against are the reference's own FP
    vectors times orbit sizes taken from the reference's own mapping: numerator / size reproduces
    every printed FP feature exactly."""
    G, load = golden
    fx, gz = load(name), load("geometry")
    e = len(G.CASES[name][0])
    for key, mkey in (("enc_mmm", "map_mmm"), ("enc_mm2_fwd", "map_mm2"), ("enc_mm2_bwd", "map_mm2")):
        sizes = _feature_orbit_sizes(gz[mkey], e)
        assert sizes.size == fx[key].shape[1] == fx[key + "_fp"].shape[1]
        assert np.array_equal(fx[key] / sizes, fx[key + "_fp"]), key


def test_mt19937_and_distributions(oracle_mod, golden):
    G, load = golden
    fx = load("rng")
    L = oracle_mod.lib()

    class MT(C.Structure):
        _fields_ = [("mt", C.c_uint64 * 312), ("idx", C.c_int)]

    L.orc_mt_seed.argtypes = [C.POINTER(MT), C.c_uint64]
    L.orc_mt_next.restype, L.orc_mt_next.argtypes = C.c_uint64, [C.POINTER(MT)]
    L.orc_mt_uniform.restype, L.orc_mt_uniform.argtypes = C.c_double, [C.POINTER(MT)]
    L.orc_mt_below.restype, L.orc_mt_below.argtypes = C.c_uint64, [C.POINTER(MT), C.c_uint64]
    for key in fx.files:
        kind, seed, rr = key.split("_")
        m = MT()
        L.orc_mt_seed(C.byref(m), int(seed))
        raw = [L.orc_mt_next(C.byref(m)) for _ in range(64)]
        real = [L.orc_mt_uniform(C.byref(m)) for _ in range(64)]
        ints = [L.orc_mt_below(C.byref(m), int(rr)) for _ in range(64)]
        got = {"raw": np.array(raw, np.uint64), "real": np.array(real), "int": np.array(ints, np.uint64)}[kind]
        assert np.array_equal(got, fx[key]), key


def test_kmc_trajectory(oracle_mod, golden):
    G, load = golden
    el, coeffs, n, sp = G.case_inputs("kmc_ternary")
    fx = load("kmc_ternary")
    lat = oracle_mod.Lattice(n)
    m = oracle_mod.Model(el, coeffs, lat)
    steps = 1500
    tr, ev = oracle_mod.kmc(m, lat, sp.copy(), G.KMC_T, G.KMC_SEED, steps, events=True, memo=True)
    ref = fx["steps"][:steps]  # steps vacancy target selected Ea dE total time energy
    assert np.array_equal(tr[:, 1], ref[:, 2]) and np.array_equal(tr[:, 2], ref[:, 3])
    assert np.array_equal(tr[:, 3], ref[:, 4]) and np.array_equal(tr[:, 4], ref[:, 5])
    np.testing.assert_allclose(tr[:, 6], ref[:, 7], rtol=1e-15)
    np.testing.assert_allclose(tr[:, 7], ref[:, 8], rtol=0, atol=1e-15)
    assert np.array_equal(ev[: G.KMC_DETAIL], fx["events"])


def test_threaded_kmc_is_the_serial_trajectory(oracle_mod, golden):
    """The CPU baseline's threaded KineticMcFirstOmp restatement (12 barriers of a step on OpenMP
    threads) takes the reference's trajectory: the golden fixture's events, as the serial loop."""
    G, load = golden
    el, coeffs, n, sp = G.case_inputs("kmc_ternary")
    fx = load("kmc_ternary")
    lat = oracle_mod.Lattice(n)
    m = oracle_mod.Model(el, coeffs, lat)
    steps = 600
    tr, loop_s = oracle_mod.kmc_threads(m, lat, sp.copy(), G.KMC_T, G.KMC_SEED, steps, 4)
    ref = fx["steps"][:steps]  # steps vacancy target selected Ea dE total time energy
    assert np.array_equal(tr[:, 1], ref[:, 2]) and np.array_equal(tr[:, 2], ref[:, 3])
    assert np.array_equal(tr[:, 3], ref[:, 4]) and np.array_equal(tr[:, 4], ref[:, 5])
    np.testing.assert_allclose(tr[:, 6], ref[:, 7], rtol=1e-15)
    assert loop_s > 0
    # the thread count changes nothing but the time
    tr1, _ = oracle_mod.kmc_threads(m, lat, sp.copy(), G.KMC_T, G.KMC_SEED, 200, 1)
    tr3, _ = oracle_mod.kmc_threads(m, lat, sp.copy(), G.KMC_T, G.KMC_SEED, 200, 3)
    assert np.array_equal(tr1, tr3) and np.array_equal(tr1, tr[:200])


def test_cmc_trajectory(oracle_mod, golden):
    G, load = golden
    el, coeffs, n, sp = G.case_inputs("cmc_quaternary")
    fx = load("cmc_quaternary")
    lat = oracle_mod.Lattice(n)
    m = oracle_mod.Model(el, coeffs, lat)
    sp2 = sp.copy()
    done, e, acc, trace = oracle_mod.cmc(m, lat, sp2, G.CMC_T, G.CMC_SEED, G.CMC_STEPS + 1, G.CMC_BATCH, 0.0,
                                         trace=True)
    assert done == int(fx["final_steps"])
    assert np.array_equal(sp2, fx["final_species"])
    np.testing.assert_allclose(trace, fx["log"][:, 2], rtol=0, atol=1e-15)
    np.testing.assert_allclose(e, fx["final_energy"][0], rtol=0, atol=1e-15)


def _baseline_kmc_check(oracle_mod, G, fx, name):
    """The oracle's KineticMcFirstOmp over the whole run of a benchmark-configuration fixture."""
    kind, el, *_, T, rseed, steps = G.BASELINE_CASES[name]
    _, coeffs, n, sp = G.baseline_inputs(name)
    lat = oracle_mod.Lattice(n)
    m = oracle_mod.Model(el, coeffs, lat)
    tr, _ = oracle_mod.kmc(m, lat, sp, T, rseed, steps, memo=True)
    return tr


def test_baseline_kmc_trajectories(oracle_mod, golden):
    """KMC of the benchmark's one-trajectory configuration (n = 10, Al/Mg/Zn .96/.02/.02, 400 K) for
    its full 1e5 steps, with the benchmark's coefficients and with the ECIs scaled so |dE| ~ kT: the
    oracle selects the reference's event at every step (the two runs in parallel threads)."""
    from concurrent.futures import ThreadPoolExecutor
    G, load = golden
    names = ["kmc_config1", "kmc_config1_strong"]
    with ThreadPoolExecutor(2) as ex:
        trs = list(ex.map(lambda nm: _baseline_kmc_check(oracle_mod, G, load(nm), nm), names))
    for name, tr in zip(names, trs):
        fx = load(name)
        assert np.array_equal(tr[:, 1], fx["target"]), name
        assert np.array_equal(tr[:, 2], fx["selected"]), name
        k = fx["sample_steps"]
        got, ref = tr[k][:, 3:8], fx["sample"]  # Ea dE total time energy
        # barriers, energy changes and energies bit for bit; the total rate and the clock to the last
        # bit or two (the reference's OpenMP reduction order of the 12 rates is not sequential)
        assert np.array_equal(got[:, [0, 1, 4]], ref[:, [0, 1, 4]]), name
        np.testing.assert_allclose(got[:, 2:4], ref[:, 2:4], rtol=1e-15, atol=0)


def test_baseline_cmc_trajectory(oracle_mod, golden):
    """CanonicalMcOmp at the benchmark's CMC size (n = 30, 108000 sites, batch 16) with ECIs scaled
    for 40-50 % acceptance at 500 K, 1.2e5 attempts: the oracle's final lattice and energies are the
    reference's."""
    G, load = golden
    name = "cmc_config2_strong"
    fx = load(name)
    kind, el, *_, T, rseed, steps = G.BASELINE_CASES[name]
    _, coeffs, n, sp = G.baseline_inputs(name)
    lat = oracle_mod.Lattice(n)
    m = oracle_mod.Model(el, coeffs, lat)
    done, e, acc, trace = oracle_mod.cmc(m, lat, sp, T, rseed, steps + 1, G.BASELINE_CMC_BATCH, 0.0, trace=True)
    assert done == int(fx["final_steps"])
    assert np.array_equal(sp, fx["final_species"])
    # the running energy to rounding (its dE terms are summed in the restatement's order)
    np.testing.assert_allclose(trace[fx["sample_steps"]], fx["sample_energy"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(e, fx["final_energy"][0], rtol=0, atol=1e-12)
    assert 0.3 < acc / done < 0.7, acc / done
