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
