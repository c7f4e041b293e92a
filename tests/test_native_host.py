"""The C-ABI library: it loads, exports every symbol of include/lmc_gb300.h,
and its host-only paths (geometry, mappings, folding layout, integer
encodings) agree with the reference's vectors. No GPU needed."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


def header_functions():
    text = (ROOT / "include" / "lmc_gb300.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(lmc_[a-z0-9_]+)\s*\(", text)))


def test_exports_every_declared_symbol(native):
    names = header_functions()
    assert len(names) > 30
    for name in names:
        assert hasattr(native.lib, name), name
        assert name in native.SIGNATURES, f"{name} missing from the ctypes table"


def test_error_codes_and_messages(native):
    assert native.lib.lmc_strerror(native.LMC_ERR_OUT_OF_RANGE) == b"out of range"
    nb = np.zeros(42, np.int64)
    rc = native.lib.lmc_geom_neighbors(4, 0, nb.ctypes.data_as(C.POINTER(C.c_int64)))
    assert rc == native.LMC_ERR_INVALID_ARGUMENT
    assert b"n must be" in native.lib.lmc_last_error()
    st = np.zeros(60, np.int64)
    rc = native.lib.lmc_geom_pair_lists(10, 0, 1, st.ctypes.data_as(C.POINTER(C.c_int64)), None, None)
    assert rc == native.LMC_ERR_OUT_OF_RANGE  # sites 0 and 1 are second neighbours
    assert b"Neighbor not found" in native.lib.lmc_last_error()


def test_mapping_sizes(native):
    c = (C.c_int * 20)()
    native.check(native.lib.lmc_geom_mapping_sizes(c))
    assert list(c)[:8] == [2, 23, 12, 48, 44, 68, 136, 140]
    assert list(c)[8:16] == [1, 12, 6, 24, 24, 36, 72, 72]
    assert list(c)[16:20] == [91, 175, 614, 614]


@pytest.mark.parametrize("elements,expect", [(("Al", "Mg", "Zn"), (95, 711, 1401)),
                                             (("Al", "Cu", "Mg", "Zn"), (167, 1240, 2452))])
def test_layout(elements, expect):
    from latticemontecarlo_gb300 import Model
    m = Model.create(list(elements))
    assert (m.num_theta, m.f_mmm, m.f_mm2) == expect
    assert m.alphabet == sorted(set(elements) | {"X"})


def test_theta_labels_match_layout():
    from latticemontecarlo_gb300 import Model, synthetic as S
    for el in (("Al", "Mg", "Zn"), ("Al", "Cu", "Mg", "Zn")):
        assert len(S.theta_labels(el)) == Model.create(list(el)).num_theta


@pytest.mark.parametrize("n", [6, 8, 10])
def test_neighbour_lists(native, golden, n):
    G, load = golden
    gz = load("geometry")
    nb = np.zeros(42, np.int64)
    ptr = nb.ctypes.data_as(C.POINTER(C.c_int64))
    for site in range(4 * n ** 3):
        native.check(native.lib.lmc_geom_neighbors(n, site, ptr))
        assert np.array_equal(nb, gz[f"n{n}_nn"][site])


@pytest.mark.parametrize("n", [6, 8, 10])
def test_pair_lists(native, golden, n):
    """Same sites in every list; same order wherever the reference picks the
    frame's vertical vector as for an interior site (it picks by id order, so
    at the periodic boundary its frame can be the 180-degree rotated one,
    which permutes sites within orbits and leaves every feature unchanged)."""
    G, load = golden
    gz = load("geometry")
    st, mm, m2 = (np.zeros(k, np.int64) for k in (60, 58, 58))
    same_order = 0
    for k, (a, b) in enumerate(gz[f"n{n}_pairs"]):
        native.check(native.lib.lmc_geom_pair_lists(n, int(a), int(b), *[x.ctypes.data_as(C.POINTER(C.c_int64))
                                                                        for x in (st, mm, m2)]))
        for mine, ref in ((st, gz[f"n{n}_state"][k]), (mm, gz[f"n{n}_mmm"][k]), (m2, gz[f"n{n}_mm2"][k])):
            assert sorted(mine) == sorted(ref)
        same_order += np.array_equal(st, gz[f"n{n}_state"][k]) and np.array_equal(mm, gz[f"n{n}_mmm"][k]) and \
            np.array_equal(m2, gz[f"n{n}_mm2"][k])
    assert same_order > 0.5 * len(gz[f"n{n}_pairs"])


def test_site_list(native, golden):
    G, load = golden
    gz = load("geometry")
    out = np.zeros(43, np.int64)
    for n in (6, 8, 10):
        native.check(native.lib.lmc_geom_site_list(n, 0, out.ctypes.data_as(C.POINTER(C.c_int64))))
        assert np.array_equal(out, gz[f"n{n}_site0"])


@pytest.mark.parametrize("which,key", [(0, "map_mmm"), (1, "map_mm2")])
def test_env_mappings(native, golden, which, key):
    """Orbit structure of the MMM / MM2 mappings equals the reference's
    (orbit order, membership, first/second order inside each cluster)."""
    G, load = golden
    ref = {}
    for r in load("geometry")[key]:
        idx = [int(x) for x in r[1:] if x != -2 and x != -1]
        ref.setdefault(int(r[0]), []).append(tuple(idx))
    n = C.c_int()
    native.check(native.lib.lmc_geom_env_mapping(which, None, 0, C.byref(n)))
    out = np.zeros((n.value, 3), np.int32)
    native.check(native.lib.lmc_geom_env_mapping(which, out.ctypes.data_as(C.POINTER(C.c_int32)), n.value,
                                                 C.byref(n)))
    mine = {}
    for o, a, b in out:
        mine.setdefault(int(o), []).append((int(a),) if b < 0 else (int(a), int(b)))
    assert {k: sorted(v) for k, v in mine.items()} == {k: sorted(v) for k, v in ref.items()}


@pytest.mark.parametrize("name", ["pred_ternary", "pred_quaternary"])
def test_host_encodings_bit_exact(golden, name):
    from latticemontecarlo_gb300 import Model
    G, load = golden
    el, coeffs, n, sp = G.case_inputs(name)
    fx = load(name)
    m = Model.create(list(el))
    qi = 0
    for k, (a, b) in enumerate(fx["pair"]):
        if not fx["jump_ok"][k]:
            continue
        cs, ce, mm, mf, mb = m.host_encode_pair(n, sp, int(a), int(b))
        assert np.array_equal(cs, fx["state_start"][qi]) and np.array_equal(ce, fx["state_end"][qi])
        assert np.array_equal(mm, fx["enc_mmm"][qi])
        assert np.array_equal(mf, fx["enc_mm2_fwd"][qi]) and np.array_equal(mb, fx["enc_mm2_bwd"][qi])
        qi += 1


def test_model_json_roundtrip(tmp_path, golden):
    from latticemontecarlo_gb300 import Model, LmcError, write_coefficients
    G, load = golden
    el, coeffs, n, sp = G.case_inputs("pred_ternary")
    p = write_coefficients(coeffs, tmp_path / "c.json")
    m = Model.from_json(p, list(el))
    assert m.num_theta == 95
    with pytest.raises(LmcError) as e:
        Model.from_json(tmp_path / "missing.json", list(el))
    assert e.value.code == 3 and "Cannot open" in str(e.value)
    bad = dict(coeffs)
    bad["Base"] = {"theta": coeffs["Base"]["theta"][:-1]}
    write_coefficients(bad, tmp_path / "bad.json")
    with pytest.raises(LmcError):
        Model.from_json(tmp_path / "bad.json", list(el))
