"""C++ host mirror on the CPU: the executable's command line and errors, CFG
write/read with atom and image tracking, parameter parsing."""
import subprocess

import pytest

from host_util import EXE, ROOT, build_check


@pytest.fixture(scope="module")
def check(native):
    import importlib.util
    from host_util import PKG
    spec = importlib.util.spec_from_file_location("lmc_build", PKG / "build.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.build_host()
    return build_check()


def test_executable_command_line(check, tmp_path):
    r = subprocess.run([str(EXE)], capture_output=True, text=True)
    assert r.returncode == 1 and "No input parameter filename." in r.stdout
    r = subprocess.run([str(EXE), "-p", str(tmp_path / "missing.txt")], capture_output=True, text=True)
    assert r.returncode == 1 and f"Cannot open {tmp_path / 'missing.txt'}" in r.stderr
    p = tmp_path / "p.txt"
    p.write_text("simulation_method Nope\n")
    r = subprocess.run([str(EXE), "-p", str(p)], capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 0 and "No such method: Nope" in r.stdout


def test_cfg_roundtrip(check, tmp_path):
    r = subprocess.run([str(check), "cfg-roundtrip", str(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("OK") and r.stdout.split()[-1] == "Al"
    gz = (tmp_path / "a.cfg.gz").read_bytes()
    assert gz[:2] == b"\x1f\x8b"


def test_element_set_order(check):
    """std::set<Element> iterates in name order (Element.hpp:44-46), as the reference's does."""
    r = subprocess.run([str(check), "element-order", "Zn,Al,X,Mg,Cu,Sn"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.split() == ["Al", "Cu", "Mg", "Sn", "X", "Zn"]


def test_parameter_keys(check, tmp_path):
    p = tmp_path / "param.txt"
    p.write_text("# comment\n\nsimulation_method KineticMcFirstOmp\nconfig_filename start.cfg\n"
                 "json_coefficients_filename c.json\nlog_dump_steps 10\nconfig_dump_steps 100\nmaximum_steps 1000\n"
                 "temperature 400\nelement_set Al Mg Zn\nrate_corrector true\nearly_stop false\nsolute_disp true\n"
                 "seed 42\nunknown_key 7\n")
    r = subprocess.run([str(check), "param", str(p)], capture_output=True, text=True)
    assert r.stdout.strip() == "KineticMcFirstOmp|start.cfg|c.json|10|100|1000|400|101|42|Al,Mg,Zn,"


def test_parameter_analysis_keys(check, tmp_path):
    """The reference's remaining keys (Parameter.cpp:66-80,125-126) are parsed into its field names."""
    p = tmp_path / "param.txt"
    p.write_text("simulation_method Ansys\ninitial_steps 100\nincrement_steps 50\nsmallest_cluster_criteria 3\n"
                 "solvent_bond_criteria 4\nescape_temperature 600\ndecrement_temperature 10\n"
                 "early_stop_steps 7\nmap_filename map9.txt\n")
    r = subprocess.run([str(check), "param-analysis", str(p)], capture_output=True, text=True)
    assert r.stdout.strip() == "100|50|3|4|600|10|7|map9.txt"


def _golden_maps(tmp_path):
    import numpy as np
    g = np.load(ROOT / "tests" / "golden" / "map_quaternary.npz")
    files = {k: bytes(g[k]) for k in g.files}
    ref = tmp_path / "ref"
    ref.mkdir()
    for name, data in files.items():
        (ref / name).write_bytes(data)
    return files, ref


def test_map_files_match_reference(check, tmp_path):
    """Config::WriteLattice / WriteElement / WriteMap (Config.cpp:887-922) of the reference's own CFG
    file equal the files the reference wrote, byte for byte (tests/golden/map_quaternary.npz)."""
    files, ref = _golden_maps(tmp_path)
    out = tmp_path / "out"
    out.mkdir()
    r = subprocess.run([str(check), "map-write", str(ref / "start.cfg"), str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    for name in ("lattice.txt", "element.txt", "map.txt"):
        assert (out / name).read_bytes() == files[name], name


def test_map_read(check, tmp_path):
    """Config::ReadMap (Config.cpp:814-885) of the reference's map files gives the CFG's configuration
    (species and atom ids per lattice id); malformed map files fail with the reference's messages."""
    files, ref = _golden_maps(tmp_path)
    r = subprocess.run([str(check), "map-read", str(ref), str(ref / "start.cfg")], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.startswith("OK"), r.stdout + r.stderr
    ids = files["map.txt"].decode().split()
    for bad, msg in (([ids[1]] + ids[1:], f"Duplicate lattice id in map file: {ids[1]}"),
                     (["864"] + ids[1:], "Lattice id out of bounds in map file: 864")):
        (ref / "map.txt").write_text("\n".join(bad) + "\n")
        r = subprocess.run([str(check), "map-read", str(ref), str(ref / "start.cfg")], capture_output=True, text=True)
        assert r.returncode != 0 and msg in r.stdout + r.stderr, (msg, r.stdout + r.stderr)

