"""C++ host mirror on the CPU: the executable's command line and errors, CFG
write/read with atom and image tracking, parameter parsing."""
import subprocess

import pytest

from host_util import EXE, build_check


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


def test_parameter_keys(check, tmp_path):
    p = tmp_path / "param.txt"
    p.write_text("# comment\n\nsimulation_method KineticMcFirstOmp\nconfig_filename start.cfg\n"
                 "json_coefficients_filename c.json\nlog_dump_steps 10\nconfig_dump_steps 100\nmaximum_steps 1000\n"
                 "temperature 400\nelement_set Al Mg Zn\nrate_corrector true\nearly_stop false\nsolute_disp true\n"
                 "seed 42\nunknown_key 7\n")
    r = subprocess.run([str(check), "param", str(p)], capture_output=True, text=True)
    assert r.stdout.strip() == "KineticMcFirstOmp|start.cfg|c.json|10|100|1000|400|101|42|Al,Mg,Zn,"
