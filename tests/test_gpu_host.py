"""C++ host mirror on the GPU, against the reference's golden vectors and the oracle:

* the predictor classes (pred::VacancyMigrationPredictorQuarticLru / E0,
  EnergyChangePredictorPairSite, EnergyPredictor) with the reference's
  signatures, on a CFG file read by cfg::Config::ReadConfig;
* `lmc_gb300 -p param.txt` with simulation_method KineticMcFirstOmp: every row
  of kmc_log.txt (time, T, energy, Ea, dE, atom id of the jumping atom,
  unwrapped vacancy position) against the oracle trajectory replayed on the host;
* simulation_method CanonicalMcOmp: cmc_log.txt energies and the final
  configuration against the oracle's CanonicalMcOmp run on the same stream."""
import gzip
import json
import subprocess

import numpy as np
import pytest

from host_util import EXE, build_check, write_cfg

pytestmark = pytest.mark.gpu

EA_RTOL = 1e-9
DE_ATOL = 1e-12


@pytest.fixture(scope="module")
def check(native):
    import importlib.util
    from host_util import PKG
    spec = importlib.util.spec_from_file_location("lmc_build", PKG / "build.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.build_host()
    return build_check()


def _alphabet(el):
    return sorted(set(el) | {"X"})


def test_predictor_classes(check, golden, tmp_path):
    G, load = golden
    fx = load("pred_ternary")
    el, coeffs, n, sp = G.case_inputs("pred_ternary")
    write_cfg(tmp_path / "start.cfg", n, sp, _alphabet(el))
    (tmp_path / "coeffs.json").write_text(json.dumps(coeffs))
    jumps = fx["pair"][fx["jump_ok"].astype(bool)]
    pairs = fx["pair"]
    args = [str(check), "predict", str(tmp_path / "coeffs.json"), str(tmp_path / "start.cfg"), ",".join(el),
            str(len(jumps))]
    args += [str(int(v)) for v in np.concatenate([jumps, pairs]).reshape(-1)]
    r = subprocess.run(args, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = r.stdout.strip().splitlines()
    assert lines[-2] == "out_of_range"
    q = np.array([list(map(float, ln.split())) for ln in lines[:len(jumps)]])
    de = np.array([float(ln) for ln in lines[len(jumps):len(jumps) + len(pairs)]])
    np.testing.assert_allclose(q[:, 0], fx["quartic"][:, 0], rtol=EA_RTOL)
    np.testing.assert_allclose(q[:, 1], fx["quartic"][:, 1], rtol=0, atol=DE_ATOL)
    np.testing.assert_allclose(q[:, 2], fx["e0"][:, 0], rtol=EA_RTOL, atol=1e-15)
    np.testing.assert_allclose(de, fx["pairsite"], rtol=0, atol=DE_ATOL)
    assert float(lines[-1]) == float(fx["energy"])


def _run(tmp_path, params):
    (tmp_path / "param.txt").write_text("".join(f"{k} {v}\n" for k, v in params.items()))
    r = subprocess.run([str(EXE), "-p", "param.txt"], capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == 0, r.stdout + r.stderr
    return r


def _read_log(path):
    # the reference prints Vector_d values space-separated under tab-separated headers
    lines = path.read_text().strip().splitlines()
    return lines[0].split("\t"), np.array([[float(v) for v in ln.split()] for ln in lines[1:]])


def test_kmc_executable(check, golden, oracle_mod, tmp_path):
    G, load = golden
    el, coeffs, n, sp = G.case_inputs("kmc_ternary")
    alpha = _alphabet(el)
    write_cfg(tmp_path / "start.cfg", n, sp, alpha)
    (tmp_path / "coeffs.json").write_text(json.dumps(coeffs))
    steps = 300
    _run(tmp_path, {"simulation_method": "KineticMcFirstOmp", "config_filename": "start.cfg",
                    "json_coefficients_filename": "coeffs.json", "log_dump_steps": 1, "config_dump_steps": 100,
                    "maximum_steps": steps, "thermodynamic_averaging_steps": 0, "temperature": G.KMC_T,
                    "element_set": " ".join(el), "seed": G.KMC_SEED})
    head, log = _read_log(tmp_path / "kmc_log.txt")
    assert head == ["steps", "time", "temperature", "energy", "Ea", "dE", "selected", "vac1", "vac2", "vac3"]
    # Simulate runs while steps <= maximum_steps: maximum_steps + 1 steps
    lat = oracle_mod.Lattice(n)
    m = oracle_mod.Model(el, coeffs, lat)
    ref, _ = oracle_mod.kmc(m, lat, sp.copy(), G.KMC_T, G.KMC_SEED, steps + 1)
    assert log.shape[0] == steps + 1
    assert np.array_equal(log[:, 0], np.arange(steps + 1))
    t_before = np.concatenate([[0.0], ref[:-1, 6]])
    e_before = np.concatenate([[0.0], ref[:-1, 7]])
    np.testing.assert_allclose(log[:, 1], t_before, rtol=1e-9, atol=1e-300)
    assert np.all(log[:, 2] == G.KMC_T)
    np.testing.assert_allclose(log[:, 3], e_before, rtol=0, atol=1e-10)
    np.testing.assert_allclose(log[:, 4], ref[:, 3], rtol=EA_RTOL)
    np.testing.assert_allclose(log[:, 5], ref[:, 4], rtol=0, atol=DE_ATOL)
    # atom ids (atom i starts on lattice id i) and the unwrapped vacancy position, replayed here
    atom = np.arange(4 * n ** 3)
    shift = np.zeros((atom.size, 3))
    L = n * 4.046

    def rel(i):
        plane = 2 * n * n
        hx, rem = divmod(int(i), plane)
        hy, k = divmod(rem, n)
        return np.array([hx, hy, 2 * k + ((hx + hy) & 1)]) / (2.0 * n)

    for s in range(steps + 1):
        vac, tgt = int(ref[s, 0]), int(ref[s, 1])
        assert log[s, 6] == atom[tgt]
        np.testing.assert_allclose(log[s, 7:10], (rel(vac) + shift[atom[vac]]) * L, rtol=0, atol=1e-9)
        d = rel(tgt) - rel(vac)
        img = np.where(np.abs(d) > 0.5 + 1e-8, np.floor(d + 0.5), 0)
        shift[atom[vac]] -= img
        shift[atom[tgt]] += img
        atom[vac], atom[tgt] = atom[tgt], atom[vac]
    for name in ("0.cfg.gz", "100.cfg.gz", "200.cfg.gz", "300.cfg.gz", "end.cfg.gz"):
        assert (tmp_path / name).exists(), name
    # end.cfg.gz is the lattice before the last step's jump
    txt = gzip.decompress((tmp_path / "end.cfg.gz").read_bytes()).decode().splitlines()
    assert txt[0] == f"Number of particles = {4 * n ** 3}"


def test_cmc_executable(check, golden, oracle_mod, tmp_path):
    G, load = golden
    el, coeffs, n, sp = G.case_inputs("cmc_quaternary")
    alpha = _alphabet(el)
    write_cfg(tmp_path / "start.cfg", n, sp, alpha)
    (tmp_path / "coeffs.json").write_text(json.dumps(coeffs))
    steps, batch, avg = 3000, G.CMC_BATCH, 200
    _run(tmp_path, {"simulation_method": "CanonicalMcOmp", "config_filename": "start.cfg",
                    "json_coefficients_filename": "coeffs.json", "log_dump_steps": 1, "config_dump_steps": 100000,
                    "maximum_steps": steps, "thermodynamic_averaging_steps": avg, "temperature": G.CMC_T,
                    "element_set": " ".join(el), "seed": G.CMC_SEED, "cmc_batch": batch})
    head, log = _read_log(tmp_path / "cmc_log.txt")
    assert head == ["steps", "temperature", "energy", "average_energy", "absolute_energy"]
    lat = oracle_mod.Lattice(n)
    m = oracle_mod.Model(el, coeffs, lat)
    work = sp.copy()
    done, e_final, acc, trace = oracle_mod.cmc(m, lat, work, G.CMC_T, G.CMC_SEED, steps + 1, batch, trace=True)
    # Simulate finishes the batch it is in: steps_ may pass maximum_steps_ (CanonicalMcOmp.cpp:82-90)
    assert done >= steps + 1 and log.shape[0] == done
    np.testing.assert_allclose(log[:, 2], trace, rtol=0, atol=1e-10)
    # ThermodynamicAveraging over the last `avg` energies (ThermodynamicAveraging.cpp:6-42)
    beta = 1.0 / 8.617333262145e-5 / G.CMC_T
    for s in (0, 57, 1999, done - 1):
        w = trace[max(0, s + 1 - avg): s + 1]
        mu = w.mean()
        x = w - mu
        ref_avg = (x * np.exp(-x * beta)).sum() / np.exp(-x * beta).sum() + mu
        np.testing.assert_allclose(log[s, 3], ref_avg, rtol=1e-9, atol=1e-12)
    e0, _ = oracle_mod.energy(m, lat, sp)
    np.testing.assert_allclose(log[:, 4], e0 + trace, rtol=0, atol=1e-9)


def test_chain_kmc_executable(check, golden, oracle_mod, tmp_path):
    """simulation_method KineticMcChainOmpi: kmc_log.txt rows against the oracle's chain KMC."""
    G, load = golden
    el, coeffs, n, sp = G.case_inputs("kmc_ternary")
    write_cfg(tmp_path / "start.cfg", n, sp, _alphabet(el))
    (tmp_path / "coeffs.json").write_text(json.dumps(coeffs))
    steps = 40
    _run(tmp_path, {"simulation_method": "KineticMcChainOmpi", "config_filename": "start.cfg",
                    "json_coefficients_filename": "coeffs.json", "log_dump_steps": 1, "config_dump_steps": 1000,
                    "maximum_steps": steps, "thermodynamic_averaging_steps": 0, "temperature": G.KMC_T,
                    "element_set": " ".join(el), "seed": G.KMC_SEED})
    head, log = _read_log(tmp_path / "kmc_log.txt")
    assert head[:6] == ["steps", "time", "temperature", "energy", "Ea", "dE"]
    lat = oracle_mod.Lattice(n)
    m = oracle_mod.Model(el, coeffs, lat)
    ref = oracle_mod.kmc_chain(m, lat, sp.copy(), G.KMC_T, G.KMC_SEED, steps + 1, rng=0)
    assert log.shape[0] == steps + 1
    t_before = np.concatenate([[0.0], ref[:-1, 6]])
    e_before = np.concatenate([[0.0], ref[:-1, 7]])
    np.testing.assert_allclose(log[:, 1], t_before, rtol=1e-9, atol=1e-300)
    np.testing.assert_allclose(log[:, 3], e_before, rtol=0, atol=1e-10)
    np.testing.assert_allclose(log[:, 4], ref[:, 3], rtol=EA_RTOL)
    np.testing.assert_allclose(log[:, 5], ref[:, 4], rtol=0, atol=DE_ATOL)


def _solute_config(n, solvent, solutes, seed, oracle_mod, alpha):
    """GenerateSoluteConfig as the host mirror restates it: mt19937_64(seed + 1), uniform over the
    sorted available sites, each placed solute removing itself and its 1-3NN sites."""
    lat = oracle_mod.Lattice(n)
    sp = np.full(4 * n ** 3, alpha.index(solvent), np.int8)
    g = oracle_mod.Mt19937_64(seed + 1)
    available = list(range(sp.size))
    for el, count in sorted(solutes.items()):
        for _ in range(count):
            site = available[g.below(len(available))]
            sp[site] = alpha.index(el)
            gone = {site} | set(int(v) for v in lat.neighbors(site))
            available = [v for v in available if v not in gone]
    return sp


def test_sa_executable(check, oracle_mod, tmp_path):
    """simulation_method SimulatedAnnealing: the solute configuration, the initial energy from the
    chemical potentials, and every sa_log.txt row against the oracle's annealing run."""
    from latticemontecarlo_gb300 import synthetic as S
    el = ("Al", "Mg", "Zn")
    alpha = _alphabet(el)
    coeffs = S.make_coefficients(el, 13)
    (tmp_path / "coeffs.json").write_text(json.dumps(coeffs))
    n, seed, max_steps, T0 = 8, 41, 1500, 700.0
    solutes = {"Mg": 12, "Zn": 9}
    r = _run(tmp_path, {"simulation_method": "SimulatedAnnealing", "json_coefficients_filename": "coeffs.json",
                        "factor": n, "solvent_element": "Al", "solute_element_set": "Mg Zn",
                        "solute_number_set": "12 9", "log_dump_steps": 10, "config_dump_steps": 1000,
                        "maximum_steps": max_steps, "initial_temperature": T0, "seed": seed})
    sp = _solute_config(n, "Al", solutes, seed, oracle_mod, alpha)
    lat = oracle_mod.Lattice(n)
    m = oracle_mod.Model(el, coeffs, lat)
    # initial energy: cluster vs pure solvent minus the solutes' chemical potentials (15^3 boxes)
    lat15 = oracle_mod.Lattice(15)
    m15 = oracle_mod.Model(el, coeffs, lat15)
    pure15 = np.full(4 * 15 ** 3, alpha.index("Al"), np.int8)
    e_pure15, _ = oracle_mod.energy(m15, lat15, pure15)
    mu = {}
    for e in ("Mg", "Zn"):
        one = pure15.copy()
        one[0] = alpha.index(e)
        mu[e] = oracle_mod.energy(m15, lat15, one)[0] - e_pure15
    e_abs0, _ = oracle_mod.energy(m, lat, sp)
    e_pure, _ = oracle_mod.energy(m, lat, np.full_like(sp, alpha.index("Al")))
    e0 = (e_abs0 - e_pure) - (12 * mu["Mg"] + 9 * mu["Zn"])
    assert f"initial_energy = " in r.stdout
    np.testing.assert_allclose(float(r.stdout.split("initial_energy = ")[1].split()[0]), e0, rtol=0, atol=1e-9)
    ref, state = oracle_mod.sa(m, lat, sp.copy(), T0, seed, max_steps, max_steps + 1, e0)
    lines = (tmp_path / "sa_log.txt").read_text().strip().splitlines()
    assert lines[0].split("\t") == ["steps", "temperature", "energy", "lowest_energy", "absolute_energy"]
    rows = np.array([[float(v) for v in ln.split("\t")] for ln in lines[1:]])
    periodic = rows[np.isin(rows[:, 0], np.arange(0, max_steps + 1, 10))]
    s = periodic[:, 0].astype(int)
    # the same step can appear twice (an improvement line, then the periodic line): compare the last
    np.testing.assert_allclose(periodic[:, 1], ref[s, 5], rtol=1e-12)
    np.testing.assert_allclose(periodic[:, 2], ref[s, 4], rtol=0, atol=1e-9)
    np.testing.assert_allclose(periodic[:, 4] - periodic[:, 2], e_abs0 - e0, rtol=0, atol=1e-9)
    assert (tmp_path / "lowest_energy.cfg.gz").exists() or np.all(ref[:, 4] >= e0 - 1e-4)
