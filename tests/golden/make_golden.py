"""Generates the golden fixtures in tests/golden/ from the reference's own code.

Runs oracle/_ref/ref_harness (the reference's hot-path sources compiled
unmodified against the shim headers by oracle/build_ref.sh) on seeded inputs
and stores its outputs as compressed .npz files. Inputs are regenerated by the
tests from the same seeds (numpy PCG64, platform independent), so only the
outputs are committed.

    python tests/golden/make_golden.py            # needs the reference sources (oracle/build_ref.sh)
    python tests/golden/make_golden.py clusters   # only clusters_quaternary.npz
    python tests/golden/make_golden.py sitede     # only site_de_quaternary.npz
    python tests/golden/make_golden.py maps       # only map_quaternary.npz
    python tests/golden/make_golden.py pred       # only pred_ternary.npz / pred_quaternary.npz
    python tests/golden/make_golden.py baseline   # the benchmark configurations (KMC n=10 1e5 steps,
                                                  # CMC n=30 batch 16), see BASELINE_CASES

The fixtures pin the oracle restatement (oracle/lmc_oracle.c); the product is
then tested against the oracle and against these fixtures directly.
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from latticemontecarlo_gb300 import synthetic as S  # noqa: E402

HERE = Path(__file__).resolve().parent
HARNESS = ROOT / "oracle" / "_ref" / "ref_harness"

# Seeded cases (shared with tests/golden_cases.py through this module's constants).
TERNARY = ("Al", "Mg", "Zn")
QUATERNARY = ("Al", "Cu", "Mg", "Zn")
CASES = {
    # name: (elements, coeff_seed, n, fractions, vacancies, lattice_seed)
    "pred_ternary": (TERNARY, 7, 10, {"Al": 0.70, "Mg": 0.15, "Zn": 0.15}, 1, 101),
    "pred_quaternary": (QUATERNARY, 11, 8, {"Al": 0.70, "Cu": 0.10, "Mg": 0.10, "Zn": 0.10}, 1, 202),
    "kmc_ternary": (TERNARY, 7, 10, {"Al": 0.96, "Mg": 0.02, "Zn": 0.02}, 1, 303),
    "cmc_quaternary": (QUATERNARY, 11, 8, {"Al": 0.94, "Cu": 0.02, "Mg": 0.02, "Zn": 0.02}, 0, 404),
    "clusters_quaternary": (QUATERNARY, 11, 10, {"Al": 0.84, "Cu": 0.04, "Mg": 0.06, "Zn": 0.06}, 2, 505),
    "map_quaternary": (QUATERNARY, 11, 6, {"Al": 0.85, "Cu": 0.05, "Mg": 0.05, "Zn": 0.05}, 1, 606),
}
CLUSTER_SMALLEST, CLUSTER_BOND = 2, 3
KMC_T, KMC_SEED, KMC_STEPS, KMC_DETAIL = 400.0, 12345, 3000, 200
CMC_T, CMC_SEED, CMC_STEPS, CMC_BATCH = 500.0, 777, 6000, 4

# The benchmark configurations at their own sizes, generated from the same seeds as bench.py. The
# "strong" variants multiply "Base".theta by STRONG_ECI_SCALE: the synthetic pair ECIs, after the
# reference's division by the cluster counts, give a median |dE| of about 1e-3 kT, so almost every
# Metropolis test accepts; x800 gives a median |dE| of about kT and 40-50 % acceptance at 500 K, so
# the rejection branch and the energy dependence of the rates are exercised.
STRONG_ECI_SCALE = 800.0
BASELINE_CASES = {
    # name: (kind, elements, coeff_seed, eci_scale, n, fractions, vacancies, lattice_seed, T, rng_seed, steps)
    "kmc_config1": ("kmc", TERNARY, 11, 1.0, 10, {"Al": 0.96, "Mg": 0.02, "Zn": 0.02}, 1, 11, 400.0, 5, 100_000),
    "kmc_config1_strong": ("kmc", TERNARY, 11, STRONG_ECI_SCALE, 10, {"Al": 0.96, "Mg": 0.02, "Zn": 0.02}, 1, 11,
                           400.0, 5, 100_000),
    "cmc_config2_strong": ("cmc", QUATERNARY, 4321, STRONG_ECI_SCALE, 30,
                           {"Al": 0.94, "Mg": 0.02, "Zn": 0.02, "Cu": 0.02}, 0, 4321, 500.0, 777, 120_000),
}
BASELINE_CMC_BATCH = 16
BASELINE_SAMPLE = 50  # every 50th step's scalars are stored (the event sequence is stored in full)


def scaled_eci(coeffs: dict, factor: float) -> dict:
    """The coefficients with "Base".theta multiplied by `factor` (barrier blocks unchanged)."""
    out = dict(coeffs)
    out["Base"] = {"theta": (np.asarray(coeffs["Base"]["theta"]) * factor).tolist()}
    return out


def baseline_inputs(name: str):
    """Inputs of a benchmark-configuration case: the calibrated coefficients bench.py uses, "Base".theta
    scaled by the case's factor, and the lattice of the same seed."""
    kind, elements, cseed, scale, n, fractions, vac, lseed, T, rseed, steps = BASELINE_CASES[name]
    coeffs = S.make_coefficients(elements, cseed)
    if scale != 1.0:
        coeffs = scaled_eci(coeffs, scale)
    species = S.make_lattice(n, fractions, vac, lseed, elements)
    return elements, coeffs, n, species


def case_inputs(name: str):
    elements, cseed, n, fractions, vac, lseed = CASES[name]
    coeffs = S.make_coefficients(elements, cseed, calibrate=False)
    species = S.make_lattice(n, fractions, vac, lseed, elements)
    return elements, coeffs, n, species


def case_pairs(name: str, n: int, species: np.ndarray, rng_seed: int = 5):
    """Jump pairs: the 12 jumps of the vacancy plus random first-neighbour pairs
    whose environments hold no vacancy; swap pairs: random pairs at 1NN, 2NN,
    3NN and beyond."""
    from latticemontecarlo_gb300 import _native as N
    import ctypes as C
    rng = np.random.default_rng(rng_seed)
    nb = np.zeros(42, np.int64)

    def neighbors(s):
        N.check(N.lib.lmc_geom_neighbors(n, int(s), nb.ctypes.data_as(C.POINTER(C.c_int64))))
        return nb.copy()

    alpha = S.alphabet(CASES[name][0])
    x = alpha.index("X")
    jumps = []
    vac = np.flatnonzero(species == x)
    if vac.size:
        for j in neighbors(vac[0])[:12]:
            jumps.append((int(vac[0]), int(j)))
    nsites = species.size
    while len(jumps) < 48:
        a = int(rng.integers(nsites))
        j = int(neighbors(a)[rng.integers(12)])
        if species[a] == x or species[j] == x:
            continue
        # skip environments holding the vacancy (the reference's encoder has no X slot)
        st = np.zeros(60, np.int64)
        N.check(N.lib.lmc_geom_pair_lists(n, a, j, st.ctypes.data_as(C.POINTER(C.c_int64)), None, None))
        if np.any(species[st] == x):
            continue
        jumps.append((a, j))
    swaps = []
    for kind in range(40):
        a = int(rng.integers(nsites))
        if kind % 4 == 3:
            b = int(rng.integers(nsites))
        else:
            ring = neighbors(a)[[range(0, 12), range(12, 18), range(18, 42)][kind % 4]]
            b = int(ring[rng.integers(len(ring))])
        swaps.append((a, b))
    return np.asarray(jumps, np.int64), np.asarray(swaps, np.int64)


def run(args, cwd, env=None):
    out = subprocess.run([str(HARNESS), *map(str, args)], cwd=cwd, capture_output=True, text=True, env=env)
    if out.returncode != 0:
        raise RuntimeError(f"harness failed: {args}\n{out.stderr}")
    return out.stdout.splitlines()


def write_inputs(tmp: Path, elements, coeffs, species):
    alpha = S.alphabet(elements)
    (tmp / "coeffs.json").write_text(json.dumps(coeffs))
    (tmp / "species.txt").write_text(" ".join(alpha[c] for c in species))
    return ",".join(elements)


def parse_pred(lines, elements, coeffs):
    from latticemontecarlo_gb300.api import Model
    model = Model.create(list(elements))
    sz_mmm, sz_mm2 = model.orbit_sizes(0), model.orbit_sizes(1)
    res = {k: [] for k in ("pair", "quartic", "state_start", "state_end", "enc_mmm", "enc_mm2_fwd", "enc_mm2_bwd",
                           "enc_mmm_fp", "enc_mm2_fwd_fp", "enc_mm2_bwd_fp", "e0", "jump_ok", "pairsite")}
    cur_ok = None
    for ln in lines:
        f = ln.split()
        key, vals = f[0], f[1:]
        if key == "pair":
            if cur_ok is not None:
                res["jump_ok"].append(cur_ok)
            res["pair"].append([int(v) for v in vals])
            cur_ok = False
        elif key == "quartic":
            res["quartic"].append([float(v) for v in vals])
            cur_ok = True
        elif key in ("state_start", "state_end"):
            res[key].append([int(v) for v in vals])
        elif key == "enc_mmm":
            res[key + "_fp"].append(np.asarray(vals, float))  # the reference's own FP vector, as printed
            res[key].append(np.rint(np.asarray(vals, float) * sz_mmm).astype(np.int32))
        elif key in ("enc_mm2_fwd", "enc_mm2_bwd"):
            res[key + "_fp"].append(np.asarray(vals, float))
            res[key].append(np.rint(np.asarray(vals, float) * sz_mm2).astype(np.int32))
        elif key == "e0":
            res[key].append([float(v) for v in vals])
        elif key == "pairsite":
            res[key].append(float(vals[0]))
        elif key == "census_encode":
            res["census_encode"] = np.asarray(vals, float)
        elif key == "energy":
            res["energy"] = float(vals[0])
    res["jump_ok"].append(cur_ok)
    out = {k: np.asarray(v) for k, v in res.items()}
    return out


def make_geom(tmp: Path) -> dict:
    fx = {}
    for n in (6, 8, 10):
        rng = np.random.default_rng(n)
        nsites = 4 * n ** 3
        lines_pairs = []
        nnz = {}
        # pairs: first neighbours of boundary and interior sites
        sites = np.unique(np.concatenate([np.arange(0, 40), rng.integers(0, nsites, 40), nsites - 1 - np.arange(20)]))
        (tmp / "pairs.txt").write_text("")
        lines = run(["geom", n, tmp / "pairs.txt"], tmp)
        for ln in lines:
            f = ln.split()
            if f[0] == "nn":
                nnz[int(f[1])] = [int(v) for v in f[2:44]]
        for s in sites:
            for j in nnz[int(s)][:12:3]:
                lines_pairs.append((int(s), int(j)))
        (tmp / "pairs.txt").write_text("\n".join(f"{a} {b}" for a, b in lines_pairs))
        lines = run(["geom", n, tmp / "pairs.txt"], tmp)
        nn = np.zeros((nsites, 42), np.int32)
        pos = np.zeros((nsites, 3))
        st, mmm, mm2, maps = [], [], [], {"map_state": [], "map_site": [], "map_mmm": [], "map_mm2": []}
        for ln in lines:
            f = ln.split()
            if f[0] == "nn":
                nn[int(f[1])] = [int(v) for v in f[2:44]]
                pos[int(f[1])] = [float(v) for v in f[45:48]]
            elif f[0] == "state":
                st.append([int(v) for v in f[1:]])
            elif f[0] == "mmm":
                mmm.append([int(v) for v in f[1:]])
            elif f[0] == "mm2":
                mm2.append([int(v) for v in f[1:]])
            elif f[0] == "site0":
                fx[f"n{n}_site0"] = np.asarray([int(v) for v in f[1:]], np.int32)
            elif f[0] in maps:
                maps[f[0]].append(ln)
        fx[f"n{n}_nn"] = nn
        fx[f"n{n}_pos"] = pos
        fx[f"n{n}_pairs"] = np.asarray(lines_pairs, np.int64)
        fx[f"n{n}_state"] = np.asarray(st, np.int32)
        fx[f"n{n}_mmm"] = np.asarray(mmm, np.int32)
        fx[f"n{n}_mm2"] = np.asarray(mm2, np.int32)
        if n == 10:
            for k, v in maps.items():
                # records: orbit, cluster, index... flattened as (orbit, slot0, slot1, slot2) with -2 padding
                rec = []
                for ln in v:
                    parts = ln.split("|")
                    orbit = int(parts[0].split()[1])
                    for cl in parts[1:]:
                        idx = [int(t) for t in cl.split()]
                        rec.append([orbit] + idx + [-2] * (4 - len(idx)))
                fx[k] = np.asarray(rec, np.int32)
    return fx


def cluster_lists(n: int, species: np.ndarray, elements):
    """The oracle's solute clusters of the case (solvent Al), the clusters of single sites, and the
    two vacancies as lists of their own: the lists whose energies the reference evaluates."""
    from oracle import oracle as O
    lat = O.Lattice(n)
    solvent = S.alphabet(elements).index("Al")
    lists = O.solute_clusters(lat, species, solvent, CLUSTER_SMALLEST, CLUSTER_BOND)
    singles = O.solute_clusters(lat, species, solvent, 1, 12)
    x = S.alphabet(elements).index("X")
    extra = [c for c in singles if len(c) == 1][:4] + [np.flatnonzero(species == x)[:1]]
    return lists + extra


def make_clusters(tmp: Path) -> dict:
    elements, coeffs, n, species = case_inputs("clusters_quaternary")
    els = write_inputs(tmp, elements, coeffs, species)
    lists = cluster_lists(n, species, elements)
    (tmp / "lists.txt").write_text("\n".join(" ".join(str(int(v)) for v in c) for c in lists))
    lines = run(["cluster", n, tmp / "species.txt", tmp / "coeffs.json", els, "Al", tmp / "lists.txt"], tmp)
    energies, mu = [], {}
    for ln in lines:
        f = ln.split()
        if f[0] == "cluster":
            energies.append([float(v) for v in f[1:]])
        elif f[0] == "mu":
            mu[f[1]] = float(f[2])
    alpha = S.alphabet(elements)
    offsets = np.concatenate([[0], np.cumsum([len(c) for c in lists])]).astype(np.int64)
    return {"offsets": offsets, "members": np.concatenate(lists).astype(np.int64), "energies": np.asarray(energies),
            "mu": np.asarray([mu[a] for a in alpha])}


def site_de_lattice():
    """The clusters_quaternary lattice with its vacancies filled by Al (ExitTime's this_config): one
    X at a time keeps every cluster indexable."""
    elements, coeffs, n, species = case_inputs("clusters_quaternary")
    alpha = S.alphabet(elements)
    vac = np.flatnonzero(species == alpha.index("X"))
    filled = species.copy()
    filled[vac] = alpha.index("Al")
    return elements, coeffs, n, filled, vac


def site_de_queries(n: int, species: np.ndarray, elements, vac, seed: int = 9):
    """(site, from, to) codes: random sites, every element to the vacancy and some element swaps,
    plus every element at the two former vacancies."""
    rng = np.random.default_rng(seed)
    alpha = S.alphabet(elements)
    x = alpha.index("X")
    sites = np.concatenate([rng.choice(species.size, 60, replace=False), vac])
    q = []
    for s in sites:
        for f in range(len(alpha)):
            if f != x:
                q.append((int(s), f, x))
        q.append((int(s), int(species[s]), int(rng.integers(len(alpha)))))
    return np.asarray(q, np.int64)


def make_site_de(tmp: Path) -> dict:
    elements, coeffs, n, species, vac = site_de_lattice()
    els = write_inputs(tmp, elements, coeffs, species)
    q = site_de_queries(n, species, elements, vac)
    alpha = S.alphabet(elements)
    (tmp / "queries.txt").write_text("\n".join(f"{s} {alpha[f]} {alpha[t]}" for s, f, t in q))
    lines = run(["sitede", n, tmp / "species.txt", tmp / "coeffs.json", els, tmp / "queries.txt"], tmp)
    return {"queries": q, "de": np.asarray([float(ln.split()[1]) for ln in lines if ln.startswith("sitede")])}


def make_map_files(tmp: Path) -> dict:
    """The reference's own CFG and map files (WriteConfig / WriteLattice / WriteElement / WriteMap)
    of a 6^3-cell quaternary lattice: the CFG is the input of the host mirror's tests, the three map
    files are compared byte for byte with what the mirror writes."""
    elements, coeffs, n, species = case_inputs("map_quaternary")
    write_inputs(tmp, elements, coeffs, species)
    out = tmp / "maps"
    out.mkdir()
    run(["writemap", n, tmp / "species.txt", out], tmp)
    return {name: np.frombuffer((out / name).read_bytes(), np.uint8)
            for name in ("start.cfg", "lattice.txt", "element.txt", "map.txt")}


def make_pred(tmp: Path, name: str) -> dict:
    elements, coeffs, n, species = case_inputs(name)
    els = write_inputs(tmp, elements, coeffs, species)
    jumps, swaps = case_pairs(name, n, species)
    allp = np.concatenate([jumps, swaps])
    (tmp / "pairs.txt").write_text("\n".join(f"{a} {b}" for a, b in allp))
    res = parse_pred(run(["pred", n, tmp / "species.txt", tmp / "coeffs.json", els, tmp / "pairs.txt"], tmp),
                     elements, coeffs)
    res["jumps"], res["swaps"] = jumps, swaps
    return res


def make_baseline_kmc(tmp: Path, name: str) -> dict:
    """KineticMcFirstOmp on its mt19937_64 stream for the whole run: the selected event of every
    step (index among the 12 jumps in id order, and the target site), every BASELINE_SAMPLE-th
    step's barrier, energy change, total rate, time and energy, and the final state."""
    kind, elements, *_ , T, rseed, steps = BASELINE_CASES[name]
    _, coeffs, n, species = baseline_inputs(name)
    els = write_inputs(tmp, elements, coeffs, species)
    env = dict(os.environ, OMP_NUM_THREADS=str(min(12, os.cpu_count() or 1)))
    lines = run(["kmc", n, tmp / "species.txt", tmp / "coeffs.json", els, T, rseed, steps, 0], tmp, env)
    rows = np.asarray([[float(v) for v in ln.split()[1:]] for ln in lines if ln.startswith("step ")])
    assert rows.shape == (steps, 9)  # steps vacancy target selected Ea dE total time energy
    k = np.arange(0, steps, BASELINE_SAMPLE)
    return {"target": rows[:, 2].astype(np.int32), "selected": rows[:, 3].astype(np.uint8),
            "sample_steps": k, "sample": rows[k][:, 4:9], "final": rows[-1, 4:9],
            "final_vacancy": int(rows[-1, 2])}


def make_baseline_cmc(tmp: Path, name: str) -> dict:
    """CanonicalMcOmp with a batch of BASELINE_CMC_BATCH (OpenMP threads) on its mt19937_64 stream:
    the final lattice, the energy before every BASELINE_SAMPLE-th Metropolis test and at the end."""
    kind, elements, *_ , T, rseed, steps = BASELINE_CASES[name]
    _, coeffs, n, species = baseline_inputs(name)
    els = write_inputs(tmp, elements, coeffs, species)
    env = dict(os.environ, OMP_NUM_THREADS=str(BASELINE_CMC_BATCH))
    lines = run(["cmc", n, tmp / "species.txt", tmp / "coeffs.json", els, T, rseed, steps], tmp, env)
    alpha = S.alphabet(elements)
    log = []
    for ln in lines:
        f = ln.split()
        if f[0] == "log":
            log.append(float(f[3]))  # energy column of cmc_log.txt
        elif f[0] == "final_species":
            final = np.asarray([alpha.index(t) for t in f[1:]], np.int8)
        elif f[0] == "final_steps":
            fsteps = int(f[1])
        elif f[0] == "final_energy":
            fenergy = [float(v) for v in f[1:]]
    log = np.asarray(log)
    k = np.arange(0, log.size, BASELINE_SAMPLE)
    return {"final_species": final, "final_steps": fsteps, "final_energy": np.asarray(fenergy),
            "sample_steps": k, "sample_energy": log[k]}


def main():
    if len(sys.argv) > 1 and sys.argv[1] == "baseline":
        names = sys.argv[2:] or list(BASELINE_CASES)
        with tempfile.TemporaryDirectory() as td:
            for name in names:
                make = make_baseline_kmc if BASELINE_CASES[name][0] == "kmc" else make_baseline_cmc
                np.savez_compressed(HERE / f"{name}.npz", **make(Path(td), name))
                print(name, (HERE / f"{name}.npz").stat().st_size)
        return
    if len(sys.argv) > 1 and sys.argv[1] == "pred":
        with tempfile.TemporaryDirectory() as td:
            for name in ("pred_ternary", "pred_quaternary"):
                np.savez_compressed(HERE / f"{name}.npz", **make_pred(Path(td), name))
        return
    if len(sys.argv) > 1 and sys.argv[1] == "maps":
        with tempfile.TemporaryDirectory() as td:
            np.savez_compressed(HERE / "map_quaternary.npz", **make_map_files(Path(td)))
        return
    if len(sys.argv) > 1 and sys.argv[1] == "sitede":
        with tempfile.TemporaryDirectory() as td:
            np.savez_compressed(HERE / "site_de_quaternary.npz", **make_site_de(Path(td)))
        return
    if len(sys.argv) > 1 and sys.argv[1] == "clusters":
        with tempfile.TemporaryDirectory() as td:
            np.savez_compressed(HERE / "clusters_quaternary.npz", **make_clusters(Path(td)))
        return
    if not HARNESS.exists():
        subprocess.run([str(ROOT / "oracle" / "build_ref.sh")], check=True)
    env = dict(os.environ)
    with tempfile.TemporaryDirectory() as td:
        tmp = Path(td)
        np.savez_compressed(HERE / "geometry.npz", **make_geom(tmp))
        for name in ("pred_ternary", "pred_quaternary"):
            np.savez_compressed(HERE / f"{name}.npz", **make_pred(tmp, name))
        elements, coeffs, n, species = case_inputs("kmc_ternary")
        els = write_inputs(tmp, elements, coeffs, species)
        lines = run(["kmc", n, tmp / "species.txt", tmp / "coeffs.json", els, KMC_T, KMC_SEED, KMC_STEPS,
                     KMC_DETAIL], tmp)
        steps, events, e_abs = [], [], None
        for ln in lines:
            f = ln.split()
            if f[0] == "step":
                steps.append([float(v) for v in f[1:]])
            elif f[0] == "events":
                events.append(np.asarray(f[1:], float).reshape(12, 3))
            elif f[0] == "absolute_energy":
                e_abs = float(f[1])
        np.savez_compressed(HERE / "kmc_ternary.npz", steps=np.asarray(steps), events=np.asarray(events),
                            absolute_energy=e_abs)
        elements, coeffs, n, species = case_inputs("cmc_quaternary")
        els = write_inputs(tmp, elements, coeffs, species)
        env["OMP_NUM_THREADS"] = str(CMC_BATCH)
        lines = run(["cmc", n, tmp / "species.txt", tmp / "coeffs.json", els, CMC_T, CMC_SEED, CMC_STEPS], tmp, env)
        alpha = S.alphabet(elements)
        log, final = [], None
        for ln in lines:
            f = ln.split()
            if f[0] == "log":
                log.append([float(v) for v in f[1:]])
            elif f[0] == "final_species":
                final = np.asarray([alpha.index(t) for t in f[1:]], np.int8)
            elif f[0] == "final_steps":
                fsteps = int(f[1])
            elif f[0] == "final_energy":
                fenergy = [float(v) for v in f[1:]]
            elif f[0] == "absolute_energy0":
                e0 = float(f[1])
        np.savez_compressed(HERE / "cmc_quaternary.npz", log=np.asarray(log), final_species=final,
                            final_steps=fsteps, final_energy=np.asarray(fenergy), absolute_energy0=e0)
        rng_fx = {}
        for seed, rng_range in ((42, 4000), (7, 108000), (2024, 2048)):
            lines = run(["rng", seed, 64, rng_range], tmp)
            for ln in lines:
                f = ln.split()
                rng_fx[f"{f[0]}_{seed}_{rng_range}"] = np.asarray(f[1:], dtype=np.uint64 if f[0] != "real" else float)
        np.savez_compressed(HERE / "rng.npz", **rng_fx)
        np.savez_compressed(HERE / "clusters_quaternary.npz", **make_clusters(tmp))
        np.savez_compressed(HERE / "site_de_quaternary.npz", **make_site_de(tmp))
        np.savez_compressed(HERE / "map_quaternary.npz", **make_map_files(tmp))
    for p in sorted(HERE.glob("*.npz")):
        print(p.name, p.stat().st_size)


if __name__ == "__main__":
    main()
