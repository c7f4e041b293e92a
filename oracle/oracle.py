"""TEST ORACLE binding: ctypes wrapper of ``oracle/lmc_oracle.c``.

Test infrastructure only (tests/, ``__graft_entry__.smoke()`` and the CPU
baseline leg of bench.py use it as the checker). It is a plain-C restatement
of the reference's hot path, pinned against vectors produced by the
reference's own sources (tests/golden/). Nothing in the product imports it.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "lmc_oracle.c"
LIB = HERE / "_build" / "liblmc_oracle.so"


def build(force: bool = False) -> Path:
    """Compiles the restatement with -ffp-contract=off (identical rounding on x86-64 and aarch64)."""
    LIB.parent.mkdir(exist_ok=True)
    if LIB.exists() and not force and LIB.stat().st_mtime >= max(SRC.stat().st_mtime,
                                                               (HERE / "lmc_oracle.h").stat().st_mtime):
        return LIB
    tmp = LIB.with_suffix(".so.tmp")
    cmd = ["gcc", "-std=c11", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fopenmp", "-o", str(tmp), str(SRC),
           "-lm"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    tmp.replace(LIB)
    return LIB


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB))
        P, I64, I32P, I64P, DP, I8P = C.c_void_p, C.c_int64, C.POINTER(C.c_int32), C.POINTER(C.c_int64), \
            C.POINTER(C.c_double), C.POINTER(C.c_int8)
        sig = {
            "orc_lattice_create": (P, [C.c_int]),
            "orc_lattice_destroy": (None, [P]),
            "orc_lattice_num_sites": (I64, [P]),
            "orc_lattice_neighbors": (None, [P, I64, I64P]),
            "orc_lattice_position": (None, [P, I64, DP]),
            "orc_pair_lists": (C.c_int, [P, I64, I64, I64P, I64P, I64P]),
            "orc_site_list": (C.c_int, [P, I64, I64P]),
            "orc_distance_label": (C.c_int, [P, I64, I64]),
            "orc_mapping": (C.c_int, [P, C.c_int, I32P, C.c_int]),
            "orc_model_create": (P, [C.POINTER(C.c_char_p), C.c_int]),
            "orc_model_destroy": (None, [P]),
            "orc_model_num_species": (C.c_int, [P]),
            "orc_model_num_theta": (C.c_int, [P]),
            "orc_model_code": (C.c_int, [P, C.c_char_p]),
            "orc_model_cluster_index": (C.c_int, [P, C.c_int, C.c_int, C.POINTER(C.c_int)]),
            "orc_model_features": (C.c_int, [P, P, C.c_int]),
            "orc_model_set_theta": (None, [P, DP, C.c_int]),
            "orc_model_set_quartic": (None, [P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, DP, DP, DP, DP, DP, DP,
                                             DP, DP, C.c_double, C.c_double, C.c_double, C.c_double]),
            "orc_model_set_e0": (None, [P, C.c_int, C.c_int, C.c_int, DP, DP, DP, DP, C.c_double, C.c_double]),
            "orc_quartic": (C.c_int, [P, P, I8P, I64, I64, DP]),
            "orc_encode": (C.c_int, [P, P, I8P, I64, I64, I32P, I32P, I32P, I32P, I32P]),
            "orc_e0": (C.c_int, [P, P, I8P, I64, I64, DP]),
            "orc_pair_site_de": (C.c_int, [P, P, I8P, I64, I64, DP]),
            "orc_energy": (C.c_int, [P, P, I8P, I64P, DP]),
            "orc_kmc": (C.c_int, [P, P, I8P, C.c_double, C.c_uint64, I64, C.c_int, C.c_int, DP, DP]),
            "orc_kmc_ex": (C.c_int, [P, P, I8P, C.c_double, C.c_uint64, I64, C.c_int, C.c_int, DP, DP, DP, DP,
                                     C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int64)]),
            "orc_cmc": (I64, [P, P, I8P, C.c_double, C.c_uint64, I64, C.c_int, DP, DP, I64, I64P]),
            "orc_kmc_threads": (C.c_int, [P, P, I8P, C.c_double, C.c_uint64, I64, C.c_int, C.c_int, DP, DP]),
            "orc_model_set_vacancy_zero": (None, [P, C.c_int]),
            "orc_sa": (C.c_int, [P, P, I8P, C.c_double, C.c_uint64, C.c_uint64, I64, C.c_double, DP, DP]),
            "orc_kmc_chain": (C.c_int, [P, P, I8P, C.c_double, C.c_uint64, I64, C.c_int, C.c_int, C.c_uint32, DP]),
            "orc_philox4x32_10": (None, [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]),
            "orc_kmc_multi": (C.c_int, [P, P, I8P, C.c_double, C.c_uint64, C.c_uint32, C.c_uint64, I64, C.c_int,
                                        I64P, C.c_int, DP, DP, DP]),
            "orc_cluster_energy": (C.c_int, [P, P, I8P, C.c_int, C.c_int, I64P, I64, DP]),
            "orc_site_de": (C.c_int, [P, P, I8P, I64, C.c_int, DP]),
            "orc_solute_clusters": (I64, [P, I8P, C.c_int, I64, I64, I64P, I64P, I64]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


class OracleError(RuntimeError):
    pass


class Lattice:
    """GenerateFCC(n^3) + ReassignLatticeVector + neighbour lists, restated."""

    def __init__(self, n: int):
        self.n = n
        self.h = lib().orc_lattice_create(n)
        if not self.h:
            raise OracleError("n too small")
        self.num_sites = lib().orc_lattice_num_sites(self.h)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_lattice_destroy(self.h)
            self.h = None

    def neighbors(self, site: int) -> np.ndarray:
        out = np.zeros(42, np.int64)
        lib().orc_lattice_neighbors(self.h, site, _p(out, C.c_int64))
        return out

    def position(self, site: int) -> np.ndarray:
        out = np.zeros(3)
        lib().orc_lattice_position(self.h, site, _p(out, C.c_double))
        return out

    def pair_lists(self, a: int, b: int):
        st, mm, m2 = np.zeros(60, np.int64), np.zeros(58, np.int64), np.zeros(58, np.int64)
        if lib().orc_pair_lists(self.h, a, b, _p(st, C.c_int64), _p(mm, C.c_int64), _p(m2, C.c_int64)):
            raise OracleError("pair lists")
        return st, mm, m2

    def site_list(self, a: int) -> np.ndarray:
        out = np.zeros(43, np.int64)
        if lib().orc_site_list(self.h, a, _p(out, C.c_int64)):
            raise OracleError("site list")
        return out

    def mapping(self, which: int) -> np.ndarray:
        n = lib().orc_mapping(self.h, which, None, 0)
        out = np.zeros((n, 6), np.int32)
        lib().orc_mapping(self.h, which, _p(out, C.c_int32), n)
        return out

    def distance_label(self, a: int, b: int) -> int:
        return lib().orc_distance_label(self.h, a, b)


class Model:
    """Element alphabet + coefficients (a parsed coefficient JSON dict)."""

    def __init__(self, elements, coeffs: dict, lattice: Lattice):
        names = (C.c_char_p * len(elements))(*[e.encode() for e in elements])
        self.h = lib().orc_model_create(names, len(elements))
        self.num_theta = lib().orc_model_num_theta(self.h)
        self.num_species = lib().orc_model_num_species(self.h)
        f_mmm = lib().orc_model_features(self.h, lattice.h, 2)
        f_mm2 = lib().orc_model_features(self.h, lattice.h, 3)
        self.f_mmm, self.f_mm2 = f_mmm, f_mm2
        self._keep = []
        theta = np.ascontiguousarray(coeffs["Base"]["theta"], dtype=np.float64)
        if theta.size != self.num_theta:
            raise OracleError(f"theta length {theta.size} != {self.num_theta}")
        lib().orc_model_set_theta(self.h, _p(theta, C.c_double), theta.size)
        for name, blk in coeffs.items():
            if name == "Base":
                continue
            code = self.code(name)
            if code < 0:
                continue
            arr = {k: np.ascontiguousarray(v, dtype=np.float64) for k, v in blk.items()
                   if isinstance(v, (list, np.ndarray))}
            self._keep.append(arr)
            if "U_mm2" in arr:
                lib().orc_model_set_quartic(
                    self.h, code, arr["U_mmm"].shape[0], f_mmm, arr["U_mm2"].shape[0], f_mm2,
                    _p(arr["mu_x_mmm"], C.c_double), _p(arr["sigma_x_mmm"], C.c_double),
                    _p(arr["mu_x_mm2"], C.c_double), _p(arr["sigma_x_mm2"], C.c_double),
                    _p(arr["U_mmm"], C.c_double), _p(arr["U_mm2"], C.c_double),
                    _p(arr["theta_D"], C.c_double), _p(arr["theta_Ks"], C.c_double),
                    blk["mu_D"], blk["sigma_D"], blk["mu_Ks"], blk["sigma_Ks"])
            if "theta_e0" in arr:
                lib().orc_model_set_e0(self.h, code, arr["U_mmm"].shape[0], f_mmm, _p(arr["mu_x_mmm"], C.c_double),
                                       _p(arr["sigma_x_mmm"], C.c_double), _p(arr["U_mmm"], C.c_double),
                                       _p(arr["theta_e0"], C.c_double), blk["mu_e0"], blk["sigma_e0"])

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_model_destroy(self.h)
            self.h = None

    def code(self, name: str) -> int:
        return lib().orc_model_code(self.h, name.encode())

    def set_vacancy_zero(self, on: bool = True):
        """Multi-vacancy extension: clusters with two vacancies count nothing, a
        vacancy in a one-hot environment is a zero vector (the reference throws)."""
        lib().orc_model_set_vacancy_zero(self.h, int(on))


def _sp(species: np.ndarray):
    assert species.dtype == np.int8 and species.flags.c_contiguous
    return _p(species, C.c_int8)


def quartic(model: Model, lat: Lattice, species, a: int, b: int) -> np.ndarray:
    out = np.zeros(4)
    rc = lib().orc_quartic(model.h, lat.h, _sp(species), a, b, _p(out, C.c_double))
    if rc:
        raise OracleError(f"orc_quartic rc={rc}")
    return out


def e0(model: Model, lat: Lattice, species, a: int, b: int) -> np.ndarray:
    out = np.zeros(3)
    rc = lib().orc_e0(model.h, lat.h, _sp(species), a, b, _p(out, C.c_double))
    if rc:
        raise OracleError(f"orc_e0 rc={rc}")
    return out


def encode(model: Model, lat: Lattice, species, a: int, b: int):
    cs, ce = np.zeros(model.num_theta, np.int32), np.zeros(model.num_theta, np.int32)
    mm = np.zeros(model.f_mmm, np.int32)
    mf, mb = np.zeros(model.f_mm2, np.int32), np.zeros(model.f_mm2, np.int32)
    rc = lib().orc_encode(model.h, lat.h, _sp(species), a, b, *[_p(x, C.c_int32) for x in (cs, ce, mm, mf, mb)])
    if rc:
        raise OracleError(f"orc_encode rc={rc}")
    return cs, ce, mm, mf, mb


def pair_site_de(model: Model, lat: Lattice, species, a: int, b: int) -> float:
    out = C.c_double()
    rc = lib().orc_pair_site_de(model.h, lat.h, _sp(species), a, b, C.byref(out))
    if rc:
        raise OracleError(f"orc_pair_site_de rc={rc}")
    return out.value


def energy(model: Model, lat: Lattice, species):
    counts = np.zeros(model.num_theta, np.int64)
    e = C.c_double()
    rc = lib().orc_energy(model.h, lat.h, _sp(species), _p(counts, C.c_int64), C.byref(e))
    if rc:
        raise OracleError(f"orc_energy rc={rc}")
    return e.value, counts


def site_de(model: Model, lat: Lattice, species, site: int, new_code: int) -> float:
    """GetDeFromLatticeIdSite: dE of changing the species at `site` to new_code."""
    out = C.c_double()
    rc = lib().orc_site_de(model.h, lat.h, _sp(species), site, new_code, C.byref(out))
    if rc:
        raise OracleError(f"orc_site_de rc={rc}")
    return out.value


def cluster_energy(model: Model, lat: Lattice, species, solvent: int, sites, mode: int = 0) -> float:
    """GetEnergyOfCluster over the sites and their 1-3NN shells; mode 0 the lattice's species, 1 the
    solvent except at the sites, 2 the solvent everywhere."""
    ids = np.ascontiguousarray(sites, np.int64)
    e = C.c_double()
    rc = lib().orc_cluster_energy(model.h, lat.h, _sp(species), solvent, mode, _p(ids, C.c_int64), ids.size,
                                  C.byref(e))
    if rc:
        raise OracleError(f"orc_cluster_energy rc={rc}")
    return e.value


def solute_clusters(lat: Lattice, species, solvent: int, smallest: int, bond: int):
    """SoluteCluster::FindAtomListOfClusters restated: a list of sorted id arrays, larger clusters first."""
    sp = np.ascontiguousarray(species, np.int8)
    offsets = np.zeros(sp.size + 1, np.int64)
    members = np.zeros(13 * sp.size, np.int64)
    k = lib().orc_solute_clusters(lat.h, _sp(sp), solvent, smallest, bond, _p(offsets, C.c_int64),
                                  _p(members, C.c_int64), members.size)
    if k < 0:
        raise OracleError(f"orc_solute_clusters rc={k}")
    return [members[offsets[i]:offsets[i + 1]].copy() for i in range(k)]


def kmc(model: Model, lat: Lattice, species, T: float, seed: int, steps: int, kind: int = 0, memo: bool = False,
        events: bool = False, tt=None, rate_corrector: bool = False, early_stop: bool = False):
    """Runs the restated KineticMcFirstOmp loop; species is modified in place.
    tt = (times, temperatures) enables the time-temperature schedule. With
    early_stop the trace is cut at the escape step (IsEscaped)."""
    trace = np.zeros((steps, 8))
    ev = np.zeros((steps, 12, 3)) if events else None
    t0 = t1 = None
    done = C.c_int64()
    if tt is not None:
        t0 = np.ascontiguousarray(tt[0], dtype=np.float64)
        t1 = np.ascontiguousarray(tt[1], dtype=np.float64)
    rc = lib().orc_kmc_ex(model.h, lat.h, _sp(species), T, seed, steps, kind, int(memo), _p(trace, C.c_double),
                          _p(ev, C.c_double) if events else None, _p(t0, C.c_double) if t0 is not None else None,
                          _p(t1, C.c_double) if t1 is not None else None, 0 if t0 is None else t0.size,
                          int(rate_corrector), int(early_stop), C.byref(done))
    if rc:
        raise OracleError(f"orc_kmc rc={rc}")
    if early_stop:
        trace = trace[:done.value]
        ev = ev[:done.value] if ev is not None else None
    return trace, ev


def kmc_threads(model: Model, lat: Lattice, species, T: float, seed: int, steps: int, threads: int, kind: int = 0):
    """KineticMcFirstOmp with the 12 barriers of each step on `threads` OpenMP threads (the
    reference's parallel loop), id tables built first; species is modified in place. Returns
    (trace [steps][8] as kmc's, wall seconds of the step loop)."""
    trace = np.zeros((steps, 8))
    loop_s = C.c_double()
    rc = lib().orc_kmc_threads(model.h, lat.h, _sp(species), T, seed, steps, kind, threads, _p(trace, C.c_double),
                               C.byref(loop_s))
    if rc != 0:
        raise OracleError("orc_kmc_threads failed")
    return trace, loop_s.value


def cmc(model: Model, lat: Lattice, species, T: float, seed: int, attempts: int, batch: int, energy0: float = 0.0,
        trace: bool = False):
    """Runs the restated CanonicalMcOmp loop; species is modified in place."""
    e = C.c_double(energy0)
    acc = C.c_int64()
    cap = attempts + 4 * batch
    tr = np.zeros(cap) if trace else None
    done = lib().orc_cmc(model.h, lat.h, _sp(species), T, seed, attempts, batch, C.byref(e),
                         _p(tr, C.c_double) if trace else None, cap, C.byref(acc))
    if done < 0:
        raise OracleError("orc_cmc failed")
    return done, e.value, acc.value, (tr[:done] if trace else None)


def philox4x32_10(counter, key) -> np.ndarray:
    """One Philox4x32-10 block (Salmon et al., SC'11)."""
    c = np.ascontiguousarray(counter, dtype=np.uint32)
    k = np.ascontiguousarray(key, dtype=np.uint32)
    out = np.zeros(4, np.uint32)
    lib().orc_philox4x32_10(_p(c, C.c_uint32), _p(k, C.c_uint32), _p(out, C.c_uint32))
    return out


def kmc_multi(model: Model, lat: Lattice, species, T: float, seed: int, vacancies, steps: int, replica: int = 0,
              step0: int = 0, kind: int = 0, time: float = 0.0, energy: float = 0.0):
    """Multi-vacancy KMC as the GPU kernel defines it (every slot re-evaluated
    every step). species and the returned slot positions are updated in place.
    Returns (trace [steps x 9]: slot, vacancy, target, selected, Ea, dE, total,
    time, energy), vacancies, time, energy)."""
    vac = np.ascontiguousarray(vacancies, dtype=np.int64).copy()
    trace = np.zeros((steps, 9))
    t, e = C.c_double(time), C.c_double(energy)
    rc = lib().orc_kmc_multi(model.h, lat.h, _sp(species), T, seed, replica, step0, steps, kind,
                             _p(vac, C.c_int64), vac.size, C.byref(t), C.byref(e), _p(trace, C.c_double))
    if rc:
        raise OracleError(f"orc_kmc_multi rc={rc}")
    return trace, vac, t.value, e.value


def kmc_chain(model: Model, lat: Lattice, species, T: float, seed: int, steps: int, kind: int = 0, rng: int = 0,
              replica: int = 0):
    """Restated KineticMcChainOmpi loop (species modified in place); trace rows as kmc()."""
    trace = np.zeros((steps, 8))
    rc = lib().orc_kmc_chain(model.h, lat.h, _sp(species), T, seed, steps, kind, rng, replica, _p(trace, C.c_double))
    if rc:
        raise OracleError(f"orc_kmc_chain rc={rc}")
    return trace


def sa(model: Model, lat: Lattice, species, T0: float, seed: int, maximum_steps: int, steps: int,
       energy0: float = 0.0):
    """Restated SimulatedAnnealing loop (species modified in place). Returns (trace [steps x 7]:
    site1, site2, accepted, dE, energy and temperature before the step, lowest energy; state:
    steps, temperature, energy, lowest)."""
    trace = np.zeros((steps, 7))
    state = np.zeros(4)
    rc = lib().orc_sa(model.h, lat.h, _sp(species), T0, seed, maximum_steps, steps, energy0,
                      _p(trace, C.c_double), _p(state, C.c_double))
    if rc:
        raise OracleError(f"orc_sa rc={rc}")
    return trace, state


class Mt19937_64:
    """std::mt19937_64 with libstdc++'s uniform_int_distribution (restated in the oracle)."""

    class _State(C.Structure):
        _fields_ = [("mt", C.c_uint64 * 312), ("idx", C.c_int)]

    def __init__(self, seed: int):
        self.s = self._State()
        L = lib()
        for name, res, args in (("orc_mt_seed", None, [C.c_void_p, C.c_uint64]),
                                ("orc_mt_below", C.c_uint64, [C.c_void_p, C.c_uint64])):
            getattr(L, name).restype = res
            getattr(L, name).argtypes = args
        L.orc_mt_seed(C.byref(self.s), seed)

    def below(self, n: int) -> int:
        """uniform_int_distribution<size_t>(0, n - 1)."""
        return int(lib().orc_mt_below(C.byref(self.s), n))
