"""Python front end of the C ABI (``include/lmc_gb300.h``).

Thin wrappers that marshal numpy arrays into the library; every computation
runs in ``liblmc_gb300.so`` (CUDA kernels for sm_103a). There is no CPU
fallback: a missing library or device raises.
"""
from __future__ import annotations

import ctypes as C
import os
import json
from pathlib import Path

import numpy as np

from . import _native as N
from ._native import check, ptr


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class Model:
    """Species alphabet and coefficient blocks (one reference coefficient file)."""

    def __init__(self, handle: int, elements):
        self._h = C.c_void_p(handle)
        self.elements = list(elements)
        nt, fm, f2 = C.c_int(), C.c_int(), C.c_int()
        check(N.lib.lmc_model_layout(self._h, C.byref(nt), C.byref(fm), C.byref(f2)))
        self.num_theta, self.f_mmm, self.f_mm2 = nt.value, fm.value, f2.value
        buf = C.create_string_buffer(128)
        check(N.lib.lmc_model_alphabet(self._h, buf, 128))
        self.alphabet = buf.value.decode().split()

    @classmethod
    def create(cls, elements) -> "Model":
        h = C.c_void_p()
        check(N.lib.lmc_model_create(N.cstrings(elements), len(elements), C.byref(h)))
        return cls(h.value, elements)

    @classmethod
    def from_json(cls, path, elements) -> "Model":
        h = C.c_void_p()
        check(N.lib.lmc_model_load_json(str(path).encode(), N.cstrings(elements), len(elements), C.byref(h)))
        return cls(h.value, elements)

    @classmethod
    def from_coefficients(cls, coeffs: dict, elements) -> "Model":
        """Builds a model from an in-memory coefficient dict (same layout as the JSON file)."""
        m = cls.create(elements)
        theta = _f64(coeffs["Base"]["theta"])
        check(N.lib.lmc_model_set_base_theta(m._h, ptr(theta, C.c_double), theta.size))
        for name, blk in coeffs.items():
            if name == "Base" or m.code(name) < 0:
                continue
            arr = {k: _f64(v) for k, v in blk.items() if isinstance(v, list)}
            if "U_mm2" in arr:
                p = N.QuarticParams(arr["U_mmm"].shape[0], arr["U_mm2"].shape[0],
                                    ptr(arr["mu_x_mmm"], C.c_double), ptr(arr["sigma_x_mmm"], C.c_double),
                                    ptr(arr["mu_x_mm2"], C.c_double), ptr(arr["sigma_x_mm2"], C.c_double),
                                    ptr(arr["U_mmm"], C.c_double), ptr(arr["U_mm2"], C.c_double),
                                    ptr(arr["theta_D"], C.c_double), ptr(arr["theta_Ks"], C.c_double),
                                    blk["mu_D"], blk["sigma_D"], blk["mu_Ks"], blk["sigma_Ks"])
                check(N.lib.lmc_model_set_quartic(m._h, name.encode(), C.byref(p)))
            if "theta_e0" in arr:
                p = N.E0Params(arr["U_mmm"].shape[0], ptr(arr["mu_x_mmm"], C.c_double),
                               ptr(arr["sigma_x_mmm"], C.c_double), ptr(arr["U_mmm"], C.c_double),
                               ptr(arr["theta_e0"], C.c_double), blk["mu_e0"], blk["sigma_e0"])
                check(N.lib.lmc_model_set_e0(m._h, name.encode(), C.byref(p)))
        return m

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            N.lib.lmc_model_destroy(h)
            self._h = None

    def code(self, name: str) -> int:
        return N.lib.lmc_model_species_code(self._h, name.encode())

    def orbit_sizes(self, which: int) -> np.ndarray:
        out = np.zeros(self.f_mmm if which == 0 else self.f_mm2, np.int32)
        check(N.lib.lmc_model_feature_orbit_sizes(self._h, which, ptr(out, C.c_int32)))
        return out

    def host_encode_pair(self, n: int, species: np.ndarray, first: int, second: int):
        sp = np.ascontiguousarray(species, dtype=np.int8)
        cs, ce = np.zeros(self.num_theta, np.int32), np.zeros(self.num_theta, np.int32)
        mm = np.zeros(self.f_mmm, np.int32)
        mf, mb = np.zeros(self.f_mm2, np.int32), np.zeros(self.f_mm2, np.int32)
        check(N.lib.lmc_host_encode_pair(self._h, n, ptr(sp, C.c_int8), first, second,
                                         *[ptr(x, C.c_int32) for x in (cs, ce, mm, mf, mb)]))
        return cs, ce, mm, mf, mb


class KmcTrace:
    """Per-step records of one replica (numpy structured view of lmc_kmc_step)."""

    DTYPE = np.dtype([("vacancy", np.int64), ("target", np.int64), ("selected", np.int32), ("slot", np.int32),
                      ("ea", np.float64), ("de", np.float64), ("total_rate", np.float64), ("time", np.float64),
                      ("energy", np.float64)])


class Context:
    """A model's tables and a set of lattices ("replicas") resident on one GPU."""

    def __init__(self, model: Model, device: int = 0):
        self.model = model
        self.device = device
        h = C.c_void_p()
        check(N.lib.lmc_ctx_create(model._h, device, C.byref(h)))
        self._h = h
        self.ns = np.zeros(0, np.int32)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            N.lib.lmc_ctx_destroy(h)
            self._h = None

    # lattices -------------------------------------------------------------
    def set_lattices(self, ns, species: np.ndarray) -> None:
        ns = np.ascontiguousarray(ns, dtype=np.int32)
        sp = np.ascontiguousarray(species, dtype=np.int8)
        check(N.lib.lmc_ctx_set_lattices(self._h, ns.size, ptr(ns, C.c_int32), ptr(sp, C.c_int8)))
        self.ns = ns

    def get_lattices(self, out: np.ndarray | None = None) -> np.ndarray:
        """Copies every replica's species back (into `out` when given, e.g. pinned memory)."""
        if out is None:
            out = np.empty(int(N.lib.lmc_ctx_total_sites(self._h)), np.int8)
        assert out.dtype == np.int8 and out.size == int(N.lib.lmc_ctx_total_sites(self._h))
        check(N.lib.lmc_ctx_get_lattices(self._h, ptr(out, C.c_int8)))
        return out

    def replica_offset(self, r: int) -> int:
        return int(N.lib.lmc_ctx_replica_offset(self._h, r))

    # predictors -----------------------------------------------------------
    def barrier_batch(self, pairs, replica: int = 0, kind: int = N.LMC_BARRIER_QUARTIC):
        p = np.ascontiguousarray(pairs, dtype=np.int64).reshape(-1, 2)
        m = p.shape[0]
        ea, de, x, ks = (np.zeros(m) for _ in range(4))
        check(N.lib.lmc_barrier_batch(self._h, replica, kind, ptr(p, C.c_int64), m, ptr(ea, C.c_double),
                                      ptr(de, C.c_double), ptr(x, C.c_double), ptr(ks, C.c_double)))
        return ea, de, x, ks

    def set_barrier_evaluation(self, evaluation: int) -> None:
        """LMC_EVAL_SPARSE (default) or LMC_EVAL_DENSE for barrier_batch and the surrogate's fallback."""
        check(N.lib.lmc_ctx_set_barrier_evaluation(self._h, evaluation))

    def set_surrogate_encoding(self, encoding: int) -> None:
        """LMC_FEATURES_ONEHOT (default) or LMC_FEATURES_SOLUTE for the surrogate's features,
        datasets and lattice-jump inference."""
        check(N.lib.lmc_surrogate_set_encoding(self._h, encoding))

    def encode_batch(self, pairs, replica: int = 0):
        p = np.ascontiguousarray(pairs, dtype=np.int64).reshape(-1, 2)
        m, mo = p.shape[0], self.model
        cs, ce = np.zeros((m, mo.num_theta), np.int32), np.zeros((m, mo.num_theta), np.int32)
        mm = np.zeros((m, mo.f_mmm), np.int32)
        mf, mb = np.zeros((m, mo.f_mm2), np.int32), np.zeros((m, mo.f_mm2), np.int32)
        check(N.lib.lmc_encode_batch(self._h, replica, ptr(p, C.c_int64), m,
                                     *[ptr(x, C.c_int32) for x in (cs, ce, mm, mf, mb)]))
        return cs, ce, mm, mf, mb

    def de_pairs(self, pairs, replica: int = 0) -> np.ndarray:
        p = np.ascontiguousarray(pairs, dtype=np.int64).reshape(-1, 2)
        de = np.zeros(p.shape[0])
        check(N.lib.lmc_de_pairs(self._h, replica, ptr(p, C.c_int64), p.shape[0], ptr(de, C.c_double)))
        return de

    def energy(self, replica: int = 0):
        e = C.c_double()
        counts = np.zeros(self.model.num_theta, np.int64)
        check(N.lib.lmc_energy(self._h, replica, C.byref(e), ptr(counts, C.c_int64)))
        return e.value, counts

    # kinetic MC -----------------------------------------------------------
    def kmc_init(self, temperatures, seed: int = 0, rng: int = N.LMC_RNG_PHILOX, kind: int = N.LMC_BARRIER_QUARTIC,
                 rate_corrector: bool = False, tt=None, warps_per_replica: int = 0, replicas_per_block: int = 0,
                 evaluation: int = N.LMC_EVAL_SPARSE, early_stop: bool = False, chain: bool = False,
                 rates: int = N.LMC_RATES_FP32):
        temps = np.ascontiguousarray(np.broadcast_to(np.asarray(temperatures, np.float64), (self.ns.size,)))
        self._tt = None
        opt = N.KmcOptions(rng, seed, kind, int(rate_corrector), None, None, 0, warps_per_replica,
                           replicas_per_block, evaluation, int(early_stop), int(chain), rates)
        if tt is not None:
            t0, t1 = _f64(tt[0]), _f64(tt[1])
            self._tt = (t0, t1)
            opt.tt_time, opt.tt_temp, opt.tt_len = ptr(t0, C.c_double), ptr(t1, C.c_double), t0.size
        check(N.lib.lmc_kmc_init(self._h, ptr(temps, C.c_double), C.byref(opt)))

    def kmc_run(self, steps: int, trace_replica: int | None = None, events: bool = False):
        trace = np.zeros(steps, KmcTrace.DTYPE) if trace_replica is not None else None
        ev = np.zeros((steps, 12, 3)) if (events and trace_replica is not None) else None
        check(N.lib.lmc_kmc_run(self._h, steps, -1 if trace_replica is None else trace_replica,
                                trace.ctypes.data_as(C.POINTER(N.KmcStep)) if trace is not None else None,
                                ptr(ev, C.c_double) if ev is not None else None))
        return trace, ev

    def kmc_state(self):
        r = self.ns.size
        vac, steps = np.zeros(r, np.int64), np.zeros(r, np.uint64)
        time, energy = np.zeros(r), np.zeros(r)
        check(N.lib.lmc_kmc_get_state(self._h, ptr(vac, C.c_int64), ptr(steps, C.c_uint64), ptr(time, C.c_double),
                                      ptr(energy, C.c_double)))
        return vac, steps, time, energy

    def kmc_launch_info(self) -> dict:
        """Block shape and occupancy the next kmc_run uses."""
        g, rpb, per_sm = C.c_int(), C.c_int(), C.c_int()
        smem = np.zeros(1, np.int64)
        check(N.lib.lmc_kmc_launch_info(self._h, C.byref(g), C.byref(rpb), C.byref(per_sm), ptr(smem, C.c_int64)))
        return {"warps_per_replica": g.value, "replicas_per_block": rpb.value, "blocks_per_sm": per_sm.value,
                "shared_bytes": int(smem[0])}

    def kmc_run_graph(self, steps_per_launch: int, launches: int = 1):
        """`launches` persistent launches of `steps_per_launch` steps as one CUDA graph (recorded once)."""
        check(N.lib.lmc_kmc_run_graph(self._h, steps_per_launch, launches))

    def kmc_autotune(self, probe_steps: int = 100, cache: str | os.PathLike | None = None) -> dict:
        """Times every KMC launch shape on a copy of the state and keeps the fastest (cached in `cache`)."""
        g, rpb, ev, hit = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        path = None if cache is None else os.fsencode(cache)
        check(N.lib.lmc_kmc_autotune(self._h, probe_steps, path, C.byref(g), C.byref(rpb), C.byref(ev),
                                     C.byref(hit)))
        return {"warps_per_replica": g.value, "replicas_per_block": rpb.value, "evaluation": ev.value,
                "from_cache": bool(hit.value)}

    # vacancy on every site (ExitTime's barrier queries) -------------------
    def site_jump_energetics(self, solvent: int, escape_temperature: float, sites=None, replica: int = 0,
                             kind: int = N.LMC_BARRIER_QUARTIC):
        """(ea [m,12], de [m,12], neighbours [m,12], mean barrier [m], exit time [m]) with the vacancy
        placed on each site (every site when `sites` is None)."""
        n = int(self.ns[replica])
        s = None if sites is None else np.ascontiguousarray(sites, dtype=np.int64)
        m = 4 * n ** 3 if s is None else s.size
        ea, de = np.zeros((m, 12)), np.zeros((m, 12))
        nb = np.zeros((m, 12), np.int64)
        avg, ext = np.zeros(m), np.zeros(m)
        check(N.lib.lmc_site_jump_energetics(self._h, replica, kind, solvent, escape_temperature,
                                             ptr(s, C.c_int64) if s is not None else None, m,
                                             ptr(ea, C.c_double), ptr(de, C.c_double), ptr(nb, C.c_int64),
                                             ptr(avg, C.c_double), ptr(ext, C.c_double)))
        return ea, de, nb, avg, ext

    # single-site energies (ExitTime's binding and profile energies) -----------
    def site_de(self, sites, to_codes, from_codes=None, fill_site: int = -1, fill_code: int = 0, replica: int = 0):
        """GetDeFromLatticeIdSite for each query: the species at sites[q] (from_codes[q], or the lattice's
        own) replaced by to_codes[q], the lattice read as if fill_site held fill_code."""
        s = np.ascontiguousarray(sites, np.int64)
        to = np.ascontiguousarray(np.broadcast_to(np.asarray(to_codes, np.int8), s.shape))
        fr = None if from_codes is None else np.ascontiguousarray(np.broadcast_to(np.asarray(from_codes, np.int8),
                                                                                  s.shape))
        de = np.zeros(s.size)
        check(N.lib.lmc_site_de_batch(self._h, replica, ptr(s, C.c_int64), ptr(fr, C.c_int8) if fr is not None else None,
                                      ptr(to, C.c_int8), s.size, fill_site, fill_code, ptr(de, C.c_double)))
        return de

    def exit_time_energies(self, solvent: int, chemical_potential, replica: int = 0):
        """ExitTime::GetBindingEnergy and GetProfileEnergy (ExitTime.cpp:401-511) per lattice site, with
        the lattice's vacancy (its lowest-id X) filled by the solvent: binding[e][i] = dE(i: e -> X) -
        (mu_X - mu_e) for every element e, profile[i] = dE(i: own -> X) + mu_own - mu_X, and at the
        vacancy the largest dE(e -> X) + mu_e - mu_X. Returns ({element name: array}, profile)."""
        alpha = self.model.alphabet
        x = alpha.index("X")
        nsites = 4 * int(self.ns[replica]) ** 3
        mu = np.ascontiguousarray(chemical_potential, np.float64)
        binding = np.zeros((len(alpha) - 1, nsites))
        profile = np.zeros(nsites)
        check(N.lib.lmc_exit_time_energies(self._h, replica, solvent, ptr(mu, C.c_double), ptr(binding, C.c_double),
                                           ptr(profile, C.c_double)))
        names = [alpha[c] for c in range(len(alpha)) if c != x]
        return {nm: binding[k] for k, nm in enumerate(names)}, profile

    def exit_time_clusters(self, clusters, solvent: int, escape_temperature: float, profile, replica: int = 0):
        """ExitTime's per-cluster quantities (ExitTime.cpp:72-128) for the given clusters (site-id
        arrays, e.g. from solute_clusters): Markov-chain escape time (BuildMarkovChain), neighbour-
        shell size, barriers [mean in/to/on/off, std in/to/on/off] (GetAverageBarriers) and the
        effective binding energy; `profile` is exit_time_energies' profile array."""
        k = len(clusters)
        off = np.concatenate([[0], np.cumsum([len(c) for c in clusters])]).astype(np.int64)
        mem = np.ascontiguousarray(np.concatenate(clusters) if k else np.zeros(1), np.int64)
        prof = np.ascontiguousarray(profile, np.float64)
        esc, eff = np.zeros(max(k, 1)), np.zeros(max(k, 1))
        nsz = np.zeros(max(k, 1), np.int64)
        bar = np.zeros((max(k, 1), 8))
        check(N.lib.lmc_exit_time_clusters(self._h, replica, solvent, escape_temperature, ptr(off, C.c_int64),
                                           ptr(mem, C.c_int64), k, ptr(prof, C.c_double), ptr(esc, C.c_double),
                                           ptr(nsz, C.c_int64), ptr(bar, C.c_double), ptr(eff, C.c_double)))
        return {"markov_escape_time": esc[:k], "neighbor_size": nsz[:k], "barriers": bar[:k],
                "effective_binding_energy": eff[:k]}

    # solute clusters ------------------------------------------------------
    def chemical_potential(self, solvent: int):
        """EnergyPredictor::GetChemicalPotential (EnergyPredictor.cpp:196-214): per species code, the
        energy of a 15^3-cell solvent lattice with one site of that species minus the pure
        solvent's (0 for the solvent), from the GPU census."""
        alpha = self.model.alphabet
        side = Context(self.model, device=self.device)
        lat = np.full(4 * 15 ** 3, solvent, np.int8)
        lats = []
        for code in range(len(alpha)):
            one = lat.copy()
            one[0] = code
            lats.append(one)
        side.set_lattices([15] * len(alpha), np.concatenate(lats))
        pure = side.energy(solvent)[0]
        return np.array([0.0 if c == solvent else side.energy(c)[0] - pure for c in range(len(alpha))])

    def solute_clusters(self, solvent: int, smallest: int = 1, solvent_bond: int = 12, chemical_potential=None,
                        replica: int = 0):
        """ansys::SoluteCluster's clusters of lattice `replica` (sorted site-id arrays, larger clusters
        first) and their formation energies (NaN without chemical potentials)."""
        k, nm = C.c_int64(), C.c_int64()
        mu = None if chemical_potential is None else np.ascontiguousarray(chemical_potential, np.float64)
        check(N.lib.lmc_solute_clusters(self._h, replica, solvent, smallest, solvent_bond,
                                        ptr(mu, C.c_double) if mu is not None else None, C.byref(k), C.byref(nm)))
        off = np.zeros(k.value + 1, np.int64)
        mem = np.zeros(max(nm.value, 1), np.int64)
        ef = np.zeros(max(k.value, 1))
        check(N.lib.lmc_solute_cluster_get(self._h, ptr(off, C.c_int64), ptr(mem, C.c_int64), ptr(ef, C.c_double)))
        return [mem[off[i]:off[i + 1]].copy() for i in range(k.value)], ef[:k.value].copy()

    # simulated annealing --------------------------------------------------
    SA_DTYPE = np.dtype([("site1", np.int64), ("site2", np.int64), ("accepted", np.int32), ("pad", np.int32),
                         ("de", np.float64), ("energy", np.float64), ("temperature", np.float64)])

    def sa_init(self, initial_temperature: float, maximum_steps: int, seed: int = 0, energy: float = 0.0,
                replica: int = 0):
        check(N.lib.lmc_sa_init(self._h, replica, seed, maximum_steps, initial_temperature, energy))

    def sa_run(self, steps: int, trace: bool = False):
        tr = np.zeros(steps, self.SA_DTYPE) if trace else None
        check(N.lib.lmc_sa_run(self._h, steps, tr.ctypes.data_as(C.c_void_p) if tr is not None else None))
        return tr

    def sa_state(self):
        """(steps, temperature, energy, lowest energy)."""
        st = C.c_uint64()
        t, e, lo = C.c_double(), C.c_double(), C.c_double()
        check(N.lib.lmc_sa_get_state(self._h, C.byref(st), C.byref(t), C.byref(e), C.byref(lo)))
        return st.value, t.value, e.value, lo.value

    # multi-vacancy kinetic MC ---------------------------------------------
    def kmc_multi_init(self, temperatures, seed: int = 0, kind: int = N.LMC_BARRIER_QUARTIC,
                       evaluation: int = N.LMC_EVAL_SPARSE, rates: int = N.LMC_RATES_FP64):
        """Tracks every vacancy of every lattice (slots in ascending site order); `rates` selects
        FP64 (the oracle's operations) or FP32 barriers and rates for the following runs."""
        temps = np.ascontiguousarray(np.broadcast_to(np.asarray(temperatures, np.float64), (self.ns.size,)))
        check(N.lib.lmc_kmc_multi_init(self._h, ptr(temps, C.c_double), seed, kind, evaluation))
        check(N.lib.lmc_kmc_multi_set_rates(self._h, rates))
        off = np.zeros(self.ns.size + 1, np.int32)
        check(N.lib.lmc_kmc_multi_slots(self._h, ptr(off, C.c_int32)))
        self._multi_off = off

    def kmc_multi_run(self, steps: int, trace_replica: int | None = None):
        trace = np.zeros(steps, KmcTrace.DTYPE) if trace_replica is not None else None
        check(N.lib.lmc_kmc_multi_run(self._h, steps, -1 if trace_replica is None else trace_replica,
                                      trace.ctypes.data_as(C.POINTER(N.KmcStep)) if trace is not None else None))
        return trace

    def kmc_multi_surrogate_run(self, model: "Surrogate", steps: int, threshold_ev: float = 0.010,
                                trace: bool = False):
        """Surrogate-assisted multi-vacancy KMC on the context's one lattice: (trace or None,
        plain barrier of each selected event or None, jumps that took the plain predictor)."""
        tr = np.zeros(steps, KmcTrace.DTYPE) if trace else None
        plain = np.zeros(steps) if trace else None
        nfb = np.zeros(1, np.uint64)
        check(N.lib.lmc_kmc_multi_surrogate_run(
            self._h, model._h, steps, threshold_ev,
            tr.ctypes.data_as(C.POINTER(N.KmcStep)) if tr is not None else None,
            ptr(plain, C.c_double) if plain is not None else None, ptr(nfb, C.c_uint64)))
        return tr, plain, int(nfb[0])

    def kmc_multi_state(self):
        """(slot offsets [R + 1], vacancy site per slot, steps, time, energy per lattice)."""
        off = self._multi_off
        r = self.ns.size
        vac = np.zeros(int(off[-1]), np.int64)
        steps, time, energy = np.zeros(r, np.uint64), np.zeros(r), np.zeros(r)
        check(N.lib.lmc_kmc_multi_get_state(self._h, ptr(vac, C.c_int64), ptr(steps, C.c_uint64),
                                            ptr(time, C.c_double), ptr(energy, C.c_double)))
        return off.copy(), vac, steps, time, energy

    def kmc_escaped(self) -> np.ndarray:
        """Per replica True when the early stop ended its trajectory."""
        out = np.zeros(self.ns.size, np.uint8)
        check(N.lib.lmc_kmc_get_escaped(self._h, ptr(out, C.c_uint8)))
        return out.astype(bool)

    def last_run_ms(self) -> float:
        ms = C.c_double()
        check(N.lib.lmc_last_run_ms(self._h, C.byref(ms)))
        return ms.value

    # canonical MC ---------------------------------------------------------
    def cmc_run(self, temperature: float, attempts: int, replica: int = 0, mode: int = N.LMC_CMC_THROUGHPUT,
                seed: int = 0, batch: int = 1, candidates: int = 0, energy: float = 0.0):
        opt = N.CmcOptions(mode, seed, batch, candidates, None)
        e = C.c_double(energy)
        done, acc = C.c_uint64(), C.c_uint64()
        check(N.lib.lmc_cmc_run(self._h, replica, temperature, attempts, C.byref(opt), C.byref(e), C.byref(done),
                                C.byref(acc)))
        return e.value, done.value, acc.value

    def cmc_rounds(self) -> int:
        """Rounds of the last throughput-mode cmc_run."""
        r = C.c_uint64()
        check(N.lib.lmc_cmc_rounds(self._h, C.byref(r)))
        return r.value

    def request_stop(self, value: int = 1) -> None:
        check(N.lib.lmc_request_stop(self._h, value))


class Surrogate:
    """BF16 MLP barrier surrogate (lmc_mlp_*): an ensemble trained on the plain
    predictor's barriers. Device arrays are torch tensors (features bfloat16
    [n][in_features], labels float32); torch only provides the device memory."""

    def __init__(self, in_features: int, hidden: int = 256, members: int = 4, seed: int = 0, device: int = 0):
        h = C.c_void_p()
        check(N.lib.lmc_mlp_create(device, in_features, hidden, members, seed, C.byref(h)))
        self._h = h
        self.in_features, self.hidden, self.members = in_features, hidden, members
        self.label_scale = (0.0, 1.0)
        n = np.zeros(1, np.int64)
        check(N.lib.lmc_mlp_layout(h, None, None, None, ptr(n, C.c_int64)))
        self.num_params = int(n[0])

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            N.lib.lmc_mlp_destroy(h)
            self._h = None

    def params(self) -> np.ndarray:
        out = np.zeros(self.num_params, np.float32)
        check(N.lib.lmc_mlp_get_params(self._h, ptr(out, C.c_float)))
        return out

    def set_params(self, p) -> None:
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == self.num_params
        check(N.lib.lmc_mlp_set_params(self._h, ptr(p, C.c_float)))

    def set_label_scale(self, mean: float, std: float) -> None:
        check(N.lib.lmc_mlp_set_label_scale(self._h, float(mean), float(std)))
        self.label_scale = (float(mean), float(std))

    def gradients(self, features_bf16_bits: np.ndarray, labels: np.ndarray):
        x = np.ascontiguousarray(features_bf16_bits, np.uint16)
        t = np.ascontiguousarray(labels, np.float32)
        g = np.zeros(self.num_params, np.float32)
        loss = np.zeros(self.members, np.float32)
        check(N.lib.lmc_mlp_gradients(self._h, x.ctypes.data_as(C.c_void_p), ptr(t, C.c_float), t.size,
                                      ptr(g, C.c_float), ptr(loss, C.c_float)))
        return g, loss

    def train(self, features, labels, batch: int = 4096, epochs: int = 10, lr: float = 2e-3, seed: int = 0):
        loss = np.zeros(self.members, np.float32)
        check(N.lib.lmc_mlp_train(self._h, C.c_void_p(features.data_ptr()), C.c_void_p(labels.data_ptr()),
                                  features.shape[0], batch, epochs, lr, seed, ptr(loss, C.c_float)))
        return loss

    def set_train_path(self, path: int) -> None:
        """0 the tcgen05 training GEMMs where the shapes allow (default), 1 mma.sync only."""
        check(N.lib.lmc_mlp_set_train_path(self._h, path))

    def set_inference_path(self, path: int) -> None:
        """0 automatic (tcgen05 when supported), 1 tcgen05, 2 mma.sync."""
        check(N.lib.lmc_mlp_set_inference_path(self._h, path))

    def predict(self, features):
        import torch
        n = features.shape[0]
        mean = torch.empty(n, dtype=torch.float32, device=features.device)
        spread = torch.empty(n, dtype=torch.float32, device=features.device)
        check(N.lib.lmc_mlp_predict(self._h, C.c_void_p(features.data_ptr()), n, C.c_void_p(mean.data_ptr()),
                                    C.c_void_p(spread.data_ptr())))
        return mean, spread


def surrogate_feature_count(ctx: "Context") -> int:
    mn, pad = C.c_int(), C.c_int()
    check(N.lib.lmc_surrogate_feature_count(ctx._h, C.byref(mn), C.byref(pad)))
    return pad.value


def surrogate_dataset(ctx: "Context", seed: int, count: int, solute_lo: float, solute_hi: float, in_features: int,
                      kind: int = N.LMC_BARRIER_QUARTIC, with_de: bool = False):
    """Seeded random environments with their features and plain-predictor barriers (torch tensors)."""
    import torch
    dev = f"cuda:{ctx.device}"
    x = torch.empty((count, in_features), dtype=torch.bfloat16, device=dev)
    ea = torch.empty(count, dtype=torch.float32, device=dev)
    ea64 = torch.empty(count, dtype=torch.float64, device=dev)
    de64 = torch.empty(count, dtype=torch.float64, device=dev) if with_de else None
    check(N.lib.lmc_surrogate_dataset(ctx._h, seed, count, solute_lo, solute_hi, kind, in_features,
                                      C.c_void_p(x.data_ptr()), C.c_void_p(ea.data_ptr()),
                                      C.c_void_p(ea64.data_ptr()),
                                      C.c_void_p(de64.data_ptr()) if de64 is not None else None))
    return x, ea, ea64, de64


def surrogate_predict(ctx: "Context", model: Surrogate, pairs_dev, replica: int = 0):
    """The network alone on lattice jumps: ensemble mean and spread, eV (torch tensors)."""
    import torch
    m = pairs_dev.shape[0]
    mean = torch.empty(m, dtype=torch.float32, device=pairs_dev.device)
    spread = torch.empty(m, dtype=torch.float32, device=pairs_dev.device)
    check(N.lib.lmc_surrogate_predict_device(ctx._h, model._h, replica, C.c_void_p(pairs_dev.data_ptr()), m,
                                             C.c_void_p(mean.data_ptr()), C.c_void_p(spread.data_ptr())))
    return mean, spread


def surrogate_features(ctx: "Context", pairs_dev, in_features: int, replica: int = 0):
    """Feature rows of lattice jumps in the context's encoding (bfloat16 torch tensor)."""
    import torch
    m = pairs_dev.shape[0]
    x = torch.empty((m, in_features), dtype=torch.bfloat16, device=pairs_dev.device)
    check(N.lib.lmc_surrogate_features(ctx._h, replica, C.c_void_p(pairs_dev.data_ptr()), m, in_features,
                                       C.c_void_p(x.data_ptr())))
    return x


def surrogate_barriers(ctx: "Context", model: Surrogate, pairs_dev, threshold_ev: float = 0.010, replica: int = 0,
                       kind: int = N.LMC_BARRIER_QUARTIC):
    """Ensemble barriers of lattice jumps with the plain predictor as fallback (torch tensors)."""
    import torch
    m = pairs_dev.shape[0]
    ea = torch.empty(m, dtype=torch.float64, device=pairs_dev.device)
    flag = torch.empty(m, dtype=torch.uint8, device=pairs_dev.device)
    nfb = C.c_int()
    check(N.lib.lmc_surrogate_barrier_batch_device(ctx._h, model._h, replica, kind, C.c_void_p(pairs_dev.data_ptr()),
                                                   m, threshold_ev, C.c_void_p(ea.data_ptr()),
                                                   C.c_void_p(flag.data_ptr()), C.byref(nfb)))
    return ea, flag, nfb.value


LATTICE_CONSTANT = 4.046  # Angstrom (lmc/cfg/include/Constants.hpp:6)


def site_relative_positions(n: int, sites) -> np.ndarray:
    """Relative positions (fractions of the cubic box) of lattice ids of an n^3-cell FCC supercell,
    in the id order of Config::ReassignLatticeVector."""
    ids = np.asarray(sites, np.int64)
    plane = 2 * n * n
    hx = ids // plane
    rem = ids - hx * plane
    hy = rem // n
    hz = 2 * (rem - hy * n) + ((hx + hy) & 1)
    return np.stack([hx, hy, hz], axis=-1) / (2.0 * n)


# Atomic masses as the reference tabulates them (lmc/cfg/include/Element.hpp:71-87).
ELEMENT_MASS = {"X": 0.00, "Al": 26.98, "Mg": 24.31, "Zn": 65.38, "Cu": 63.55, "Sn": 118.71}


def _periodic_mean(rel, weights):
    """Circular mean of relative positions per dimension (SoluteCluster::GetGeometryCenter /
    GetMassCenter, SoluteCluster.cpp:412-455): theta = 2 pi r, atan2 of the weighted mean sine
    and cosine, mapped to [0, 1)."""
    theta = rel * 2 * np.pi
    w = np.asarray(weights, np.float64)[:, None]
    cbar = (np.cos(theta) * w).sum(0) / w.sum()
    sbar = (np.sin(theta) * w).sum(0) / w.sum()
    return (np.arctan2(-sbar, -cbar) + np.pi) / (2 * np.pi)


def _wrapped(rel, centre_rel):
    d = rel - centre_rel
    return d - np.floor(d + 0.5)  # into [-0.5, 0.5), as the reference's while loops


def cluster_info(clusters, formation_energy, species, n: int, alphabet):
    """The per-cluster fields of SoluteCluster::GetClustersInfo (SoluteCluster.cpp:110-257) for the
    lists of Context.solute_clusters: cluster_atom_id_list (lattice ids), cluster_id (1-based),
    cluster_size (sites other than vacancies), elements_number (every element and X),
    effective_radius (of a sphere of the cluster's atomic volume), cluster_mass, cluster_energy
    (formation energy per non-vacancy site, 0 for a cluster of vacancies only), geometry_center
    and mass_center (periodic circular means, Angstrom), mass_gyration_tensor (Angstrom^2,
    GetMassGyrationTensor :457-492) with its eigenvalue measures mass_gyration_radius,
    asphericity, acylindricity and anisotropy (NaN for single-site clusters), and
    mass_inertia_tensor (GetMassInertiaTensor :494-528)."""
    sp = np.asarray(species)
    x = alphabet.index("X")
    box = n * LATTICE_CONSTANT
    mass_of = np.array([ELEMENT_MASS[a] for a in alphabet])
    out = []
    for k, (c, ef) in enumerate(zip(clusters, formation_energy)):
        codes = sp[c]
        counts = {name: int(np.count_nonzero(codes == code)) for code, name in enumerate(alphabet)}
        size = len(c)
        size_wo_x = size - counts["X"]
        volume = size * LATTICE_CONSTANT ** 3 / 4
        rel = site_relative_positions(n, c)
        masses = mass_of[codes]
        total_mass = float(masses.sum())
        centre = _periodic_mean(rel, np.ones(size))
        with np.errstate(invalid="ignore", divide="ignore"):
            mcentre = _periodic_mean(rel, masses)
            d = _wrapped(rel, mcentre)
            gyr = (d[:, :, None] * d[:, None, :] * masses[:, None, None]).sum(0) / total_mass * box * box
        ev = np.linalg.eigvalsh(gyr) if size > 1 and np.all(np.isfinite(gyr)) else np.full(3, np.nan)
        cart = d * box
        inertia = np.zeros((3, 3))
        for a in range(3):
            for b in range(3):
                inertia[a, b] = -(masses * cart[:, a] * cart[:, b]).sum()
            inertia[a, a] = (masses * ((cart ** 2).sum(1) - cart[:, a] ** 2)).sum()
        out.append({"cluster_atom_id_list": np.asarray(c, np.int64), "cluster_id": k + 1,
                    "cluster_size": size_wo_x, "elements_number": counts,
                    "effective_radius": (3 * volume / (4 * np.pi)) ** (1.0 / 3.0), "cluster_mass": total_mass,
                    "cluster_energy": 0.0 if size_wo_x == 0 else float(ef) / size_wo_x,
                    "geometry_center": centre * box, "mass_center": mcentre * box,
                    "mass_gyration_tensor": gyr, "mass_gyration_radius": float(np.sqrt(ev.sum())),
                    "asphericity": float(ev[2] - 0.5 * (ev[0] + ev[1])), "acylindricity": float(ev[1] - ev[0]),
                    "anisotropy": float(1.5 * (ev ** 2).sum() / ev.sum() ** 2 - 0.5),
                    "mass_inertia_tensor": inertia, "vacancies": int(np.count_nonzero(codes == x))})
    return out


def clusters_frame_info(clusters, formation_energy, species, n: int, alphabet):
    """SoluteCluster::GetClustersInfo's frame record (SoluteCluster.cpp:254-275): the per-cluster
    records of cluster_info under "clusters", and num_cluster, num_atom (summed cluster_size),
    num_<element> for every element of the element set (the alphabet without X) and
    cluster_size_list (strings, as the reference writes them)."""
    info = cluster_info(clusters, formation_energy, species, n, alphabet)
    frame = {"clusters": info, "num_cluster": len(info), "num_atom": int(sum(d["cluster_size"] for d in info)),
             "cluster_size_list": [str(d["cluster_size"]) for d in info]}
    for name in alphabet:
        if name != "X":
            frame["num_" + name] = int(sum(d["elements_number"][name] for d in info))
    return frame


def load_coefficients(path) -> dict:
    with open(path) as f:
        return json.load(f)


def write_coefficients(coeffs: dict, path) -> Path:
    path = Path(path)
    with open(path, "w") as f:
        json.dump(coeffs, f)
    return path
