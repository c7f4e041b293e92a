"""Benchmark of the lattice-MC hot path on GB300.

One JSON line on rank 0. The headline workload is the batched-replica KMC
configuration: 4096 independent trajectories, cubic supercells with edges
n ~ U{8..24} (2048 to 55296 sites), one vacancy each, Al/Mg/Zn 0.96/0.02/0.02,
T ~ U(350, 550) K, 1e4 steps each in one persistent graph-captured launch. One
bench step is that launch: every replica advances by 1e4 KMC steps (later steps
continue the same trajectories). `value` is KMC
events/s over all replicas with the lattices resident in HBM; `e2e` is the same
metric through the public C ABI with host buffers (lattice upload, KMC init,
run, lattice and state download inside the timed region). The CMC pair-swap
configuration (30^3 FCC, 108000 sites, Al/Mg/Zn/Cu 0.94/0.02/0.02/0.02,
T = 500 K) is reported alongside under "cmc".

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

--impl reference times the CPU restatement of the reference's path (the
oracle, compiled C, OpenMP) on the host cores for the same configuration.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "KMC events/s and CMC swaps/s at 1 GB300; surrogate vs plain at <=5 meV barrier MAE"
KMC_STEPS_PER_BENCH_STEP = 10_000
BYTES_PER_EVENT = 225       # algorithmic HBM bytes per KMC event
# DRAM bytes (read + write) of one full-size kmc_kernel launch (4096 replicas x 1e4 steps), one ncu
# capture with the L2 flushed before the launch; the command and figures are in the kmc_kernel
# summary under profiles/. The lattices and tables stay in L2, hence far below the algorithmic bytes.
KMC_TRAFFIC_PER_LAUNCH = 102_407_936 + 70_376_704
# What bounds kmc_kernel instead of HBM (the ncu --set full capture summarised under profiles/): the
# lattices sit in L2 and the per-event work is a dependent chain of gathers and integer table sums.
KMC_LIMITER = ("issue and latency: issue active 61 % of active cycles, FP64 pipe 20 %, ALU 44 %, 27 of 64 warps "
               "resident (one warp per replica, 72 registers), DRAM 6 % of the algorithmic bytes")
BYTES_PER_ATTEMPT = 100     # algorithmic HBM bytes per CMC attempt
L2_BYTES = 129 * 1024 * 1024


def rank_seed(rank: int) -> int:
    """Each rank simulates its own replicas (replicas only: no exchange between ranks)."""
    return 1234 + rank


def max_over_ranks(value: float, device) -> float:
    """The slowest rank's time (whole-job throughput = all ranks' units / this)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return value
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons while the timed region runs."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_min_mhz": min(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d["hbm_gbs"], "measured"
    return 6800.0, "fallback"


# ---------------------------------------------------------------------------
# workloads
# ---------------------------------------------------------------------------
def kmc_config(args, world: int, sites_total: int) -> dict:
    """The batched-KMC workload's description; both arms print the same dict."""
    return {"workload": f"batched replica KMC: {args.replicas} FCC supercells n~U{{8..24}}, 1 vacancy, "
                        f"Al/Mg/Zn .96/.02/.02, T~U(350,550) K, {args.kmc_steps_per_launch} KMC steps per "
                        "replica per step",
            "replicas": int(args.replicas), "sites_total": int(sites_total),
            "kmc_steps_per_step": args.kmc_steps_per_launch, "seed": rank_seed(0),
            "l2": "flushed between timed steps (2x L2 write)", "parallelism": f"replicas x{world}"}


def kmc_inputs(seed: int, replicas: int):
    from latticemontecarlo_gb300 import synthetic as S
    cfg = S.KMC_BATCHED
    coeffs = S.make_coefficients(cfg["elements"], seed)
    ns, species, temps = S.batched_replicas(seed, replicas, cfg["n_range"], cfg["fractions"], cfg["T_range"],
                                            cfg["elements"])
    return cfg, coeffs, ns, species, temps


def cmc_inputs(seed: int):
    from latticemontecarlo_gb300 import synthetic as S
    cfg = S.CMC_SINGLE
    coeffs = S.make_coefficients(cfg["elements"], seed)
    sp = S.make_lattice(cfg["n"], cfg["fractions"], 0, seed, cfg["elements"])
    return cfg, coeffs, sp


def run_ours(args, rank, world, local):
    import torch  # device memory for the L2 flush and distributed plumbing only

    from latticemontecarlo_gb300 import Context, Model
    from latticemontecarlo_gb300 import _native as N

    device = local
    torch.cuda.set_device(device)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    seed = rank_seed(rank)
    cfg, coeffs, ns, species, temps = kmc_inputs(seed, args.replicas)
    model = Model.from_coefficients(coeffs, list(cfg["elements"]))
    ctx = Context(model, device=device)
    ctx.set_lattices(ns, species)
    ctx.kmc_init(temps, seed=seed, rng=N.LMC_RNG_PHILOX)
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device=f"cuda:{device}")

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    # launch shape from the project's autotuner (timed on a copy of the state, cached per GPU and size histogram)
    tune = ctx.kmc_autotune(probe_steps=args.tune_probe_steps, cache=args.tune_cache or None)
    shape = {k: tune[k] for k in ("warps_per_replica", "replicas_per_block", "evaluation")}
    events_per_step = int(ns.size) * args.kmc_steps_per_launch
    for _ in range(args.warmup):
        ctx.kmc_run_graph(args.kmc_steps_per_launch)
    kernel_ms = []
    barrier()
    with ClockSampler(device) as clocks:
        for _ in range(args.steps):
            flush.fill_(1.0)  # evict L2 between timed steps (outside the kernel timing)
            torch.cuda.synchronize()
            ctx.kmc_run_graph(args.kmc_steps_per_launch)  # one recorded graph: the persistent launch
            kernel_ms.append(ctx.last_run_ms())
    barrier()
    t_ms = max_over_ranks(float(np.sum(kernel_ms)), f"cuda:{device}")
    total_events = events_per_step * args.steps * world
    value = total_events / (t_ms / 1e3)
    # end to end through the C ABI with host buffers (pinned host memory)
    pinned = torch.empty(species.size, dtype=torch.int8, pin_memory=True).numpy()
    pinned[:] = species
    species_out = torch.empty(species.size, dtype=torch.int8, pin_memory=True).numpy()
    e2e_steps = max(1, min(args.steps, 3))
    h2d = species.nbytes + ns.nbytes + temps.nbytes
    d2h = species.nbytes + ns.size * (8 + 8 + 8 + 8)

    def e2e_step():
        ctx.set_lattices(ns, pinned)
        ctx.kmc_init(temps, seed=seed, rng=N.LMC_RNG_PHILOX, **shape)
        ctx.kmc_run_graph(args.kmc_steps_per_launch)
        return ctx.get_lattices(species_out), ctx.kmc_state()

    e2e_step()  # one untimed pass, as the device-timed steps have warm-up launches
    barrier()
    with ClockSampler(device) as e2e_clocks:
        t0 = time.perf_counter()
        e2e_kernel_ms = []
        for _ in range(e2e_steps):
            out, (vac, st, tm, en) = e2e_step()
            e2e_kernel_ms.append(ctx.last_run_ms())
        barrier()
        e2e_s = time.perf_counter() - t0
    assert out.size == species.size and np.all(st == args.kmc_steps_per_launch)
    e2e_value = events_per_step * e2e_steps * world / e2e_s
    peak, peak_kind = peaks()
    launch_ms = t_ms / args.steps
    achieved = BYTES_PER_EVENT * events_per_step / (launch_ms / 1e3) / 1e9
    traffic = args.traffic
    if traffic is None and args.replicas == 4096 and args.kmc_steps_per_launch == KMC_STEPS_PER_BENCH_STEP \
            and KMC_TRAFFIC_PER_LAUNCH is not None:
        traffic = KMC_TRAFFIC_PER_LAUNCH
    result = {
        "metric": METRIC,
        "value": value,
        "unit": "events/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": t_ms / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "int64 fixed-point cluster sums, f32 barriers and rates, f64 rate sum and clock",
        "data": "synthetic (seeded lattices and coefficients; the reference ships none)",
        "config": kmc_config(args, world, int(species.size)),
        "rng": "philox4x32-10",
        "launch": dict(shape, autotuned=True, from_cache=tune["from_cache"], cuda_graph=True),
        "e2e": {"value": e2e_value, "unit": "events/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h),
                "step": "upload the 4096 lattices (pinned host buffer), kmc_init, one graph launch of the "
                        "1e4-step persistent kernel from the initial state, download lattices and state",
                "kernel_ms_per_step": float(np.mean(e2e_kernel_ms)), "clocks": e2e_clocks.summary()},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "peak_source": peak_kind,
                     "kernel": "kmc_kernel", "bytes_per_event": BYTES_PER_EVENT,
                     "limiter": KMC_LIMITER},
        "gpu_launches": args.steps,
        "clocks": clocks.summary(),
    }
    if args.cmc_steps > 0:
        result["cmc"] = run_cmc(args, device, flush, barrier)
    if args.surrogate_samples > 0:
        result["surrogate"] = run_surrogate(args, device)
    if not args.no_large:
        result["large_lattice"] = run_large(args, device)
    if args.chain_steps > 0:
        result["chain_kmc"] = run_chain(args, device, seed)
    if args.single_steps > 0:
        result["single_trajectory"] = run_single(args, device)
    if args.sa_steps > 0:
        result["simulated_annealing"] = run_sa(args, device)
    if not args.no_large:
        result["exit_time_barriers"] = run_site_jumps(args, device)
        result["solute_clusters"] = run_solute_clusters(args, device)
    return result, (cfg, coeffs, ns, species, temps)


def run_cmc(args, device, flush, barrier):
    import torch

    from latticemontecarlo_gb300 import Context, Model
    from latticemontecarlo_gb300 import _native as N

    cfg, coeffs, sp = cmc_inputs(4321)
    model = Model.from_coefficients(coeffs, list(cfg["elements"]))
    ctx = Context(model, device=device)
    ctx.set_lattices([cfg["n"]], sp)
    attempts = args.cmc_sweeps_per_step * sp.size
    e = 0.0
    for _ in range(2):
        e, _, _ = ctx.cmc_run(cfg["T"], attempts, mode=N.LMC_CMC_THROUGHPUT, seed=1, energy=e)
    ms, done_total, rounds = [], 0, 0
    barrier()
    for k in range(args.cmc_steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        e, done, acc = ctx.cmc_run(cfg["T"], attempts, mode=N.LMC_CMC_THROUGHPUT, seed=2 + k, energy=e)
        ms.append(ctx.last_run_ms())
        done_total += done
        rounds += ctx.cmc_rounds()
    barrier()
    value = done_total / (np.sum(ms) / 1e3)
    peak, _ = peaks()
    out = {"value": value, "unit": "swaps/s (Metropolis attempts)",
           "workload": "CMC 30^3 FCC (108000 sites), Al/Mg/Zn/Cu .94/.02/.02/.02, T=500 K, "
                       f"{args.cmc_sweeps_per_step} sweeps per step, non-overlapping pairs per round",
           "steps": args.cmc_steps, "ms_per_step": float(np.mean(ms)),
           "rounds": {"count": rounds, "survivors_per_round": done_total / max(1, rounds),
                      "us_per_round": float(np.sum(ms)) * 1e3 / max(1, rounds)},
           "roofline": {"bound": "hbm", "achieved": BYTES_PER_ATTEMPT * value / 1e9, "peak": peak,
                        "unit": "GB/s", "frac": BYTES_PER_ATTEMPT * value / 1e9 / peak}}
    if args.cmc_ref_attempts > 0:
        # CanonicalMcOmp's own order on its mt19937_64 stream (what the host executable runs), with the
        # batch the CPU baseline's OpenMP threads give
        batch = min(256, os.cpu_count() or 1)
        e, _, _ = ctx.cmc_run(cfg["T"], 20_000, mode=N.LMC_CMC_REFERENCE_BATCH, seed=1, batch=batch, energy=e)
        e, done, _ = ctx.cmc_run(cfg["T"], args.cmc_ref_attempts, mode=N.LMC_CMC_REFERENCE_BATCH, seed=2,
                                 batch=batch, energy=e)
        ms_ref = ctx.last_run_ms()
        out["reference_batch"] = {"value": done / (ms_ref / 1e3), "unit": "swaps/s (Metropolis attempts)",
                                  "batch": batch, "attempts": int(done), "ms": ms_ref,
                                  "workload": "the same lattice, CanonicalMcOmp batch order and RNG stream"}
    return out


def run_single(args, device):
    """One trajectory (KineticMcFirstOmp's own case: n = 10, 1 vacancy, Al/Mg/Zn .96/.02/.02, 400 K)
    on the reference's mt19937_64 stream: the latency of a step, one replica on the GPU (12 warps,
    one per jump), beside the oracle's restatement of the reference loop on one host core and with the
    12 barriers of a step on 12 host threads (the reference's OpenMP loop)."""
    from latticemontecarlo_gb300 import Context, Model
    from latticemontecarlo_gb300 import _native as N
    from latticemontecarlo_gb300 import synthetic as S
    from oracle import oracle as O

    cfg = S.KMC_SINGLE
    coeffs = S.make_coefficients(cfg["elements"], 11)
    sp = S.make_lattice(cfg["n"], cfg["fractions"], 1, 11, cfg["elements"])
    ctx = Context(Model.from_coefficients(coeffs, list(cfg["elements"])), device=device)
    ctx.set_lattices([cfg["n"]], sp)
    ctx.kmc_init([cfg["T"]], seed=5, rng=N.LMC_RNG_MT19937_64)
    ctx.kmc_run(1000)
    ctx.kmc_run(args.single_steps)
    gpu = args.single_steps / (ctx.last_run_ms() / 1e3)
    out = {"workload": f"n={cfg['n']} (4000 sites), 1 vacancy, T={cfg['T']} K, mt19937_64 stream, "
                       f"{args.single_steps} steps", "value": gpu, "unit": "events/s",
           "launch": ctx.kmc_launch_info()}
    if not args.no_cpu_baseline:
        O.build()
        lat = O.Lattice(cfg["n"])
        m = O.Model(cfg["elements"], coeffs, lat)
        steps = max(1000, args.single_steps // 20)
        t0 = time.perf_counter()
        O.kmc(m, lat, sp.copy(), cfg["T"], 5, steps, memo=True)
        w = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": steps / w, "unit": "events/s", "cores": 1, "kind": "port",
                               "sample": f"{steps} steps of the same trajectory, oracle C restatement with "
                                         f"barrier memo, {w:.1f} s"}
        # the reference's OpenMP loop over the 12 jumps of a step, on 12 host threads (more cannot help)
        threads = min(12, os.cpu_count() or 1)
        _, loop_s = O.kmc_threads(m, lat, sp.copy(), cfg["T"], 5, steps, threads)
        out["cpu_baseline_threads"] = {
            "value": steps / loop_s, "unit": "events/s", "cores": threads, "kind": "port",
            "sample": f"{steps} steps of the same trajectory, oracle C restatement with the 12 barriers of a "
                      f"step on {threads} OpenMP threads (id tables built first, not timed), {loop_s:.1f} s"}
    return out


def run_site_jumps(args, device):
    """ExitTime's barrier queries: the vacancy placed on each of the 2^20 sites of an n = 64 lattice
    (Al/Mg/Zn/Cu .93/.03/.03/.01, one vacancy), 12 barriers per site, mean barrier and exit time;
    beside the oracle's predictor on one host core for a sample of sites."""
    from latticemontecarlo_gb300 import Context, Model
    from latticemontecarlo_gb300 import synthetic as S
    from oracle import oracle as O

    L = S.LARGE
    el = L["elements"]
    coeffs = S.make_coefficients(el, 65)
    sp = S.make_lattice(L["n"], L["fractions"], 1, 65, el)
    alpha = S.alphabet(el)
    ctx = Context(Model.from_coefficients(coeffs, list(el)), device=device)
    ctx.set_lattices([L["n"]], sp)
    ctx.site_jump_energetics(alpha.index("Al"), 600.0, sites=np.arange(1024))
    t0 = time.perf_counter()
    ea, _, _, _, ext = ctx.site_jump_energetics(alpha.index("Al"), 600.0)
    wall = time.perf_counter() - t0
    ms = ctx.last_run_ms()
    out = {"workload": f"vacancy on each of the {sp.size} sites of an n=64 lattice, 12 barriers each",
           "value": sp.size / (ms / 1e3), "unit": "sites/s", "kernel_ms": ms,
           "wall_ms_with_host_copies": wall * 1e3, "barriers_per_s": 12 * sp.size / (ms / 1e3)}
    if not args.no_cpu_baseline:
        O.build()
        lat = O.Lattice(L["n"])
        m = O.Model(el, coeffs, lat)
        x, al = alpha.index("X"), alpha.index("Al")
        vac = int(np.flatnonzero(sp == x)[0])
        mod = sp.copy()
        mod[vac] = al
        sites = np.random.default_rng(0).choice(sp.size, 40, replace=False)
        t0 = time.perf_counter()
        for s in sites:
            keep = mod[s]
            mod[s] = x
            for t in lat.neighbors(int(s))[:12]:
                O.quartic(m, lat, mod, int(s), int(t))
            mod[s] = keep
        w = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": len(sites) / w, "unit": "sites/s", "cores": 1, "kind": "port",
                               "sample": f"{len(sites)} sites x 12 barriers, oracle C restatement, {w:.1f} s"}
    # GetBindingEnergy + GetProfileEnergy: a site substitution dE per (site, element) and per site
    al = alpha.index("Al")
    mu = ctx.chemical_potential(al)
    ctx.exit_time_energies(al, mu)
    t0 = time.perf_counter()
    ctx.exit_time_energies(al, mu)
    w_be = time.perf_counter() - t0
    queries = sp.size * (len(alpha) - 1) + sp.size
    out["binding_profile_energies"] = {"value": queries / w_be, "unit": "site substitutions/s",
                                       "wall_ms": w_be * 1e3, "queries": queries,
                                       "kernel_ms": ctx.last_run_ms(),
                                       "note": "wall clock of one lmc_exit_time_energies call (vacancy scan, "
                                               "one warp per site, every element in one pass, results copied "
                                               "back); kernel_ms is the kernel alone"}
    if not args.no_cpu_baseline:
        x = alpha.index("X")
        this = sp.copy()
        this[this == x] = al
        sites = np.random.default_rng(1).choice(sp.size, 2000, replace=False)
        t0 = time.perf_counter()
        for s in sites:
            O.site_de(m, lat, this, int(s), x)
        w = time.perf_counter() - t0
        out["binding_profile_energies"]["cpu_baseline"] = {
            "value": len(sites) / w, "unit": "site substitutions/s", "cores": 1, "kind": "port",
            "sample": f"{len(sites)} site substitutions, oracle C restatement, {w:.2f} s"}
    return out


def run_solute_clusters(args, device):
    """SoluteCluster's analysis of one frame: the solute clusters of the n = 64 lattice (Al/Mg/Zn/Cu
    .93/.03/.03/.01, 64 vacancies; clusters of at least 2 sites, solvent shells above 3 bonds) with
    their formation energies; beside the oracle's restatement on one host core."""
    from latticemontecarlo_gb300 import Context, Model
    from latticemontecarlo_gb300 import synthetic as S
    from oracle import oracle as O

    L = S.LARGE
    el = L["elements"]
    coeffs = S.make_coefficients(el, 31)
    sp = S.make_lattice(L["n"], L["fractions"], L["vacancies"], 31, el)
    solvent = S.alphabet(el).index("Al")
    ctx = Context(Model.from_coefficients(coeffs, list(el)), device=device)
    ctx.set_lattices([L["n"]], sp)
    mu = ctx.chemical_potential(solvent)
    ctx.solute_clusters(solvent, 2, 3, chemical_potential=mu)  # warm-up
    t0 = time.perf_counter()
    clusters, ef = ctx.solute_clusters(solvent, 2, 3, chemical_potential=mu)
    wall = time.perf_counter() - t0
    sizes = np.array([len(c) for c in clusters])
    out = {"workload": f"solute clusters of an n=64 lattice ({sp.size} sites, 64 vacancies), clusters >= 2 sites, "
                       "solvent shells above 3 bonds, formation energies",
           "value": sp.size / wall, "unit": "sites/s", "wall_ms": wall * 1e3, "clusters": len(clusters),
           "largest": int(sizes.max()) if sizes.size else 0, "members": int(sizes.sum())}
    if not args.no_cpu_baseline:
        O.build()
        lat = O.Lattice(L["n"])
        m = O.Model(el, coeffs, lat)
        m.set_vacancy_zero(True)
        t0 = time.perf_counter()
        ref = O.solute_clusters(lat, sp, solvent, 2, 3)
        for c in ref:
            O.cluster_energy(m, lat, sp, solvent, c, 1) - O.cluster_energy(m, lat, sp, solvent, c, 2)
        w = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": sp.size / w, "unit": "sites/s", "cores": 1, "kind": "port",
                               "sample": f"the same frame, oracle C restatement, {w:.1f} s"}
    return out


def run_sa(args, device):
    """Simulated annealing (SimulatedAnnealing's sequential trial moves, one warp) on a 20^3 box with
    200 Mg and 200 Zn solutes in Al, beside the oracle's restatement on one host core."""
    from latticemontecarlo_gb300 import Context, Model
    from latticemontecarlo_gb300 import synthetic as S
    from oracle import oracle as O

    el = ("Al", "Mg", "Zn")
    coeffs = S.make_coefficients(el, 20)
    n = 20
    sp = S.make_lattice(n, {"Al": 0.9875, "Mg": 0.00625, "Zn": 0.00625}, 0, 20, el)
    ctx = Context(Model.from_coefficients(coeffs, list(el)), device=device)
    ctx.set_lattices([n], sp)
    ctx.sa_init(600.0, args.sa_steps, seed=3)
    ctx.sa_run(1000)
    ctx.sa_run(args.sa_steps)
    v = args.sa_steps / (ctx.last_run_ms() / 1e3)
    out = {"workload": f"n={n} ({sp.size} sites), Al/Mg/Zn .9875/.00625/.00625, T0=600 K, {args.sa_steps} trial "
                       "moves (one sequential chain)", "value": v, "unit": "trial moves/s"}
    if not args.no_cpu_baseline:
        O.build()
        lat = O.Lattice(n)
        m = O.Model(el, coeffs, lat)
        steps = max(2000, args.sa_steps // 10)
        t0 = time.perf_counter()
        O.sa(m, lat, sp.copy(), 600.0, 3, args.sa_steps, steps)
        w = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": steps / w, "unit": "trial moves/s", "cores": 1, "kind": "port",
                               "sample": f"the first {steps} moves of the same run, oracle C restatement, {w:.1f} s"}
    return out


def run_chain(args, device, seed: int):
    """Second-order chain KMC (KineticMcChainOmpi) on the batched-replica workload: per step the
    12 x 12 jump barriers after each first jump, one block of 12 warps per replica."""
    from latticemontecarlo_gb300 import Context, Model
    from latticemontecarlo_gb300 import _native as N

    cfg, coeffs, ns, species, temps = kmc_inputs(seed, args.replicas)
    ctx = Context(Model.from_coefficients(coeffs, list(cfg["elements"])), device=device)
    ctx.set_lattices(ns, species)
    ctx.kmc_init(temps, seed=seed, rng=N.LMC_RNG_PHILOX, chain=True)
    ctx.kmc_run(10)  # warm-up
    ctx.kmc_run(args.chain_steps)
    ms = ctx.last_run_ms()
    ev = int(ns.size) * args.chain_steps
    v = ev / (ms / 1e3)
    peak, _ = peaks()
    return {"workload": f"{int(ns.size)} replicas (the batched-KMC lattices), {args.chain_steps} chain steps each",
            "value": v, "unit": "events/s", "ms": ms, "jump_evaluations_per_s": 144 * v,
            "roofline": {"bound": "latency", "achieved": BYTES_PER_EVENT * v / 1e9, "peak": peak, "unit": "GB/s",
                         "frac": BYTES_PER_EVENT * v / 1e9 / peak}}


def run_large(args, device):
    """Large-lattice workload: one n = 64 FCC supercell (2^20 sites), Al/Mg/Zn/Cu
    .93/.03/.03/.01 with 64 vacancies, T = 500 K: one EnergyPredictor census,
    CMC sweeps (throughput mode), and multi-vacancy KMC events (every vacancy
    tracked, one event per step among 64 x 12)."""
    from latticemontecarlo_gb300 import Context, Model
    from latticemontecarlo_gb300 import _native as N
    from latticemontecarlo_gb300 import synthetic as S

    L = S.LARGE
    el = L["elements"]
    coeffs = S.make_coefficients(el, 64)
    sp = S.make_lattice(L["n"], L["fractions"], L["vacancies"], 64, el)
    ctx = Context(Model.from_coefficients(coeffs, list(el)), device=device)
    ctx.set_lattices([L["n"]], sp)
    T = 500.0
    ctx.energy()
    reps = 20
    t0 = time.perf_counter()
    for _ in range(reps):
        e0, _ = ctx.energy()
    census_ms = (time.perf_counter() - t0) / reps * 1e3
    peak, _ = peaks()
    out = {"workload": "n=64 FCC (1048576 sites), Al/Mg/Zn/Cu .93/.03/.03/.01, 64 vacancies, T=500 K",
           "census": {"ms": census_ms, "sites_per_s": sp.size / (census_ms / 1e3),
                      "note": "wall clock per lmc_energy call (launch, census, energy, counts copied back)"}}
    if args.large_cmc_sweeps > 0:
        attempts = args.large_cmc_sweeps * sp.size
        ctx.cmc_run(T, sp.size, mode=N.LMC_CMC_THROUGHPUT, seed=1, energy=e0)  # warm-up sweep
        ctx.set_lattices([L["n"]], sp)
        e, done, acc = ctx.cmc_run(T, attempts, mode=N.LMC_CMC_THROUGHPUT, seed=2, energy=e0)
        ms = ctx.last_run_ms()
        v = done / (ms / 1e3)
        rounds = ctx.cmc_rounds()
        out["cmc"] = {"sweeps": args.large_cmc_sweeps, "attempts": int(done), "accepted": int(acc), "ms": ms,
                      "value": v, "unit": "swaps/s (Metropolis attempts)",
                      "rounds": {"count": rounds, "survivors_per_round": done / max(1, rounds),
                                 "us_per_round": ms * 1e3 / max(1, rounds)},
                      "roofline": {"bound": "hbm", "achieved": BYTES_PER_ATTEMPT * v / 1e9, "peak": peak,
                                   "unit": "GB/s", "frac": BYTES_PER_ATTEMPT * v / 1e9 / peak}}
        ctx.set_lattices([L["n"]], sp)
    if args.large_kmc_events > 0:
        # production arithmetic (FP32 barriers and rates, FP64 rate sums and clock), then the
        # FP64 mode (the oracle's operations) on a shorter run of the same lattice
        ctx.kmc_multi_init([T], seed=3, rates=N.LMC_RATES_FP32)
        ctx.kmc_multi_run(2000)  # warm-up
        ctx.kmc_multi_run(args.large_kmc_events)
        ms = ctx.last_run_ms()
        off, vac, steps, tm, en = ctx.kmc_multi_state()
        v = args.large_kmc_events / (ms / 1e3)
        ctx.set_lattices([L["n"]], sp)
        ctx.kmc_multi_init([T], seed=3, rates=N.LMC_RATES_FP64)
        ctx.kmc_multi_run(2000)
        ev64 = min(args.large_kmc_events, 200_000)
        ctx.kmc_multi_run(ev64)
        v64 = ev64 / (ctx.last_run_ms() / 1e3)
        out["kmc_multi_vacancy"] = {
            "events": args.large_kmc_events, "ms": ms, "value": v, "unit": "events/s",
            "simulated_time_s": float(tm[0]), "vacancies": int(off[-1]),
            "rates": "FP32 barriers and rates, FP64 rate sums and clock, exact energy sums",
            "fp64_rates": {"events": ev64, "value": v64, "unit": "events/s"},
            "launch": "one block of 8 warps (a single lattice is one sequential trajectory)",
            "roofline": {"bound": "latency", "achieved": BYTES_PER_EVENT * v / 1e9, "peak": peak, "unit": "GB/s",
                         "frac": BYTES_PER_EVENT * v / 1e9 / peak}}
        ctx.set_lattices([L["n"]], sp)
        if args.surrogate_samples > 0:
            out["kmc_multi_vacancy_surrogate"] = run_large_surrogate(args, ctx, sp, T)
    if not args.no_cpu_baseline:
        # the oracle's EnergyPredictor census (serial, as the reference's) and CanonicalMcOmp on all
        # host cores, on the same lattice; clusters holding two vacancies count nothing, as on the GPU
        from oracle import oracle as O
        O.build()
        lat = O.Lattice(L["n"])
        m = O.Model(el, coeffs, lat)
        m.set_vacancy_zero(True)
        t0 = time.perf_counter()
        O.energy(m, lat, sp)
        w = time.perf_counter() - t0
        out["census"]["cpu_baseline"] = {"value": sp.size / w, "unit": "sites/s", "cores": 1, "kind": "port",
                                         "sample": f"one census of the same lattice, oracle C restatement, {w:.2f} s"}
        if args.large_cmc_sweeps > 0:
            threads = os.cpu_count() or 1
            os.environ["OMP_NUM_THREADS"] = str(threads)
            attempts = min(args.cpu_cmc_attempts, sp.size)
            filled = sp.copy()  # the restated CanonicalMcOmp takes lattices without vacancies
            filled[filled == S.alphabet(el).index("X")] = S.alphabet(el).index("Al")
            t0 = time.perf_counter()
            done, _, _, _ = O.cmc(m, lat, filled, T, 1, attempts, threads)
            w = time.perf_counter() - t0
            out["cmc"]["cpu_baseline"] = {"value": done / w, "unit": "swaps/s (Metropolis attempts)", "cores": threads,
                                          "kind": "port",
                                          "sample": f"{done} attempts of CanonicalMcOmp (batch = {threads}) on the "
                                                    f"lattice with its vacancies filled by Al, oracle C restatement, "
                                                    f"{w:.1f} s"}
    return out


def run_large_surrogate(args, ctx, sp, T):
    """Surrogate-assisted multi-vacancy KMC on the large lattice (the same lattice, seed and
    temperature as the plain run): the compact ensemble (2 members of 128-128 GELU over the
    solute-channel features, 192 for the four species) trained on barriers of random environments
    with 0-15 % solutes; per step the fused jump kernel evaluates the jumps of the vacancies whose
    neighbourhood changed, the plain predictor takes the jumps where the ensemble spread exceeds
    10 meV, and the energy change of each selected jump is the plain predictor's."""
    import torch

    from latticemontecarlo_gb300 import api
    from latticemontecarlo_gb300 import _native as N
    from latticemontecarlo_gb300 import synthetic as S

    L = S.LARGE
    ctx.set_lattices([L["n"]], sp)
    ctx.set_surrogate_encoding(N.LMC_FEATURES_SOLUTE)
    nin = api.surrogate_feature_count(ctx)
    x, ea, _, _ = api.surrogate_dataset(ctx, 1, args.surrogate_samples, 0.0, 0.15, nin)
    net = api.Surrogate(nin, 128, 2, seed=1, device=ctx.device)
    net.set_label_scale(float(ea.mean()), float(ea.std()))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    net.train(x, ea, batch=2048, epochs=args.surrogate_epochs_compact, lr=3e-3, seed=2)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    del x, ea
    ctx.kmc_multi_init([T], seed=3)
    # a traced run: the barriers used for the selected events against the plain predictor's
    traced = args.large_surrogate_traced
    tr, plain_ea, nfb_traced = ctx.kmc_multi_surrogate_run(net, traced, 0.010, trace=True)
    err = np.abs(tr["ea"] - plain_ea)
    events = args.large_kmc_events
    _, fb = ctx.kmc_multi_surrogate_run(net, events, 0.010)[1:]
    ms = ctx.last_run_ms()
    off, vac, steps, tm, en = ctx.kmc_multi_state()
    ctx.set_surrogate_encoding(N.LMC_FEATURES_ONEHOT)
    return {"events": events, "ms": ms, "value": events / (ms / 1e3), "unit": "events/s",
            "simulated_time_s": float(tm[0]), "network": f"2 x {nin}-128-128-1, fused jump kernel",
            "train_s": t_train, "fallback_jumps_per_event": fb / events,
            "selected_event_barrier_mae_mev": 1e3 * float(err.mean()),
            "selected_event_barrier_max_err_mev": 1e3 * float(err.max()), "traced_events": traced,
            "launch": "per step: the fused network kernel on the re-evaluated slots' jumps, then a one-block "
                      "step kernel; chunks of 256 steps captured in a CUDA graph"}


def _vacancy_grid_lattice(n: int, spacing: int, fractions, seed: int, elements):
    """n^3 FCC cells, vacancies on every site with all half-lattice coordinates
    divisible by `spacing` (far enough apart that no jump environment holds a
    second vacancy), the rest drawn i.i.d. from `fractions`; returns species and
    the 12 jumps of every vacancy as (vacancy, neighbour) pairs."""
    from latticemontecarlo_gb300 import synthetic as S
    alpha = S.alphabet(elements)
    rng = np.random.default_rng(seed)
    names = list(fractions)
    probs = np.array([fractions[k] for k in names], float)
    probs /= probs.sum()
    nsites = 4 * n ** 3
    sp = np.array([alpha.index(k) for k in names], np.int8)[rng.choice(len(names), size=nsites, p=probs)]
    m = 2 * n
    g = np.arange(0, m, spacing)
    hx, hy, hz = (a.ravel() for a in np.meshgrid(g, g, g, indexing="ij"))
    vac = hx * 2 * n * n + hy * n + hz // 2
    sp[vac] = alpha.index("X")
    dirs = np.array([(a, b, 0) for a in (-1, 1) for b in (-1, 1)] + [(a, 0, b) for a in (-1, 1) for b in (-1, 1)] +
                    [(0, a, b) for a in (-1, 1) for b in (-1, 1)])
    pairs = []
    for d in dirs:
        x, y, z = (hx + d[0]) % m, (hy + d[1]) % m, (hz + d[2]) % m
        pairs.append(np.stack([vac, x * 2 * n * n + y * n + z // 2], 1))
    # a vacancy's 12 jumps together, as KineticMcFirstOmp::BuildEventList asks for them
    return sp, np.stack(pairs, 1).reshape(-1, 2).astype(np.int64)


def run_surrogate(args, device):
    """Learned barrier surrogate against the plain barrier predictor on the same lattice jumps: the
    12 jumps of every vacancy of a vacancy grid in a 192^3-cell lattice (1.33e6 jumps), in a dilute
    alloy (Al .96) and a solute-rich one (Al .70), each with ensembles trained on 2e6 barriers of
    random environments of that composition range:

    * the workload's ensemble: 4 members of 256-256 GELU over the one-hot features (the streaming
      tcgen05 inference kernel on feature rows written by a separate gather kernel);
    * a compact ensemble: 2 members of 128-128 GELU over the solute-channel features, run by the
      fused jump kernel (the lattice gather in its producer warps, both members' weights resident
      in shared memory, tcgen05 with the hidden layer in tensor memory).

    The plain path is timed with its sparse evaluation (a vacancy's jumps from the solvent-relative
    sums) and with the dense cluster sums; the surrogate path includes the fallback (the plain dense
    predictor on the jumps whose ensemble spread exceeds 10 meV). Accuracy: MAE against the plain
    predictor's FP64 barriers on the same jumps (fallback merged) and on held-out random
    environments (network alone)."""
    import ctypes as C

    import torch

    from latticemontecarlo_gb300 import api
    from latticemontecarlo_gb300 import _native as N
    from latticemontecarlo_gb300 import synthetic as S

    el = ("Al", "Mg", "Zn")
    coeffs = S.make_coefficients(el, 1234)
    model = api.Model.from_coefficients(coeffs, list(el))
    ctx = api.Context(model, device=device)
    n, spacing = args.surrogate_n, 8
    # composition of the lattice, solute-fraction range of the training environments
    cases = {"dilute": ({"Al": 0.96, "Mg": 0.02, "Zn": 0.02}, (0.0, 0.1)),
             "solute_rich": ({"Al": 0.70, "Mg": 0.15, "Zn": 0.15}, (0.2, 0.4))}
    peak = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())["bf16_tflops"] \
        if (ROOT / "MEASURED_PEAKS.json").exists() else 1900.0
    # networks: (encoding, hidden, members, epochs, lr, batch)
    nets_spec = {"ensemble_4x256_onehot": (N.LMC_FEATURES_ONEHOT, 256, 4, args.surrogate_epochs, 2e-3, 4096),
                 "ensemble_2x128_fused": (N.LMC_FEATURES_SOLUTE, 128, 2, args.surrogate_epochs_compact, 3e-3, 2048)}

    def timed(fn, reps):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        t = time.perf_counter()
        for _ in range(reps):
            fn()
        torch.cuda.synchronize()
        return (time.perf_counter() - t) / reps

    out_cases, roofline = {}, {}
    for case, (frac, (lo, hi)) in cases.items():
        sp, pairs = _vacancy_grid_lattice(n, spacing, frac, 77, el)
        ctx.set_lattices([n], sp)
        pd = torch.from_numpy(pairs).to(f"cuda:{device}")
        m = pd.shape[0]
        ea_plain = torch.empty(m, dtype=torch.float64, device=pd.device)
        de_plain = torch.empty(m, dtype=torch.float64, device=pd.device)

        def plain():
            N.check(N.lib.lmc_barrier_batch_device(ctx._h, 0, 0, C.c_void_p(pd.data_ptr()), m,
                                                   C.c_void_p(ea_plain.data_ptr()), C.c_void_p(de_plain.data_ptr())))
            N.check(N.lib.lmc_ctx_synchronize(ctx._h))

        ctx.set_barrier_evaluation(N.LMC_EVAL_DENSE)
        t_dense = timed(plain, 10)
        ctx.set_barrier_evaluation(N.LMC_EVAL_SPARSE)
        t_sparse = timed(plain, 10)
        t_plain = min(t_dense, t_sparse)
        rec = {"training_solute_range": [lo, hi], "jumps": m, "plain_sparse_barriers_per_s": m / t_sparse,
               "plain_dense_barriers_per_s": m / t_dense}
        for name, (enc, hidden, members, epochs, lr, batch) in nets_spec.items():
            ctx.set_surrogate_encoding(enc)
            nin = api.surrogate_feature_count(ctx)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            x, ea, _, _ = api.surrogate_dataset(ctx, 1, args.surrogate_samples, lo, hi, nin)
            torch.cuda.synchronize()
            t_data = time.perf_counter() - t0
            xt, _, eat, _ = api.surrogate_dataset(ctx, 99, 1 << 17, lo, hi, nin)
            net = api.Surrogate(nin, hidden, members, seed=1, device=device)
            net.set_label_scale(float(ea.mean()), float(ea.std()))
            t0 = time.perf_counter()
            net.train(x, ea, batch=batch, epochs=epochs, lr=lr, seed=2)
            torch.cuda.synchronize()
            t_train = time.perf_counter() - t0
            flop_fwd = 2 * members * (nin * hidden + hidden * hidden + hidden)
            r = {"features": nin, "hidden": hidden, "members": members, "epochs": epochs, "dataset_s": t_data,
                 "train_s": t_train,
                 "train_tflops": 3 * flop_fwd * args.surrogate_samples * epochs / t_train / 1e12,
                 "mae_mev_heldout_network_only": 1e3 * float((net.predict(xt)[0].double() - eat).abs().mean())}
            del x, ea, xt, eat
            res = {}

            def network():
                res["n"] = api.surrogate_predict(ctx, net, pd)

            t_net = timed(network, 10)

            def surrogate():
                res["s"] = api.surrogate_barriers(ctx, net, pd, 0.010)

            t_sur = timed(surrogate, 10)
            ea_sur, flag, nfb = res["s"]
            r.update({"network_barriers_per_s": m / t_net, "network_tflops": flop_fwd * m / t_net / 1e12,
                      "surrogate_barriers_per_s": m / t_sur, "over_best_plain": t_plain / t_sur,
                      "over_dense_plain": t_dense / t_sur, "fallback_fraction": nfb / m,
                      "mae_mev_with_fallback": 1e3 * float((ea_sur - ea_plain).abs().mean())})
            rec[name] = r
            if case == "solute_rich":
                kernel = ("mlp_fused_jump_kernel (tcgen05, features gathered in the kernel)"
                          if enc == N.LMC_FEATURES_SOLUTE else
                          "surrogate_features_thread_kernel + mlp_tc_infer_kernel (tcgen05)")
                tf = flop_fwd * m / t_net / 1e12
                roofline[name] = {"bound": "tensor", "kernel": kernel, "achieved": tf, "peak": peak,
                                  "unit": "TFLOP/s", "frac": tf / peak,
                                  "flop_per_jump": flop_fwd, "timing": "wall clock per synchronised call"}
            del net
        ctx.set_surrogate_encoding(N.LMC_FEATURES_ONEHOT)
        out_cases[case] = rec
    cands = [(c, k) for c in out_cases for k in nets_spec
             if out_cases[c][k]["mae_mev_with_fallback"] <= 5.0]
    best = max(cands, key=lambda ck: out_cases[ck[0]][ck[1]]["over_best_plain"]) if cands else None
    return {
        "workload": f"the 12 jumps of each of {out_cases['dilute']['jumps'] // 12} vacancies in a {n}^3-cell FCC "
                    f"lattice per composition; ensembles trained on {args.surrogate_samples:.0e} barriers of that "
                    "composition range; fallback to the plain predictor where the ensemble spread exceeds 10 meV",
        "compositions": out_cases,
        "best": ({"composition": best[0], "ensemble": best[1], **out_cases[best[0]][best[1]]} if best else None),
        "timing": "wall clock over 10 device-synchronised calls",
        "roofline": roofline,
    }


# ---------------------------------------------------------------------------
# CPU restatement of the reference path (baseline)
# ---------------------------------------------------------------------------
class CpuKmcSampler:
    """The batched-KMC workload on the host cores: independent trajectories, one per thread (the
    reference's own advice for many trajectories, KineticMcAbstract.cpp:188-189), each a replica of
    the GPU arm's replica set (same seed, edges, temperatures and lattices) advanced by the GPU arm's
    steps per bench step, with the barrier memo that plays the role of the reference's LRU cache.
    Built from oracle/ alone (inputs from oracle/workload.py), so the timed process never loads the
    product library. Successive samples take successive replicas of the set."""

    def __init__(self, seed: int, replicas: int, threads: int, steps_per_replica: int):
        from oracle import oracle as O
        from oracle import workload as W
        self.O, self.W = O, W
        cfg = W.KMC_BATCHED
        self.elements = cfg["elements"]
        coeffs = W.make_coefficients(self.elements, seed)
        self.coeffs = {k: {kk: np.asarray(vv) if isinstance(vv, list) else vv for kk, vv in blk.items()}
                       for k, blk in coeffs.items()}
        self.seed, self.threads, self.steps = seed, threads, steps_per_replica
        self.ns, self.temps = W.batched_edges_and_temperatures(seed, replicas, cfg["n_range"], cfg["T_range"])
        self.next = 0

    def sample(self):
        """Runs one sample; returns (events/s over all threads, wall seconds, replica ids)."""
        from concurrent.futures import ThreadPoolExecutor
        O, W = self.O, self.W
        ids = [(self.next + i) % self.ns.size for i in range(self.threads)]
        self.next += self.threads
        jobs = []
        for r in ids:  # set-up outside the timed region
            n = int(self.ns[r])
            lat = O.Lattice(n)
            jobs.append((lat, O.Model(self.elements, self.coeffs, lat), W.batched_replica_lattice(self.seed, r, n),
                         float(self.temps[r])))

        def one(job):
            lat, m, sp, T = job
            O.kmc(m, lat, sp, T, self.seed, self.steps, memo=True)

        t0 = time.perf_counter()
        with ThreadPoolExecutor(max_workers=self.threads) as ex:  # ctypes releases the GIL in the C call
            list(ex.map(one, jobs))
        wall = time.perf_counter() - t0
        return self.threads * self.steps / wall, wall, ids


def cpu_cmc_baseline(threads: int, attempts: int):
    """CanonicalMcOmp restated (batch = threads) on the CMC workload's lattice, inputs from oracle/."""
    from oracle import oracle as O
    from oracle import workload as W

    cfg = W.CMC_SINGLE
    coeffs = W.make_coefficients(cfg["elements"], 4321)
    sp = W.make_lattice(cfg["n"], cfg["fractions"], 0, 4321, cfg["elements"])
    lat = O.Lattice(cfg["n"])
    m = O.Model(cfg["elements"], coeffs, lat)
    os.environ["OMP_NUM_THREADS"] = str(threads)
    t0 = time.perf_counter()
    done, _, _, _ = O.cmc(m, lat, sp, cfg["T"], 1, attempts, threads)
    wall = time.perf_counter() - t0
    return done / wall, wall


def run_reference(args, rank, world):
    """The reference's algorithm on the host cores for the GPU arm's workload and config: the oracle's
    C restatement of KineticMcFirstOmp (the reference's own build cannot run here: see the CPU
    baseline section of the design notes). Every step is a bounded sample of the same replica set."""
    from oracle import oracle as O
    from oracle import workload as W

    O.build()
    threads = os.cpu_count() or 1
    sampler = CpuKmcSampler(rank_seed(0), args.replicas, threads, args.kmc_steps_per_launch)
    warm = CpuKmcSampler(rank_seed(0), args.replicas, threads, min(1000, args.kmc_steps_per_launch))
    warm.next = args.replicas // 2
    for _ in range(args.warmup):  # untimed, shorter samples of other replicas
        warm.sample()
    walls = []
    for _ in range(args.steps):
        walls.append(sampler.sample()[1])
    events = threads * args.kmc_steps_per_launch * args.steps
    value = events / float(np.sum(walls))
    cmc_v, cmc_w = cpu_cmc_baseline(threads, args.cpu_cmc_attempts)
    sites_total = int(np.sum(4 * sampler.ns.astype(np.int64) ** 3))
    sample = (f"per step {threads} of the {args.replicas} replicas (one per host thread, the next {threads} each "
              f"step), {args.kmc_steps_per_launch} KMC steps each, oracle C restatement of KineticMcFirstOmp with "
              "barrier memo; inputs from oracle/workload.py")
    return {
        "metric": METRIC, "value": value, "unit": "events/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": float(np.mean(walls) * 1e3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64 (reference algorithm)",
        "data": "synthetic (seeded lattices and coefficients; the reference ships none)", "impl": "reference",
        "config": kmc_config(args, world, sites_total),
        "cpu_baseline": {"value": value, "unit": "events/s", "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "events/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "cmc": {"value": cmc_v, "unit": "swaps/s (Metropolis attempts)", "cores": threads,
                "sample": f"{args.cpu_cmc_attempts} attempts, batch = {threads} (CanonicalMcOmp), {cmc_w:.1f} s"},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--replicas", type=int, default=4096)
    ap.add_argument("--kmc-steps-per-launch", type=int, default=KMC_STEPS_PER_BENCH_STEP)
    ap.add_argument("--cmc-steps", type=int, default=5)
    ap.add_argument("--cmc-sweeps-per-step", type=int, default=2)
    ap.add_argument("--cpu-cmc-attempts", type=int, default=1_500_000)
    ap.add_argument("--cmc-ref-attempts", type=int, default=400_000,
                    help="attempts of the reference-order CMC kernel (0 skips)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--surrogate-samples", type=int, default=2_000_000, help="0 skips the surrogate block")
    ap.add_argument("--surrogate-epochs", type=int, default=30, help="epochs of the 4 x 256 one-hot ensemble")
    ap.add_argument("--surrogate-n", type=int, default=192, help="cube edge of the surrogate block's lattices")
    ap.add_argument("--surrogate-epochs-compact", type=int, default=80,
                    help="epochs of the 2 x 128 solute-channel ensemble (fused jump kernel)")
    ap.add_argument("--traffic", type=float, default=None, help="ncu DRAM bytes per launch (profiles/)")
    ap.add_argument("--chain-steps", type=int, default=100, help="chain KMC steps per replica (0 skips)")
    ap.add_argument("--single-steps", type=int, default=100_000, help="steps of the one-trajectory case (0 skips)")
    ap.add_argument("--sa-steps", type=int, default=200_000, help="simulated-annealing trial moves (0 skips)")
    ap.add_argument("--large-cmc-sweeps", type=int, default=100, help="CMC sweeps on the n=64 lattice")
    ap.add_argument("--large-kmc-events", type=int, default=1_000_000, help="multi-vacancy KMC events, n=64")
    ap.add_argument("--large-surrogate-traced", type=int, default=20_000,
                    help="traced surrogate-assisted steps (barrier error of the selected events), n=64")
    ap.add_argument("--no-large", action="store_true", help="skip the n=64, 64-vacancy block")
    ap.add_argument("--tune-probe-steps", type=int, default=100, help="KMC steps per autotuner probe")
    ap.add_argument("--tune-cache", default=os.environ.get("LMC_KMC_TUNE_CACHE", ""),
                    help="JSON cache of autotuned KMC launch shapes (empty: tune every run)")
    args = ap.parse_args()
    rank, world, local = dist_info()
    if args.impl == "reference":
        if rank != 0:
            return
        print(json.dumps(run_reference(args, rank, world)), flush=True)
        return
    result, _ = run_ours(args, rank, world, local)
    if rank == 0:
        if not args.no_cpu_baseline:
            threads = os.cpu_count() or 1
            sampler = CpuKmcSampler(rank_seed(0), args.replicas, threads, args.kmc_steps_per_launch)
            v, w, ids = sampler.sample()
            result["cpu_baseline"] = {
                "value": v, "unit": "events/s", "cores": threads, "kind": "port",
                "sample": f"replicas {ids[0]}..{ids[-1]} of the same replica set (one per host thread), "
                          f"{args.kmc_steps_per_launch} KMC steps each, oracle C restatement of KineticMcFirstOmp "
                          f"with barrier memo, {w:.1f} s wall"}
            if "cmc" in result:
                cv, cw = cpu_cmc_baseline(threads, args.cpu_cmc_attempts)
                result["cmc"]["cpu_baseline"] = {
                    "value": cv, "unit": "swaps/s (Metropolis attempts)", "cores": threads, "kind": "port",
                    "sample": f"{args.cpu_cmc_attempts} attempts of CanonicalMcOmp (batch = {threads} OpenMP "
                              f"threads), same lattice, oracle C restatement, {cw:.1f} s wall"}
        print(json.dumps(result), flush=True)


if __name__ == "__main__":
    main()
