"""Batched replica KMC as one CUDA graph, and the launch-shape autotuner.

* lmc_kmc_run_graph records the persistent launches once and replays them: the
  lattices and per-replica states must equal plain lmc_kmc_run calls bit for bit,
  also after the launch arguments change (the graph is re-recorded).
* lmc_kmc_autotune times every accepted launch shape on a copy of the state: the
  state must be unchanged afterwards, the chosen shape must give the same
  trajectories as the default shape, and the JSON cache must be reused."""
import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

EL = ("Al", "Cu", "Mg", "Zn")


def _inputs(replicas=48, seed=11):
    from latticemontecarlo_gb300 import synthetic as S
    coeffs = S.make_coefficients(EL, 5)
    ns, sp, temps = S.batched_replicas(seed, replicas, n_range=(8, 12),
                                       fractions={"Al": 0.9, "Cu": 0.03, "Mg": 0.04, "Zn": 0.03}, elements=EL)
    return coeffs, ns, sp, temps


def _ctx(coeffs, ns, sp, temps, **kw):
    from latticemontecarlo_gb300 import api
    ctx = api.Context(api.Model.from_coefficients(coeffs, list(EL)))
    ctx.set_lattices(ns, sp)
    ctx.kmc_init(temps, seed=3, rng=1, **kw)
    return ctx


def _snapshot(ctx):
    return (ctx.get_lattices().copy(),) + tuple(a.copy() for a in ctx.kmc_state())


def _assert_same(a, b):
    assert len(a) == len(b)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_graph_equals_direct_launches(native):
    coeffs, ns, sp, temps = _inputs()
    direct = _ctx(coeffs, ns, sp, temps)
    for _ in range(4):
        direct.kmc_run(60)
    graph = _ctx(coeffs, ns, sp, temps)
    graph.kmc_run_graph(60, launches=2)  # recorded
    graph.kmc_run_graph(60, launches=2)  # replayed
    _assert_same(_snapshot(direct), _snapshot(graph))
    assert np.all(graph.kmc_state()[1] == 240)


def test_graph_rerecords_when_arguments_change(native):
    coeffs, ns, sp, temps = _inputs(replicas=24, seed=4)
    direct = _ctx(coeffs, ns, sp, temps, warps_per_replica=2)
    direct.kmc_run(50)
    direct.kmc_run(30)
    graph = _ctx(coeffs, ns, sp, temps, warps_per_replica=2)
    graph.kmc_run_graph(50)
    graph.kmc_run_graph(30)  # new step count: a new graph
    _assert_same(_snapshot(direct), _snapshot(graph))
    # a fresh kmc_init with another shape and evaluation: same trajectories from the start
    graph.set_lattices(ns, sp)
    graph.kmc_init(temps, seed=3, rng=1, warps_per_replica=1, evaluation=1)
    graph.kmc_run_graph(80)
    fresh = _ctx(coeffs, ns, sp, temps)
    fresh.kmc_run(80)
    _assert_same(_snapshot(fresh), _snapshot(graph))


def test_graph_reports_stop(native):
    coeffs, ns, sp, temps = _inputs(replicas=8, seed=2)
    ctx = _ctx(coeffs, ns, sp, temps)
    ctx.request_stop(1)
    with pytest.raises(native.LmcError) as e:
        ctx.kmc_run_graph(100)
    assert e.value.code == native.LMC_ERR_STOPPED
    ctx.request_stop(0)
    ctx.kmc_run_graph(100)
    ref = _ctx(coeffs, ns, sp, temps)
    ref.kmc_run(100)
    _assert_same(_snapshot(ref), _snapshot(ctx))


def test_autotune_keeps_state_and_results(native, tmp_path):
    coeffs, ns, sp, temps = _inputs(replicas=96, seed=9)
    tuned = _ctx(coeffs, ns, sp, temps)
    tuned.kmc_run(25)
    before = _snapshot(tuned)
    cache = tmp_path / "kmc_tune.json"
    choice = tuned.kmc_autotune(probe_steps=20, cache=cache)
    assert not choice["from_cache"]
    _assert_same(before, _snapshot(tuned))  # the sweep ran on a copy
    info = tuned.kmc_launch_info()
    assert info["warps_per_replica"] == choice["warps_per_replica"]
    assert info["replicas_per_block"] == choice["replicas_per_block"]
    assert info["blocks_per_sm"] >= 1
    tuned.kmc_run_graph(75)
    plain = _ctx(coeffs, ns, sp, temps)
    plain.kmc_run(100)
    _assert_same(_snapshot(plain), _snapshot(tuned))
    # the cache holds one entry keyed by the GPU and the size histogram, and is reused
    data = json.loads(cache.read_text())
    assert len(data) == 1
    (key, entry), = data.items()
    assert "|sms=" in key and "|n=" in key and entry["ms"] > 0
    again = _ctx(coeffs, ns, sp, temps)
    hit = again.kmc_autotune(probe_steps=20, cache=cache)
    assert hit["from_cache"]
    assert {k: hit[k] for k in ("warps_per_replica", "replicas_per_block", "evaluation")} == \
           {k: choice[k] for k in ("warps_per_replica", "replicas_per_block", "evaluation")}
    # another batch (another size histogram) is another key
    coeffs2, ns2, sp2, temps2 = _inputs(replicas=64, seed=10)
    other = _ctx(coeffs2, ns2, sp2, temps2)
    assert not other.kmc_autotune(probe_steps=20, cache=cache)["from_cache"]
    assert len(json.loads(cache.read_text())) == 2
