"""The multi-rank path of bench.py on the CPU (gloo, world size 2): every rank
simulates its own replicas (distinct seeded lattices, no data exchange), and
the job's time is the slowest rank's, so the whole-job throughput is all ranks'
events over that time."""
import os
import socket

import numpy as np
import pytest


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out_dir):
    import torch.distributed as dist

    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        seed = bench.rank_seed(rank)
        cfg, coeffs, ns, species, temps = bench.kmc_inputs(seed, 8)
        t = bench.max_over_ranks(10.0 * (rank + 1), "cpu")
        np.savez(os.path.join(out_dir, f"r{rank}.npz"), ns=ns, species=species, t=t)
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_ranks_gloo(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    port = _free_port()
    mp.start_processes(_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    r0, r1 = np.load(tmp_path / "r0.npz"), np.load(tmp_path / "r1.npz")
    assert float(r0["t"]) == 20.0 and float(r1["t"]) == 20.0  # max over ranks on every rank
    # the ranks hold different replicas (independent shards of the workload)
    assert not (np.array_equal(r0["ns"], r1["ns"]) and np.array_equal(r0["species"], r1["species"]))


def test_single_process_is_identity():
    import bench
    assert bench.max_over_ranks(3.5, "cpu") == 3.5
