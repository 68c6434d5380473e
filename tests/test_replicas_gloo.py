"""The multi-GPU path is replicas only: every rank scans its own seeded
targets and the one collective is the max over ranks of the timed region.
Covered here with two gloo ranks on CPU (no GPU): the reduction returns the
slowest rank's times on every rank, the aggregate rate counts all ranks'
residues over that time, and different ranks draw different targets."""
import os
import socket

import numpy as np
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import sys
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        t_dev, t_e2e = bench.max_over_ranks([1.0 + rank, 5.0 - rank], world, device="cpu")
        from infernal_gb300 import cmfile
        m = cmfile.load_npz(os.path.join(ROOT, "tests", "golden", "tRNA.model.npz"))
        fwd, _ = bench.make_step_input(m, bench.rank_step_seed(rank, 0), 0.01)
        out[rank] = (t_dev, t_e2e, int(fwd[1:-1].astype(np.int64).sum()))
    finally:
        dist.destroy_process_group()


def test_two_gloo_replicas():
    world = 2
    out = mp.Manager().dict()
    mp.spawn(_rank, args=(world, _free_port(), out), nprocs=world, join=True)
    assert out[0][:2] == out[1][:2] == (2.0, 5.0)        # every rank sees the slowest rank's times
    assert out[0][2] != out[1][2]                         # each replica scans its own targets
    residues_per_rank = 2 * 10_000
    value = residues_per_rank * world / out[0][0] / 1e6   # whole-job rate over the max time
    assert abs(value - 0.02) < 1e-12
