"""Multi-GPU is replicas only (no data-path collective): each rank steps its
own copy of the mesh and the job's time is the slowest rank's.  Checked here
with two gloo ranks on the CPU, each running the oracle as its replica."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, out):
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parents[1]
    sys.path[:0] = [str(root / "dynearthsol-old_gb300"), str(root), str(root / "tests")]
    import torch.distributed as tdist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    tdist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    from des_gb300 import workload as W
    from helpers import Case
    c = Case(W.CONFIGS["tiny"])
    s = c.initial_state()
    c.oracle.step(s, 5)
    ms = 10.0 * (rank + 1)            # ranks report different local times
    value, ms_max = bench.replica_throughput(ms, c.mesh.nelem, 5, world, bench.torch_reduce_max("cpu"))
    out[rank] = (value, ms_max, float(np.abs(s.stress).sum()), float(np.abs(s.vel).sum()))
    tdist.destroy_process_group()


def test_two_replicas_with_gloo():
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    procs = [ctx.Process(target=_rank, args=(r, world, port, out)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    v0, ms0, s0, u0 = out[0]
    v1, ms1, s1, u1 = out[1]
    assert ms0 == ms1 == 20.0                     # max over ranks
    assert v0 == v1 == 2 * 144 * 5 / 0.020        # whole-job element-steps/s
    assert (s0, u0) == (s1, u1)                   # replicas are deterministic and identical
