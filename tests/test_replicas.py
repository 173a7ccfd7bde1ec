"""Multi-rank host path on CPU: two gloo ranks split the partial waves of a
sweep, propagate them (CPU oracle) and gather P(E) on rank 0; the result equals
one process doing all waves.  No GPU is involved."""
import os
import socket

import numpy as np

from madwave3_gb300 import replicas


def test_partition_balanced_and_complete():
    costs = [float(c) for c in (7, 1, 3, 3, 5, 2, 8, 1)]
    parts = replicas.partition(costs, 3)
    flat = sorted(i for p in parts for i in p)
    assert flat == list(range(len(costs)))
    loads = [sum(costs[i] for i in p) for p in parts]
    assert max(loads) - min(loads) <= max(costs)
    assert replicas.partition([1.0], 4)[0] == [0]


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, case_dirs, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from madwave3_gb300.host import setup
    from oracle.mw3ref import Oracle
    names = sorted(case_dirs)
    runs = {n: setup.load(os.path.join(case_dirs[n], "input.dat")) for n in names}
    costs = [float(runs[n].ntot) for n in names]
    mine = replicas.partition(costs, world)[rank]
    local = {}
    for i in mine:
        n = names[i]
        o = Oracle(runs[n])
        o.start(runs[n].psi0)
        o.run_iters(20)
        local[n] = o.totalflux()[0]
    t = replicas.max_over_ranks(float(rank + 1))
    merged = replicas.gather_results(local)
    if rank == 0:
        np.savez(out, t=t, **merged)
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_split_waves(case_dirs, tmp_path):
    import torch.multiprocessing as mp
    out = str(tmp_path / "merged.npz")
    mp.start_processes(_worker, args=(2, _free_port(), dict(case_dirs), out), nprocs=2, join=True,
                       start_method="spawn")
    got = np.load(out)
    assert float(got["t"]) == 2.0
    from madwave3_gb300.host import setup
    from oracle.mw3ref import Oracle
    for n, d in case_dirs.items():
        run = setup.load(os.path.join(d, "input.dat"))
        o = Oracle(run)
        o.start(run.psi0)
        o.run_iters(20)
        assert np.array_equal(got[n], o.totalflux()[0])
