"""Multi-process (N > 1) path on CPU with gloo, world size 2: bench.py's
--gpus N mode runs independent replicas and reduces the step time with MAX
over ranks; replicas of the deterministic solve agree bit for bit."""
import os
import socket

import numpy as np
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    import torch
    import torch.distributed as dist

    import bench
    from oracle import pyoracle as po

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    P = po.OracleProblem(po.default_params(6), nthreads=1)
    u = np.zeros(P.neq)
    st, _ = P.solve_steps(u, 4, 0, 2)
    t = bench.reduce_max(float(rank + 1), dist)
    digest = float(np.abs(u).sum())
    g = [None] * world
    dist.all_gather_object(g, (digest, st.newton_iters))
    out[rank] = (t, g)
    dist.destroy_process_group()


def test_two_rank_replicas_gloo():
    port = _free_port()
    with mp.get_context("spawn").Manager() as m:
        out = m.dict()
        mp.start_processes(_worker, args=(2, port, out), nprocs=2, start_method="spawn")
        res = dict(out)
    assert res[0][0] == 2.0 and res[1][0] == 2.0
    (d0, i0), (d1, i1) = res[0][1]
    assert d0 == d1 and i0 == i1
