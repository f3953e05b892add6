"""bench.py's multi-GPU path is replicas only (the Stokes path here runs on one
GPU; the reference's MPI decomposition is not rebuilt).  The combination of
the replicas' lines is checked with two gloo ranks on the CPU."""
import os
import socket
import sys

import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    line = {"value": 2.0 + rank, "ms_per_step": 100.0 * (rank + 1), "e2e": {"value": 3.0 - rank},
            "particles_per_s": 1e6 / (rank + 1), "config": {}}
    res = bench.combine_replicas(line, world, "cpu")
    out[rank] = (res["value"], res["ms_per_step"], res["e2e"]["value"], res["particles_per_s"], res["n_gpus"])
    dist.destroy_process_group()


def test_replicas_combine_with_gloo():
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        procs = [ctx.Process(target=_rank, args=(r, world, port, out)) for r in range(world)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        for r in range(world):
            value, ms, e2e, pps, n = out[r]
            assert value == 3.0 and ms == 200.0 and e2e == 3.0 and n == 2
            assert abs(pps - 2 * 1e6 / 2) < 1e-6
