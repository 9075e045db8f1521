"""The bench's multi-rank plumbing on the CPU: two gloo ranks on 127.0.0.1.  Replicas only (the
build has no exchange step across GPUs): ranks meet at a barrier, the timed figure is the
maximum over ranks, and the reference arm runs on rank 0 alone while the other ranks exit
without work."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import json
    import sys
    import io
    import contextlib
    import torch.distributed as dist
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import bench

    class A:
        impl = "reference"
        gpus = world
        steps = 1
        warmup = 0
        max_pairs = 300

    ws, rk, local = bench.dist_setup(A)
    assert (ws, rk) == (world, rank)
    bench.barrier(ws)
    m = bench.max_over_ranks(ws, 1.5 + rank)
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        bench.run_reference(A, ws, rk)
    bench.barrier(ws)
    dist.destroy_process_group()
    out[rank] = json.dumps({"max": m, "printed": buf.getvalue()})


def test_two_gloo_ranks():
    import json
    world, port = 2, _free_port()
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = {k: json.loads(v) for k, v in out.items()}
    assert res[0]["max"] == res[1]["max"] == 2.5
    assert res[1]["printed"] == ""
    line = json.loads(res[0]["printed"].strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port"
    assert line["e2e"]["h2d_bytes_per_step"] == 0
