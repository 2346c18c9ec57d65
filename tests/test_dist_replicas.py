"""The multi-rank path of bench.py on CPU: world size 2 over gloo, as the
driver's torchrun launch sets it up (RANK / WORLD_SIZE / MASTER_* from the
environment, 127.0.0.1).  The path runs independent replicas: the only
collectives are the barrier, the max over ranks of the timed region and the
whole-job sums; the reference arm runs on rank 0 alone and the other ranks
exit 0 without work."""
import io
import multiprocessing as mp
import os
import socket
import sys
from contextlib import redirect_stdout
from types import SimpleNamespace

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, REPO)
    import bench

    out = {}
    try:
        import torch.distributed as dist

        args = SimpleNamespace(impl="reference", gpus=world, steps=1, warmup=0, cpu_planes=4)
        buf = io.StringIO()
        with redirect_stdout(buf):
            out["rc"] = bench.run_reference(args)  # sets up the process group on every rank
        out["printed"] = buf.getvalue()
        out["world"], out["rank"] = dist.get_world_size(), dist.get_rank()
        bench.barrier(dist)
        out["max"] = bench.allmax(dist, 10.0 * (rank + 1))
        out["sum"] = bench.allsum(dist, rank + 1)
        bench.barrier(dist)
        dist.destroy_process_group()
    except Exception as e:  # reported to the parent, which fails the test
        out["error"] = repr(e)
    q.put((rank, out))


def test_two_rank_replicas_over_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = {}
    try:
        for _ in procs:
            rank, out = q.get(timeout=300)
            res[rank] = out
    finally:
        for p in procs:
            p.join(timeout=30)
            if p.is_alive():
                p.terminate()
                p.join()
    errors = {r: res[r]["error"] for r in res if "error" in res[r]}
    assert not errors, errors
    for r in (0, 1):
        assert res[r]["world"] == 2 and res[r]["rank"] == r
        assert res[r]["max"] == 20.0 and res[r]["sum"] == 3.0
        assert res[r]["rc"] == 0
    # the reference arm prints one JSON line on rank 0 only
    import json

    line = json.loads(res[0]["printed"].strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert res[1]["printed"] == ""
    assert all(p.exitcode == 0 for p in procs)


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, REPO)
    import bench

    env = {k: os.environ.pop(k) for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK") if k in os.environ}
    try:
        w, r, local, pg = bench.dist_setup(SimpleNamespace(impl="gcm"))
        assert (w, r, local, pg) == (1, 0, 0, None)
        assert bench.allmax(pg, 3.5) == 3.5 and bench.allsum(pg, 7) == 7
        bench.barrier(pg)
    finally:
        os.environ.update(env)
