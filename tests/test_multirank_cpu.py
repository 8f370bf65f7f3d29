"""bench.py's multi-rank host logic on CPU: two gloo ranks on 127.0.0.1.

A run over N GPUs is N independent replicas (the path has no exchange step):
the whole-job value is the units of all ranks over the slowest rank's time,
and the reference arm runs on rank 0 alone while the other ranks exit 0."""
import argparse
import io
import json
import multiprocessing as mp
import os
import socket
import sys
from contextlib import redirect_stdout

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _env(rank, port):
    os.environ.update({"RANK": str(rank), "LOCAL_RANK": str(rank), "WORLD_SIZE": "2",
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)


def _reductions(rank, port, q):
    _env(rank, port)
    import bench
    ws, r, _ = bench.dist_info()
    dist = bench.init_dist(ws)
    t = bench.allreduce_max(dist, 10.0 + 5.0 * r)  # rank 1 is the slower replica
    units = bench.allreduce_sum(dist, 1000.0 * (r + 1))
    bench.barrier(dist)
    q.put((r, ws, t, units, units / (t / 1e3)))
    dist.destroy_process_group()


def _reference_arm(rank, port, q):
    _env(rank, port)
    import bench
    args = argparse.Namespace(workload="box", particles=None, boxes=512, steps=1, warmup=1)
    buf = io.StringIO()
    with redirect_stdout(buf):
        rc = bench.run_reference(args, lambda m: None)
    q.put((rank, rc, buf.getvalue()))


def _run(target):
    pytest.importorskip("torch")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=target, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=300) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    return sorted(out)


def test_replicas_take_the_slowest_rank_and_sum_the_units():
    out = _run(_reductions)
    for r, ws, t, units, value in out:
        assert ws == 2 and t == 15.0 and units == 3000.0
        assert value == pytest.approx(3000.0 / 0.015)


def test_reference_arm_runs_on_rank_zero_only():
    out = _run(_reference_arm)
    (r0, rc0, text0), (r1, rc1, text1) = out
    assert (r0, rc0, rc1) == (0, 0, 0)
    assert text1.strip() == ""
    line = json.loads(text0.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
