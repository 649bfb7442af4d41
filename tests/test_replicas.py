"""The N > 1 path on the host: world_size-2 gloo process groups.  Replicas
meet at barriers, reduce their timings (max over ranks), seed independent
inputs; under torchrun the reference arm prints exactly one line, from rank 0."""

import json
import os
import socket
import subprocess
import sys

import pytest

from tests.conftest import ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    from arborx_gb300.replicas import Replicas, replica_seed, whole_job_rate

    g = Replicas("gloo")
    g.barrier()
    mx = g.max(10.0 + rank)
    sm = g.sum(1.0 + rank)
    rate = whole_job_rate(1000, mx, g.world)
    g.barrier()
    g.close()
    with open(os.path.join(out, "r%d.json" % rank), "w") as f:
        json.dump({"max": mx, "sum": sm, "rate": rate, "seed": replica_seed(3, rank)}, f)


def test_gloo_world_size_2(tmp_path):
    import torch.multiprocessing as mp

    port = _free_port()
    ctx = mp.get_context("spawn")
    ps = [ctx.Process(target=_worker, args=(r, 2, port, str(tmp_path))) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(120)
        assert p.exitcode == 0
    res = [json.load(open(tmp_path / ("r%d.json" % r))) for r in range(2)]
    for r in res:
        assert r["max"] == 11.0 and r["sum"] == 3.0
        assert r["rate"] == pytest.approx(2000 / 11.0)
    assert res[0]["seed"] != res[1]["seed"]


def test_reference_arm_under_torchrun_prints_one_line():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl",
           "reference", "--gpus", "2", "--steps", "1", "--warmup", "1", "--points", "20000",
           "--queries", "4000", "--cpu-sample", "2000"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0
