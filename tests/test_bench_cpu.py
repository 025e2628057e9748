"""bench.py's host logic on CPU: the max-over-ranks / sum-of-pairs aggregation of a
multi-GPU run (two gloo ranks), and the reference arm (the oracle on the host cores) with
its JSON line, alone and under torchrun with two ranks (rank 0 alone prints)."""
import json
import os
import socket
import subprocess
import sys

import pytest
import torch.multiprocessing as mp

from conftest import ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _aggregate_rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        secs, pairs = bench.aggregate(1.0 + rank, 10.0 * (rank + 1), world)
        out[rank] = (secs, pairs)
    finally:
        dist.destroy_process_group()


def test_aggregate_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        port = _free_port()
        procs = [ctx.Process(target=_aggregate_rank, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        # the time is the slowest rank's, the pairs are all ranks' together
        assert out[0] == (2.0, 30.0) and out[1] == (2.0, 30.0)


def _run(cmd, env=None):
    e = dict(os.environ)
    e.update(env or {})
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600, env=e)
    assert r.returncode == 0, r.stderr[-2000:]
    return [json.loads(l) for l in r.stdout.splitlines() if l.startswith("{")]


ARGS = ["--impl", "reference", "--steps", "1", "--warmup", "1", "--n-side", "24",
        "--cpu-sample", "4000"]


def test_reference_arm_json_line():
    lines = _run([sys.executable, "bench.py"] + ARGS)
    assert len(lines) == 1
    d = lines[0]
    assert d["impl"] == "reference" and d["unit"] == "pair-evals/s" and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["e2e"]["value"] == d["value"]
    assert d["higher_is_better"] is True and d["steps"] == 1 and d["warmup"] == 1


@pytest.mark.timeout(600)
def test_reference_arm_two_ranks_prints_once():
    port = _free_port()
    lines = _run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1",
                  "--nproc-per-node", "2", "--master-addr", "127.0.0.1", "--master-port",
                  str(port), "bench.py", "--gpus", "2"] + ARGS)
    assert len(lines) == 1 and lines[0]["impl"] == "reference"
