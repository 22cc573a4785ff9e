"""Replicas across ranks, as bench.py runs under torchrun, on CPU with gloo: the
barrier and the max / sum over ranks that make a multi-GPU line (value = the units all
ranks processed / the slowest rank's time), and the reference arm's rank rule (rank 0
alone measures and prints; the other ranks exit 0 without work)."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def run_ranks(argv, world=2, timeout=240):
    port = free_port()
    procs = []
    for r in range(world):
        env = dict(os.environ, WORLD_SIZE=str(world), RANK=str(r), LOCAL_RANK=str(r),
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable] + argv, cwd=ROOT, env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    out = []
    try:
        for p in procs:
            o, e = p.communicate(timeout=timeout)
            out.append((p.returncode, o, e))
    finally:
        for p in procs:
            if p.poll() is None:
                p.kill()
    return out


def test_rank_reductions_two_ranks():
    pytest.importorskip("torch.distributed")
    code = ("import json, bench; d = bench.Dist(); d.barrier(); "
            "print(json.dumps([d.rank, d.world, d.max(d.rank + 1.5), d.sum(10.0 * (d.rank + 1))]))")
    res = run_ranks(["-c", code])
    for rc, _, err in res:
        assert rc == 0, err[-2000:]
    vals = [json.loads(o.strip().splitlines()[-1]) for _, o, _ in res]
    assert sorted(v[0] for v in vals) == [0, 1]
    for _, world, mx, total in vals:
        assert world == 2
        assert mx == 2.5          # the slowest rank's time
        assert total == 30.0      # the units of both ranks


def test_reference_arm_runs_on_rank_zero_only():
    pytest.importorskip("torch.distributed")
    res = run_ranks(["bench.py", "--impl", "reference", "--config", "small", "--steps", "1",
                     "--warmup", "0", "--cpu-threads", "2", "--gpus", "2"])
    for rc, _, err in res:
        assert rc == 0, err[-2000:]
    lines = [[ln for ln in o.splitlines() if ln.startswith("{")] for _, o, _ in res]
    assert len(lines[0]) == 1 and lines[1] == []
    line = json.loads(lines[0][0])
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["cpu_baseline"]["cores"] == 2
    assert line["e2e"]["h2d_bytes_per_step"] == 0
