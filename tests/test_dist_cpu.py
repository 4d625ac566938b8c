"""The N > 1 plumbing of bench.py on CPU: world size 2 over gloo.  The stencil
path does not shard (replicas only), so what runs across ranks is the barrier,
the max-over-ranks timing and the reference arm's rank-0-only rule."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _torchrun(args, timeout=240):
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port())] + args
    env = dict(os.environ, MASTER_ADDR="127.0.0.1")
    return subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=timeout,
                          env=env)


def _json_lines(text):
    return [json.loads(l) for l in text.splitlines() if l.startswith("{")]


def test_barrier_and_reductions_over_two_ranks(tmp_path):
    r = _torchrun([os.path.join("tests", "dist_worker.py"), str(tmp_path)])
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.load(open(tmp_path / ("rank%d.json" % k))) for k in (0, 1)]
    assert [l["rank"] for l in lines] == [0, 1]
    for l in lines:
        assert l["max"] == 2.5 and l["sum"] == 30.0


def test_reference_arm_runs_on_rank_zero_only():
    pytest.importorskip("numpy")
    r = _torchrun(["bench.py", "--impl", "reference", "--gpus", "2", "--steps", "1",
                   "--warmup", "0"])
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _json_lines(r.stdout)
    assert len(lines) == 1  # rank 1 exits without work or output
    line = lines[0]
    assert line["impl"] == "reference" and line["n_gpus"] == 2
    assert line["cpu_baseline"]["kind"] == "port"
    # rank 0 takes every host core although torchrun sets OMP_NUM_THREADS=1
    try:
        cores = len(os.sched_getaffinity(0))
    except AttributeError:
        cores = os.cpu_count()
    assert line["cpu_baseline"]["cores"] == cores
    assert line["e2e"]["h2d_bytes_per_step"] == 0
