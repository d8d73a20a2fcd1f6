"""bench.py's multi-GPU form is replicas only (no data-path collective): each
rank renders its own frame range and rank 0 reports the max of the timings and
the sum of the ray counts.  Checked here with world_size-2 gloo ranks on CPU."""
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

WORKER = r"""
import os, sys, json
sys.path.insert(0, os.environ["ROOT"])
import torch.distributed as dist
import bench
dist.init_process_group("gloo")
r = dist.get_rank()
times, counts = bench.reduce_replicas(dist, [1.0 + r, 5.0 - 3 * r], [100.0 * (r + 1), 7.0], "cpu")
frames = bench.replica_frame_index(r)
out = {"rank": r, "times": times, "counts": counts, "frame0": frames}
print(json.dumps(out), flush=True)
dist.destroy_process_group()
"""


def _port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def test_replica_reduction_two_gloo_ranks(tmp_path):
    pytest.importorskip("torch")
    w = tmp_path / "worker.py"
    w.write_text(WORKER)
    port = _port()
    procs = []
    for r in range(2):
        env = dict(os.environ, ROOT=ROOT, RANK=str(r), WORLD_SIZE="2", LOCAL_RANK=str(r),
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, str(w)], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    import json
    outs = []
    for p in procs:
        o, e = p.communicate(timeout=120)
        assert p.returncode == 0, e
        outs.append(json.loads(o.strip().splitlines()[-1]))
    for o in outs:
        assert o["times"] == [2.0, 5.0]            # max over ranks
        assert o["counts"] == [300.0, 14.0]        # sum over ranks
    assert {o["frame0"] for o in outs} == {0, 1_000_000}


def test_reference_arm_other_ranks_exit_without_work(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")

    class A:
        gpus, steps, warmup = 2, 1, 0
    assert bench.run_reference(A()) == 0
    assert capsys.readouterr().out == ""
