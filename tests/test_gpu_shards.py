"""Shots sharded across ranks with the gradients computed on the GPU: two
processes (gloo, world size 2; both on the one GPU this run has, each with
its own context and kernels that wait on nothing of the other's) each run the
exact gradient of their share of a small PSV problem's shots through a Sim,
then sum the fields in rank order (seiswg_gb300.shards).  Both ranks hold the
same bits, and the sum matches one process running every shot to FP32
rounding (the shots are summed in a different order)."""
import os
import socket
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _run(args, timeout=600):
    procs = [subprocess.Popen([sys.executable, os.path.join(HERE, "shard_gpu_worker.py")] + a,
                              stdout=subprocess.PIPE, stderr=subprocess.STDOUT) for a in args]
    logs = []
    for p in procs:
        try:
            logs.append(p.communicate(timeout=timeout)[0].decode(errors="replace"))
        except subprocess.TimeoutExpired:
            for q in procs:
                q.kill()
            raise
    assert all(p.returncode == 0 for p in procs), logs


def test_two_rank_gpu_gradient_sum_matches_single_process(tmp_path):
    out, ref = str(tmp_path / "g.npz"), str(tmp_path / "single.npz")
    port = str(_free_port())
    _run([[str(r), "2", port, out] for r in range(2)])
    _run([["0", "1", "0", ref]])
    r0, r1, single = np.load(out), np.load(out + ".r1.npz"), np.load(ref)
    assert sorted(list(r0["units"]) + list(r1["units"])) == list(single["units"])
    for name in ("lambda", "mu", "buoyancy"):
        assert np.array_equal(r0[name], r1[name])            # same bits on every rank
        s = single[name].astype(np.float64)
        assert np.abs(s).max() > 0
        err = np.linalg.norm(r0[name] - s) / np.linalg.norm(s)
        assert err < 1e-6, (name, err)
