"""Shot/problem sharding across ranks (one process per GPU): the assignment
rule, and a world-size-2 gloo run on the CPU whose rank-ordered gradient sum
matches the single-process sum over all shots."""
import os
import socket
import subprocess
import sys

import numpy as np
import pytest

from seiswg_gb300 import shards

HERE = os.path.dirname(os.path.abspath(__file__))


def test_assign_covers_every_unit_once_and_balances():
    rng = np.random.default_rng(0)
    costs = list(rng.integers(256, 1537, 48) * rng.integers(256, 1537, 48) * rng.integers(1000, 3001, 48))
    for world in (1, 2, 3, 4, 8):
        parts = shards.assign(costs, world)
        flat = sorted(u for p in parts for u in p)
        assert flat == list(range(len(costs)))
        assert all(p == sorted(p) for p in parts)
        assert shards.imbalance(costs, world) < 1.15
        assert shards.assign(costs, world) == parts          # deterministic
    assert shards.assign([1.0] * 5, 2) == [[0, 2, 4], [1, 3]]
    assert shards.assign([], 3) == [[], [], []]
    with pytest.raises(ValueError):
        shards.assign([1.0], 0)
    with pytest.raises(ValueError):
        shards.my_units([1.0], 2, 2)


def test_reduce_without_process_group_is_identity():
    g = {"mu": np.arange(6, dtype=np.float32).reshape(2, 3)}
    out = shards.reduce_gradients(g)
    assert np.array_equal(out["mu"], g["mu"])


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_rank_gradient_sum_matches_single_process(tmp_path):
    sys.path.insert(0, HERE)
    import shard_worker as W

    out = str(tmp_path / "g.npz")
    port = str(_free_port())
    env = dict(os.environ, OMP_NUM_THREADS="2")
    procs = [subprocess.Popen([sys.executable, os.path.join(HERE, "shard_worker.py"), str(r), "2", port, out],
                              env=env, stdout=subprocess.PIPE, stderr=subprocess.STDOUT) for r in range(2)]
    logs = []
    for p in procs:
        try:
            logs.append(p.communicate(timeout=240)[0].decode(errors="replace"))
        except subprocess.TimeoutExpired:
            for q in procs:
                q.kill()
            raise
    assert all(p.returncode == 0 for p in procs), logs
    r0, r1 = np.load(out), np.load(out + ".r1.npz")
    assert sorted(list(r0["units"]) + list(r1["units"])) == list(range(len(W.SHOTS)))
    single = W.local_sum(range(len(W.SHOTS)))
    for name in ("lambda", "mu", "buoyancy"):
        assert np.array_equal(r0[name], r1[name])            # same bits on every rank
        ref = single[name].astype(np.float64)
        err = np.linalg.norm(r0[name] - ref) / np.linalg.norm(ref)
        assert err < 1e-6, (name, err)
