"""Whole forward runs of small SH grids in one thread-block cluster
(fd_cluster.cu) against the one-launch-per-step kernel: the same expressions
in the same order, so traces, snapshots and the final state are equal bit for
bit.  Cases: the 200 x 200 benchmark geometry with snapshots, a grid narrower
than a strip, odd sizes, sources and receivers on the edges, several sources
in one cell, and a grid too large for the cluster (the step kernels run)."""
import numpy as np
import pytest

from tests.test_gpu_parity import _model

pytestmark = pytest.mark.gpu

FIELDS = ("vy", "sxy", "szy")


def _run(nx, nz, nt, src, rec, cluster, snap=0, isrc=-1, graphs=None, **flags):
    import seiswg_gb300 as sw

    dt = 1.0e-3
    stf = np.stack([sw.ricker(nt, dt, s[2], s[3], s[4], 1.0e10) for s in src], axis=1)
    with sw.Sim(nx, nz, nt, 10.0, 10.0, dt, sh=True, psv=False, **flags) as sim:
        sim.set_option("cluster", 1 if cluster else 0)
        sim.set_option("two_step", 0)   # the one-step kernel where the cluster does not run
        if graphs is not None:
            sim.set_option("graphs", graphs)
        for k, v in _model(nx, nz, 3).items():
            sim.upload_model(k, v)
        sim.prepare()
        sim.set_sources([s[0] for s in src], [s[1] for s in src], stf)
        sim.set_receivers([r[0] for r in rec], [r[1] for r in rec])
        snaps = sim.forward(isrc, snap, ["vy"] if snap else [])
        out = dict(traces=sim.traces(), snaps=snaps, **{f: sim.state(f) for f in FIELDS})
        again = sim.forward(isrc, snap, ["vy"] if snap else [])   # graph replay
        out["replay"] = np.array_equal(sim.traces(), out["traces"]) and (not snap or np.array_equal(again, snaps))
    return out


CASES = [
    (200, 200, 300, [(100, 100, 10.0, 0.12, 0.0)], [(i, 20) for i in range(10, 191, 8)] + [(100, 100)], 100,
     dict(abs_left=True, abs_right=True, abs_bottom=True, abs_top=True, abs_width=20)),
    (150, 37, 160, [(75, 18, 20.0, 0.05, 0.0), (75, 18, 15.0, 0.06, 0.0)], [(0, 0), (75, 2), (149, 36), (1, 1)],
     0, dict(abs_left=True, abs_bottom=True, abs_width=10)),
    (33, 251, 120, [(16, 120, 22.0, 0.04, 0.0), (2, 3, 25.0, 0.05, 0.0)], [(16, j) for j in (0, 1, 119, 120, 249)],
     7, dict(abs_top=True, abs_width=8)),
    (9, 7, 40, [(4, 3, 30.0, 0.03, 0.0)], [(4, 2), (2, 3)], 0, {}),
    (700, 900, 30, [(350, 450, 20.0, 0.02, 0.0)], [(350, 440)], 0, {}),   # too large: step kernels
]


@pytest.mark.parametrize("case", range(len(CASES)))
def test_cluster_is_bitwise_the_step_kernel(case):
    nx, nz, nt, src, rec, snap, flags = CASES[case]
    one = _run(nx, nz, nt, src, rec, False, snap=snap, **flags)
    clu = _run(nx, nz, nt, src, rec, True, snap=snap, **flags)
    assert np.abs(one["traces"]).max() > 0
    assert np.array_equal(one["traces"], clu["traces"])
    for f in FIELDS:
        assert np.array_equal(one[f], clu[f]), f
    if snap:
        assert np.array_equal(one["snaps"], clu["snaps"])
    assert one["replay"] and clu["replay"]


def test_cluster_per_shot_without_graphs():
    nx, nz, nt = 120, 140, 90
    src = [(30, 40, 20.0, 0.04, 0.0), (90, 100, 20.0, 0.04, 0.0)]
    rec = [(i, 60) for i in range(0, 120, 10)]
    for isrc in (0, 1):
        one = _run(nx, nz, nt, src, rec, False, isrc=isrc, graphs=0)
        clu = _run(nx, nz, nt, src, rec, True, isrc=isrc, graphs=0)
        assert np.array_equal(one["traces"], clu["traces"]) and np.array_equal(one["vy"], clu["vy"])


@pytest.mark.parametrize("nt,snap", [(1, 0), (2, 1), (5, 2)])
def test_cluster_short_runs(nt, snap):
    src = [(20, 20, 40.0, 0.0, 0.0)]
    rec = [(20, 20), (20, 21), (21, 20)]
    one = _run(40, 44, nt, src, rec, False, snap=snap)
    clu = _run(40, 44, nt, src, rec, True, snap=snap)
    assert np.array_equal(one["traces"], clu["traces"])
    for f in FIELDS:
        assert np.array_equal(one[f], clu[f]), f
    if snap:
        assert np.array_equal(one["snaps"], clu["snaps"])
