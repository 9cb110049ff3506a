"""The two-step kernels (two PSV or SH time steps per launch) against the
one-step kernels: the same expressions, with multiply-add contraction and dt
folded into the difference factors, so traces, snapshots and the final state
agree to rounding (relative L2 within 1e-5, the FP32 tolerance of the parity
tests); plus one case of each against the FP32 oracle.  Cases: grids narrower
than one strip, strip and chunk boundaries, odd nt, snapshot steps that split
a pair, receivers and sources on the edges, every taper edge, chunks shorter
than the two-step reach."""
import numpy as np
import pytest

from tests.examples import rel_l2
from tests.test_gpu_parity import _check, _model, _run_pair

pytestmark = pytest.mark.gpu
TOL = 1e-5

FIELDS = {"psv": ("vx", "vz", "sxx", "szz", "sxz"), "sh": ("vy", "sxy", "szy")}
SNAP = {"psv": ["vx", "sxz"], "sh": ["vy"]}


def _run(nx, nz, nt, src, rec, two, rows=0, snap=0, isrc=-1, graphs=None, seed=0, physics="psv", **flags):
    import seiswg_gb300 as sw

    dt = 1.2e-3
    stf = np.stack([sw.ricker(nt, dt, s[2], s[3], s[4], 1.0e10) for s in src], axis=1)
    with sw.Sim(nx, nz, nt, 10.0, 10.0, dt, sh=physics == "sh", psv=physics == "psv", **flags) as sim:
        sim.set_option("cluster", 0)   # SH: the step kernels, not the whole-run cluster kernel
        if graphs is not None:
            sim.set_option("graphs", graphs)
        for k, v in _model(nx, nz, seed).items():
            sim.upload_model(k, v)
        sim.prepare()
        sim.set_sources([s[0] for s in src], [s[1] for s in src], stf)
        sim.set_receivers([r[0] for r in rec], [r[1] for r in rec])
        sim.set_option("two_step", 1 if two else 0)
        if two and rows:
            sim.set_option("two_step_rows", rows)
        snaps = sim.forward(isrc, snap, SNAP[physics] if snap else [])
        out = dict(traces=sim.traces(), snaps=snaps, **{f: sim.state(f) for f in FIELDS[physics]})
        # a second run on the same Sim (graph replay) gives the same bits
        again = sim.forward(isrc, snap, SNAP[physics] if snap else [])
        out["replay"] = np.array_equal(sim.traces(), out["traces"]) and (not snap or np.array_equal(again, snaps))
    return out


CASES = [
    # nx, nz, nt, src, rec, rows, snap, flags
    (60, 37, 121, [(30, 18, 20.0, 0.05, 30.0)], [(0, 0), (59, 36), (30, 2), (1, 35)], 0, 0,
     dict(abs_left=True, abs_right=True, abs_bottom=True, abs_top=True, abs_width=10)),
    (97, 113, 90, [(50, 56, 20.0, 0.04, 60.0), (3, 108, 25.0, 0.04, 10.0)],
     [(i, 105) for i in range(0, 97, 8)] + [(3, 110), (5, 112)], 4, 20, dict(abs_bottom=True, abs_width=12)),
    (33, 250, 75, [(16, 120, 22.0, 0.04, 0.0)], [(16, j) for j in (0, 1, 111, 112, 113, 224, 249)], 5, 0,
     dict(abs_left=True, abs_top=True, abs_width=8)),
    (130, 341, 64, [(64, 170, 20.0, 0.04, 45.0), (64, 170, 18.0, 0.05, 90.0)],
     [(0, 170), (129, 170), (64, 0), (64, 160), (50, 170), (64, 185)], 16, 9,
     dict(abs_left=True, abs_right=True, abs_bottom=True, abs_top=True, abs_width=20)),
    (9, 7, 40, [(4, 3, 30.0, 0.03, 0.0)], [(4, 0), (8, 6), (4, 2), (2, 3)], 0, 0, {}),
]


@pytest.mark.parametrize("physics", ["psv", "sh"])
@pytest.mark.parametrize("case", range(len(CASES)))
def test_two_step_matches_the_one_step_kernel(case, physics):
    nx, nz, nt, src, rec, rows, snap, flags = CASES[case]
    one = _run(nx, nz, nt, src, rec, False, snap=snap, physics=physics, **flags)
    two = _run(nx, nz, nt, src, rec, True, rows=rows, snap=snap, physics=physics, **flags)
    assert np.abs(one["traces"]).max() > 0
    assert rel_l2(two["traces"], one["traces"]) <= TOL
    for f in FIELDS[physics]:
        assert rel_l2(two[f], one[f]) <= TOL, f
    if snap:
        assert rel_l2(two["snaps"], one["snaps"]) <= TOL
    assert one["replay"] and two["replay"]


@pytest.mark.parametrize("physics", ["psv", "sh"])
def test_two_step_without_graphs_and_per_shot(physics):
    nx, nz, nt = 70, 150, 51
    src = [(20, 30, 20.0, 0.04, 0.0), (50, 120, 20.0, 0.04, 90.0)]
    rec = [(i, 5) for i in range(0, 70, 7)]
    f = FIELDS[physics][1]
    for isrc in (0, 1):
        one = _run(nx, nz, nt, src, rec, False, isrc=isrc, graphs=0, physics=physics, abs_right=True, abs_width=10)
        two = _run(nx, nz, nt, src, rec, True, isrc=isrc, graphs=0, physics=physics, abs_right=True, abs_width=10)
        assert rel_l2(two["traces"], one["traces"]) <= TOL and rel_l2(two[f], one[f]) <= TOL


@pytest.mark.parametrize("physics", ["psv", "sh"])
def test_two_step_against_the_oracle(physics):
    import seiswg_gb300 as sw

    nx, nz, nt, dx = 80, 130, 140, 10.0
    flags = dict(sh=physics == "sh", psv=physics == "psv", abs_left=True, abs_right=True, abs_bottom=True,
                 abs_top=True, abs_width=12)
    src = [(40, 60, 20.0, 0.05, 30.0)]
    rec = [(0, 0), (40, 2), (79, 129), (10, 112)]
    orig = sw.Sim.prepare

    def prepare_two_step(self):
        orig(self)
        self.set_option("cluster", 0)
        self.set_option("two_step", 1)

    sw.Sim.prepare = prepare_two_step
    try:
        gpu, ref = _run_pair(nx, nz, nt, dx, 1.5e-3, src, rec, _model(nx, nz, 9), **flags)
    finally:
        sw.Sim.prepare = orig
    _check(gpu, ref, flags)


def test_two_step_is_refused_where_it_does_not_apply():
    import seiswg_gb300 as sw

    for flags in (dict(sh=True, psv=True), dict(psv=True, spin=True)):
        with sw.Sim(40, 40, 10, 10.0, 10.0, 1e-3, **flags) as sim:
            with pytest.raises(sw.SeiswgError):
                sim.set_option("two_step", 1)


@pytest.mark.parametrize("physics", ["psv", "sh"])
@pytest.mark.parametrize("nt,snap", [(1, 0), (2, 0), (3, 0), (6, 1), (7, 2)])
def test_two_step_short_runs_and_dense_snapshots(nt, snap, physics):
    """Runs shorter than a pair, odd lengths, and snapshots after every step
    (no pairs at all) or every second step."""
    src = [(20, 20, 40.0, 0.0, 30.0)]
    rec = [(20, 20), (20, 21), (21, 20), (19, 19)]
    one = _run(40, 44, nt, src, rec, False, snap=snap, physics=physics)
    two = _run(40, 44, nt, src, rec, True, snap=snap, physics=physics)
    assert np.abs(one["traces"]).max() > 0
    assert rel_l2(two["traces"], one["traces"]) <= TOL
    for f in FIELDS[physics]:
        assert rel_l2(two[f], one[f]) <= TOL or np.abs(one[f]).max() == 0, f
    if snap:
        assert two["snaps"].shape == one["snaps"].shape
        assert rel_l2(two["snaps"], one["snaps"]) <= TOL


@pytest.mark.parametrize("physics", ["psv", "sh"])
def test_tensor_copies_fetch_the_same_rows(physics):
    """Rows fetched by 3-D tensor copies (several fields per copy, the
    default) or by one bulk copy per field: the same bytes reach the kernel,
    so the results are the same bits."""
    import seiswg_gb300 as sw

    nx, nz, nt = 97, 241, 60
    src = [(48, 120, 20.0, 0.04, 30.0), (3, 5, 25.0, 0.05, 0.0)]
    rec = [(0, 0), (96, 240), (48, 2), (50, 230)]
    out = []
    for tma in (1, 0):
        dt = 1.2e-3
        stf = np.stack([sw.ricker(nt, dt, s[2], s[3], s[4], 1.0e10) for s in src], axis=1)
        with sw.Sim(nx, nz, nt, 10.0, 10.0, dt, sh=physics == "sh", psv=physics == "psv", abs_left=True,
                    abs_top=True, abs_width=10) as sim:
            sim.set_option("cluster", 0)
            sim.set_option("tma", tma)
            for k, v in _model(nx, nz, 4).items():
                sim.upload_model(k, v)
            sim.prepare()
            sim.set_sources([s[0] for s in src], [s[1] for s in src], stf)
            sim.set_receivers([r[0] for r in rec], [r[1] for r in rec])
            sim.forward(-1)
            out.append((sim.traces(), {f: sim.state(f) for f in FIELDS[physics]}))
    assert np.abs(out[0][0]).max() > 0
    assert np.array_equal(out[0][0], out[1][0])
    for f in FIELDS[physics]:
        assert np.array_equal(out[0][1][f], out[1][1][f]), f
