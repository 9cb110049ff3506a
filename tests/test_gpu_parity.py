"""CUDA path against the FP32 CPU oracle on seeded inputs (relative L2 within
1e-5, the FP32 tolerance the path is held to; where the problem's own FP32
rounding exceeds that, at least as accurate against the FP64 oracle as the
reference's FP32 arithmetic, see _agrees; the FP64 oracle error is reported
in the assertion message).  Cases cover the edge rules of fd2d.wgsl: grids
narrower than one warp strip, odd sizes, every taper edge, sources and
receivers on and next to the boundary, co-located sources, per-shot source
selection, SH+PSV together, spin, snapshots, and the reference adjoint with
smoothing."""
import numpy as np
import pytest

from tests.examples import rel_l2

pytestmark = pytest.mark.gpu

L2_TOL = 1e-5


def _model(nx, nz, seed, spin=False, dx=10.0):
    rng = np.random.default_rng(seed)
    p = 1.0 + 0.05 * np.tanh(rng.standard_normal((nx, nz)))
    if spin:
        mu = 8.1e9 * p
        return dict(rho=np.full((nx, nz), 2700.0) * p, **{"lambda": 8.1e9 * p}, mu=mu, nu=1.005e9 * p,
                    j=np.full((nx, nz), 2700.0), lambda_c=7.75e8 * p, mu_c=1.5e8 * p, nu_c=3.0e8 * p)
    vp = 3000.0 * p
    return dict(vp=vp, vs=vp / np.sqrt(3.0), rho=2500.0 * p ** 0.25)


_ORACLE_SLOT = dict(vp="LAM", vs="MU", rho="RHO", mu="MU", nu="NU", j="J", lambda_c="LAM_C", mu_c="MU_C",
                    nu_c="NU_C", **{"lambda": "LAM"})
_STATE = dict(vy="VY", sxy="SXY", szy="SZY", vx="VX", vz="VZ", sxx="SXX", szz="SZZ", sxz="SXZ", vyc="VY_C",
              syx="SYX_C", syy="SYY_C", syz="SYZ_C")


def _run_pair(nx, nz, nt, dx, dt, src, rec, model, isrc=-1, snap=0, snap_fields=(), chunk_rows=None,
              graphs=None, loader=None, two_step=None, **flags):
    """Runs the same problem on the GPU and in both oracles."""
    import seiswg_gb300 as sw
    from oracle import oracle as O

    si = np.array([s[0] for s in src], np.int32)
    sj = np.array([s[1] for s in src], np.int32)
    stf = np.stack([sw.ricker(nt, dt, s[2], s[3], s[4], 1.0e10) for s in src], axis=1)  # [3][nsrc][nt]
    ri = np.array([r[0] for r in rec], np.int32)
    rj = np.array([r[1] for r in rec], np.int32)
    with sw.Sim(nx, nz, nt, dx, dx, dt, **flags) as sim:
        if chunk_rows:
            sim.set_option("chunk_rows", chunk_rows)
        if graphs is not None:
            sim.set_option("graphs", graphs)
        if loader is not None:
            sim.set_option("loader", loader)
        if two_step is not None:
            sim.set_option("two_step", two_step)
        for k, v in model.items():
            sim.upload_model(k, v)
        sim.prepare()
        sim.set_sources(si, sj, stf)
        sim.set_receivers(ri, rj)
        snaps = sim.forward(isrc, snap, snap_fields)
        traces = sim.traces()
        state = {f: sim.state(f) for f in _STATE if _present(f, flags)}
    res = {}
    for prec in (32, 64):
        s = O.Setup(nx, nz, nt, dx, dx, dt, **flags)
        o = O.FD2DOracle(s, si * nz + sj, stf.astype(np.float64), ri * nz + rj, prec)
        for k, v in model.items():
            o.set_field(_ORACLE_SLOT[k], v)
        o.init_model()
        osn = o.run_forward(isrc, snap, [_STATE[f] for f in snap_fields])
        res[prec] = dict(obs=np.stack([o.obs(c) for c in ("X", "Y", "Z", "YI", "YC")]),
                         state={f: o.field(_STATE[f]) for f in state}, snaps=osn)
    return dict(traces=traces, state=state, snaps=snaps), res


def _present(f, flags):
    if f in ("vy", "sxy", "szy"):
        return flags.get("sh", False)
    if f in ("vyc", "syx", "syy", "syz"):
        return flags.get("psv", True) and flags.get("spin", False)
    return flags.get("psv", True)


def _comps(flags):
    c = []
    if flags.get("sh"):
        c.append(1)
    if flags.get("psv", True):
        c += [0, 2]
        if flags.get("spin"):
            c += [1, 3, 4]
    return sorted(set(c))


def _agrees(e32, e64, floor, tol, cancel=False):
    """1e-5 relative L2 against the FP32 oracle.  Where the FP32 rounding of
    the problem itself exceeds that (the FP32 oracle is more than 1e-5 from
    the FP64 one: traces ahead of the first arrival, long runs, cells the
    edge rule isolates), two FP32 results that round differently cannot
    agree to 1e-5; the result must then be at least as close to FP64 as the
    reference's own FP32 arithmetic, and within twice that distance of it.
    The spin rotation yi = uy_c - curl/2 differences two displacement
    derivatives (cancel): 3x the oracle's distance from FP64 is allowed."""
    if e32 <= tol:
        return True
    if e64 <= floor and e32 <= 2 * floor:
        return True
    return cancel and e32 <= 3 * floor


def _check(gpu, ref, flags, tol=L2_TOL):
    for c in _comps(flags):
        e32 = rel_l2(gpu["traces"][c], ref[32]["obs"][c])
        e64 = rel_l2(gpu["traces"][c], ref[64]["obs"][c])
        floor = rel_l2(ref[32]["obs"][c], ref[64]["obs"][c])
        assert _agrees(e32, e64, floor, tol, cancel=c == 3), \
            f"trace comp {c}: rel L2 {e32:.2e} vs FP32 oracle (FP64: {e64:.2e}, FP32 oracle vs FP64 {floor:.2e})"
    for f, a in gpu["state"].items():
        e32 = rel_l2(a, ref[32]["state"][f])
        e64 = rel_l2(a, ref[64]["state"][f])
        floor = rel_l2(ref[32]["state"][f], ref[64]["state"][f])
        assert _agrees(e32, e64, floor, tol), \
            f"state {f}: rel L2 {e32:.2e} vs FP32 oracle (FP64: {e64:.2e}, FP32 oracle vs FP64 {floor:.2e})"


def _check_plain(gpu, ref, flags, tol=L2_TOL):
    """Plain 1e-5 against the FP32 oracle on every trace component and state
    field (the spin rotation yi aside, as in _agrees)."""
    for c in _comps(flags):
        e32 = rel_l2(gpu["traces"][c], ref[32]["obs"][c])
        floor = rel_l2(ref[32]["obs"][c], ref[64]["obs"][c])
        assert e32 <= (max(tol, 3 * floor) if c == 3 else tol), \
            f"trace comp {c}: rel L2 {e32:.2e} vs FP32 oracle (FP32 oracle vs FP64 {floor:.2e})"
    for f, a in gpu["state"].items():
        e32 = rel_l2(a, ref[32]["state"][f])
        assert e32 <= tol, f"state {f}: rel L2 {e32:.2e} vs FP32 oracle"


LOADERS = pytest.mark.parametrize("loader", [0, 1], ids=["direct", "bulk"])


@LOADERS
def test_sh_two_strips_all_tapers(loader):
    nx, nz, nt, dx = 64, 200, 150, 10.0
    flags = dict(sh=True, psv=False, abs_left=True, abs_right=True, abs_bottom=True, abs_top=True, abs_width=15)
    src = [(30, 100, 20.0, 0.05, 0.0), (31, 121, 15.0, 0.06, 0.0)]
    rec = [(0, 0), (1, 1), (2, 119), (5, 120), (63, 199), (62, 198), (32, 60)]
    gpu, ref = _run_pair(nx, nz, nt, dx, 1.5e-3, src, rec, _model(nx, nz, 1), chunk_rows=16, loader=loader, **flags)
    _check(gpu, ref, flags)


@LOADERS
def test_psv_narrow_grid_odd_chunks_no_graphs(loader):
    nx, nz, nt, dx = 150, 37, 160, 10.0
    flags = dict(psv=True, abs_left=True, abs_right=True, abs_bottom=True, abs_width=10)
    src = [(75, 18, 20.0, 0.05, 30.0)]
    rec = [(10, 0), (75, 2), (140, 36), (149, 35), (1, 1)]
    gpu, ref = _run_pair(nx, nz, nt, dx, 1.5e-3, src, rec, _model(nx, nz, 2), chunk_rows=7, graphs=0,
                         loader=loader, **flags)
    _check(gpu, ref, flags)


def test_psv_top_taper_three_strips():
    nx, nz, nt, dx = 41, 333, 140, 10.0
    flags = dict(psv=True, abs_top=True, abs_bottom=True, abs_width=20)
    src = [(20, 5, 18.0, 0.05, 90.0)]
    rec = [(i, 0) for i in range(0, 41, 5)] + [(20, 240), (20, 241)]
    gpu, ref = _run_pair(nx, nz, nt, dx, 1.5e-3, src, rec, _model(nx, nz, 3), chunk_rows=64, **flags)
    _check(gpu, ref, flags)


@LOADERS
def test_spin_receivers_near_edges(loader):
    nx, nz, nt, dx = 90, 130, 500, 1.0
    flags = dict(psv=True, spin=True)
    src = [(45, 60, 50.0, 0.024, 0.0)]  # t0 = 1.2/f0: the pulse fires within nt*dt = 0.05 s
    rec = [(0, 60), (1, 60), (88, 60), (87, 60), (45, 0), (45, 1), (45, 128), (45, 127), (60, 100)]
    gpu, ref = _run_pair(nx, nz, nt, dx, 1e-4, src, rec, _model(nx, nz, 4, spin=True), chunk_rows=24,
                         loader=loader, **flags)
    _check(gpu, ref, flags)


def test_sh_and_psv_together_odd_nz():
    nx, nz, nt, dx = 61, 251, 120, 10.0
    flags = dict(sh=True, psv=True, abs_left=True, abs_right=True, abs_width=8)
    src = [(30, 125, 20.0, 0.05, 45.0)]
    rec = [(30, 10), (10, 250), (60, 0)]
    gpu, ref = _run_pair(nx, nz, nt, dx, 1.5e-3, src, rec, _model(nx, nz, 5), **flags)
    _check(gpu, ref, flags)


@pytest.mark.parametrize("isrc", [-1, 0, 2])
def test_source_selection_and_colocated_sources(isrc):
    nx, nz, nt, dx = 48, 140, 120, 10.0
    flags = dict(sh=True, psv=True, abs_bottom=True)
    src = [(20, 70, 20.0, 0.05, 0.0), (20, 70, 12.0, 0.07, 60.0), (30, 121, 25.0, 0.04, 10.0)]
    rec = [(10, 10), (40, 130), (20, 71)]
    gpu, ref = _run_pair(nx, nz, nt, dx, 1.5e-3, src, rec, _model(nx, nz, 6), isrc=isrc, **flags)
    _check(gpu, ref, flags)


def test_snapshots_match_oracle_timing():
    nx, nz, nt, dx = 40, 130, 95, 10.0
    flags = dict(psv=True, spin=False, abs_left=True)
    src = [(20, 65, 20.0, 0.05, 0.0)]
    rec = [(5, 5)]
    gpu, ref = _run_pair(nx, nz, nt, dx, 1.5e-3, src, rec, _model(nx, nz, 7), snap=30, snap_fields=("vx", "vz"),
                         **flags)
    assert gpu["snaps"].shape == ref[32]["snaps"].shape == (3, 2, nx, nz)
    for q in range(3):
        for f in range(2):
            assert rel_l2(gpu["snaps"][q, f], ref[32]["snaps"][q, f]) <= L2_TOL


def test_reference_adjoint_and_smoothing():
    """Two shots of the reference adjoint (solver.rs:1380-1507) against the oracle."""
    import seiswg_gb300 as sw
    from oracle import oracle as O

    nx, nz, nt, dx, dt, adj, sigma = 70, 150, 200, 10.0, 1.5e-3, 10, 3.0
    flags = dict(sh=True, psv=False, abs_left=True, abs_right=True, abs_bottom=True, abs_width=12)
    src = [(20, 20, 20.0, 0.05, 0.0), (50, 20, 20.0, 0.05, 0.0)]
    rec = [(i, 30) for i in range(5, 66, 6)]
    si = np.array([s[0] for s in src], np.int32)
    sj = np.array([s[1] for s in src], np.int32)
    ri = np.array([r[0] for r in rec], np.int32)
    rj = np.array([r[1] for r in rec], np.int32)
    stf = np.stack([sw.ricker(nt, dt, s[2], s[3], s[4], 1.0e10) for s in src], axis=1)
    true = _model(nx, nz, 8)
    init = dict(vp=np.full((nx, nz), 3000.0), vs=np.full((nx, nz), 3000.0 / np.sqrt(3.0)),
                rho=np.full((nx, nz), 2500.0))
    s = O.Setup(nx, nz, nt, dx, dx, dt, **flags)
    # observed data from the true model (oracle)
    ot = O.FD2DOracle(s, si * nz + sj, stf.astype(np.float64), ri * nz + rj, 32)
    for k, v in true.items():
        ot.set_field(_ORACLE_SLOT[k], v)
    ot.init_model()
    obs = []
    for i in range(len(src)):
        ot.run_forward(i)
        obs.append(ot.obs("Y").astype(np.float32))
    obs = np.array(obs)
    # oracle adjoint
    oi = O.FD2DOracle(s, si * nz + sj, stf.astype(np.float64), ri * nz + rj, 32)
    for k, v in init.items():
        oi.set_field(_ORACLE_SLOT[k], v)
    oi.init_model()
    mis = oi.run_adjoint(np.arange(len(src)), obs, adj, sigma)
    ref_kmu = oi.field("K_MU")
    # GPU
    with sw.Sim(nx, nz, nt, dx, dx, dt, **flags) as sim:
        for k, v in init.items():
            sim.upload_model(k, v)
        sim.prepare()
        sim.set_sources(si, sj, stf)
        sim.set_receivers(ri, rj)
        sim.kernel_clear()
        gm = []
        for i in range(len(src)):
            sim.adjoint_forward(i, adj)
            syn = sim.traces()[1]
            m, adstf = sw.waveform_misfit(syn, obs[i], dt)
            gm.append(m)
            sim.adjoint_backward(adstf, adj)
        sim.kernel_smooth(sigma)
        kmu = sim.kernel()
    np.testing.assert_allclose(gm, mis, rtol=1e-5)
    assert rel_l2(kmu, ref_kmu) <= L2_TOL


@pytest.mark.parametrize("two_step", [1, 0], ids=["two_step", "one_step"])
def test_c2_geometry_plain_tolerance(two_step):
    """The headline workload's geometry at 512 x 480: PSV, absorbing width 40
    on every edge, a 90-degree Ricker 50 cells below the top, receivers on the
    top row and one at depth.  Traces and the final state within 1e-5 of the
    FP32 oracle, for the two-step kernel (the default) and the one-step one.

    The top row (j = 0) is decoupled from the grid by the edge rule (no z
    difference reaches it or leaves it, fd2d.wgsl:151-180), so its traces
    stay exactly zero; within 400 steps the deep receiver sees only the
    signal ahead of the first arrival, whose ux is subnormal in FP32 -- the
    most rounding-sensitive part of a trace."""
    nx, nz, nt, dx, dt = 512, 480, 400, 5.0, 4.0e-4
    flags = dict(psv=True, abs_left=True, abs_right=True, abs_bottom=True, abs_top=True, abs_width=40)
    src = [(256, 50, 15.0, 0.05, 90.0)]
    rec = [(i, 0) for i in range(0, 512, 32)] + [(256, 240)]
    gpu, ref = _run_pair(nx, nz, nt, dx, dt, src, rec, _model(nx, nz, 11, dx=dx), two_step=two_step, **flags)
    _check_plain(gpu, ref, flags)
    top = slice(0, 16)
    for c in (0, 2):
        assert not np.any(gpu["traces"][c][top]) and not np.any(ref[64]["obs"][c][top])
