"""The inversion loop on the GPU: a few descent steps on a small PSV problem
with three shots reduce the waveform misfit and move vp toward the anomaly of
the true model."""
import os

import numpy as np
import pytest

from seiswg_gb300 import configs

pytestmark = pytest.mark.gpu


def _problem():
    n, w = 140, 15
    dx = 10.0
    ii, jj = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    bump = (1.0 + 0.06 * np.exp(-((ii - n // 2) ** 2 + (jj - 45) ** 2) / 12.0 ** 2)).astype(np.float32)
    true = dict(vp=(3000.0 * bump).astype(np.float32), vs=(1732.0 * bump).astype(np.float32),
                rho=np.full((n, n), 2600.0, np.float32))
    init = dict(vp=np.full((n, n), 3000.0, np.float32), vs=np.full((n, n), 1732.0, np.float32),
                rho=np.full((n, n), 2600.0, np.float32))
    dt = float(np.float32(0.4 * dx / float(true["vp"].max())))
    flags = dict(sh=False, psv=True, abs_left=True, abs_right=True, abs_bottom=True, abs_top=True, abs_width=w,
                 abs_alpha=0.015)
    rec_i = np.arange(w, n - w, 3).astype(np.int32)
    srcs = [(int(i), w + 3, 25.0, 0.05, 0.0, 1.0e10) for i in (35, 70, 105)]
    return configs.Workload("inversion test", n, n, 900, dx, dx, dt, flags, init, srcs, rec_i,
                            np.full(rec_i.size, w, np.int32), dict(true_model=true)), true


def test_descent_reduces_misfit_and_finds_the_anomaly():
    from seiswg_gb300.inversion import ShotInversion

    W, true = _problem()
    sim = W.make_sim(model=true)
    obs = []
    for s in range(len(W.sources)):
        sim.forward(s)
        obs.append(sim.traces()[[0, 2]])
    sim.close()
    inv = ShotInversion(W, obs, params=("vp", "vs"), smooth_sigma=3.0, alpha0=0.01, alpha_max=0.03)
    try:
        m = inv.run(iterations=4)
    finally:
        inv.close()
    h = inv.history
    assert sum(r.accepted for r in h) >= 3
    Js = [h[0].misfit] + [r.new_misfit for r in h]
    assert all(b <= a for a, b in zip(Js, Js[1:]))
    assert Js[-1] < 0.8 * Js[0]
    dvp = m["vp"].astype(np.float64) - 3000.0
    ptrue = true["vp"].astype(np.float64) - 3000.0
    corr = float((dvp * ptrue).sum() / (np.linalg.norm(dvp) * np.linalg.norm(ptrue)))
    assert corr > 0.3, corr


def _write_model(d, nx, nz, dx, vp, vs, rho):
    from tests.examples import write_bin

    os.makedirs(d, exist_ok=True)
    x = np.repeat(np.arange(nx, dtype=np.float32) * np.float32(dx), nz)
    z = np.tile(np.arange(nz, dtype=np.float32) * np.float32(dx), nx)
    for name, a in (("x", x), ("z", z), ("vp", vp), ("vs", vs), ("rho", rho)):
        write_bin(os.path.join(d, f"proc000000_{name}.bin"), a)


def test_cli_inversion_lowers_the_misfit(tmp_path):
    """`mode = inversion` through the drop-in command line (the reference
    rejects it as not yet implemented, main.rs:93-94): observed traces from a
    forward run of the true model, then three descent steps from the
    homogeneous initial model; the misfit falls at every accepted step and
    the final model files are written."""
    import subprocess

    import seiswg_gb300 as sw

    W, true = _problem()
    d = str(tmp_path)
    n, dx = W.nx, W.dx
    _write_model(os.path.join(d, "model_true"), n, n, dx, true["vp"], true["vs"], true["rho"])
    _write_model(os.path.join(d, "model_init"), n, n, dx, W.model["vp"], W.model["vs"], W.model["rho"])
    with open(os.path.join(d, "sources.dat"), "w") as f:
        for (i, j, f0, t0, ang, amp) in W.sources:
            f.write(f"{i * dx} {j * dx} 0 {f0} {t0} {ang} {amp}\n")
    with open(os.path.join(d, "stations.dat"), "w") as f:
        for i, j in zip(W.rec_i, W.rec_j):
            f.write(f"{i * dx} {j * dx}\n")
    solver = (f"[solver]\nsh = no\npsv = yes\nnt = {W.nt}\ndt = {W.dt!r}\nabs_left = yes\nabs_right = yes\n"
              f"abs_bottom = yes\nabs_top = yes\nabs_width = {W.flags['abs_width']}\ncombine_sources = no\n")
    open(os.path.join(d, "forward.ini"), "w").write(
        "[workflow]\nmode = forward\n" + solver +
        "[path]\noutput = fwd\noutput_traces = obs\nmodel_true = model_true\nsources = sources.dat\n"
        "stations = stations.dat\n")
    open(os.path.join(d, "inversion.ini"), "w").write(
        "[workflow]\nmode = inversion\n" + solver +
        "[path]\noutput = inv\nmodel_init = model_init\nsources = sources.dat\nstations = stations.dat\n"
        "traces = obs\n[inversion]\niterations = 3\nparameters = vp, vs\nstep = 0.01\nmax_step = 0.03\n"
        "smooth = 3\n")
    for ini in ("forward.ini", "inversion.ini"):
        r = subprocess.run([sw.CLI_PATH, os.path.join(d, ini)], capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stderr[-3000:]
    rows = [ln.split() for ln in open(os.path.join(d, "inv", "inversion_misfit.txt")) if not ln.startswith("#")]
    J0, J1, acc = [float(r[1]) for r in rows], [float(r[2]) for r in rows], [int(r[5]) for r in rows]
    assert len(rows) >= 2 and sum(acc) >= 2, rows
    assert all(b < a for a, b, ok in zip(J0, J1, acc) if ok)
    assert J1[-1] < 0.9 * J0[0]
    vp = np.fromfile(os.path.join(d, "inv", "proc000000_vp.bin"), "<f4")
    assert int(vp[:1].view(np.int32)[0]) == n * n and vp.size == n * n + 1
    dvp = vp[1:].reshape(n, n).astype(np.float64) - 3000.0
    ptrue = true["vp"].astype(np.float64) - 3000.0
    assert float((dvp * ptrue).sum() / (np.linalg.norm(dvp) * np.linalg.norm(ptrue))) > 0.2
    for f in ("vs", "rho", "x", "z"):
        assert os.path.exists(os.path.join(d, "inv", f"proc000000_{f}.bin"))
