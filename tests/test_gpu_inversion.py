"""The inversion loop on the GPU: a few descent steps on a small PSV problem
with three shots reduce the waveform misfit and move vp toward the anomaly of
the true model."""
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
