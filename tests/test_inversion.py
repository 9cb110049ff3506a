"""Host logic of the inversion loop (seiswg_gb300.inversion.Descent) on
analytic misfits: relative steps, Armijo backtracking, rejection."""
import numpy as np

from seiswg_gb300.inversion import Descent, apply_step, relative_direction


def _quadratic(target, weight):
    def evaluate(m):
        return float(sum((weight[p] * (m[p].astype(np.float64) - target[p]) ** 2).sum() for p in target))

    def gradient(m):
        g = {p: 2.0 * weight[p] * (m[p].astype(np.float64) - target[p]) for p in target}
        return evaluate(m), g

    return evaluate, gradient


def test_relative_direction_scales_to_unit_max():
    m = {"vp": np.full((3, 4), 3000.0, np.float32), "vs": np.full((3, 4), 1700.0, np.float32)}
    g = {"vp": np.linspace(-1, 2, 12).reshape(3, 4), "vs": np.zeros((3, 4))}
    s = relative_direction(m, g, ("vp", "vs"))
    assert np.isclose(np.abs(s["vp"]).max(), 1.0) and not s["vs"].any()
    new = apply_step(m, s, 0.05)
    rel = np.abs(new["vp"] / m["vp"] - 1.0)
    assert np.isclose(rel.max(), 0.05, rtol=1e-5)
    zero = relative_direction(m, {"vp": np.zeros((3, 4)), "vs": np.zeros((3, 4))}, ("vp", "vs"))
    assert not zero["vp"].any()


def test_descent_decreases_a_quadratic_monotonically():
    rng = np.random.default_rng(0)
    target = {"vp": 3000 * (1 + 0.05 * rng.standard_normal((8, 9))), "vs": 1700 * (1 + 0.05 * rng.standard_normal((8, 9)))}
    weight = {"vp": np.full((8, 9), 1.0), "vs": np.full((8, 9), 3.0)}
    ev, gr = _quadratic(target, weight)
    d = Descent(ev, gr, params=("vp", "vs"), alpha0=0.2, alpha_max=0.2)
    m = {"vp": np.full((8, 9), 3000.0, np.float32), "vs": np.full((8, 9), 1700.0, np.float32)}
    J0 = ev(m)
    m = d.run(m, 25)
    Js = [h.new_misfit for h in d.history]
    assert all(b <= a for a, b in zip([J0] + Js, Js))
    assert Js[-1] < 0.2 * J0
    assert any(h.trials > 1 for h in d.history)       # a too-long first step was backtracked
    assert all(h.alpha <= 0.2 for h in d.history)


def test_descent_rejects_when_no_step_decreases():
    def evaluate(m):
        return 1.0 + float(np.abs(m["vp"] - 3000.0).sum())    # minimum at the start point

    def gradient(m):
        return evaluate(m), {"vp": np.ones_like(m["vp"], dtype=np.float64)}   # a wrong gradient

    d = Descent(evaluate, gradient, params=("vp",), alpha0=0.1, max_trials=3)
    m0 = {"vp": np.full((4, 4), 3000.0, np.float32)}
    m1 = d.step(m0)
    assert m1 is m0
    assert not d.history[-1].accepted and d.history[-1].trials == 3
    assert np.isclose(d.alpha0, 0.1 * 0.5 ** 3)
