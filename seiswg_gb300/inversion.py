"""Model-update loop around the exact gradient: the inversion workflow the
reference lists as planned (`mode = inversion`, README.md:61, main.rs:93-94).

Steepest descent in relative model units with a backtracking line search:

  s_p   = m_p * g_p / max_{p, cells} |m_p * g_p|     (p in the inverted parameters)
  m_p  <- m_p * (1 - alpha * s_p)                     (largest relative change = alpha)
  accept when J(m_new) <= J(m) + c1 * (g . (m_new - m))   (Armijo), else alpha *= shrink

`Descent` is the host logic (independent of the GPU: it only needs a misfit
function and a gradient function).  `ShotInversion` drives it for one problem
and its shots on the GPU: each gradient is the sum over shots of the exact
discrete adjoint (Sim.forward_op / Sim.backward_op, checkpointed), the misfit
is the L2 waveform misfit of solver.rs:432-467, and the chain rule to
(vp, vs, rho) is seiswg_velocity_gradients.  An optional Gaussian smoothing
of the gradients runs on the GPU (seiswg_smooth_noalloc).
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Callable, Dict, List, Optional, Sequence, Tuple

import numpy as np

Model = Dict[str, np.ndarray]


@dataclass
class StepRecord:
    iteration: int
    misfit: float            # J before the step
    new_misfit: float        # J after the step (== misfit when rejected)
    alpha: float             # accepted relative step (0 when rejected)
    trials: int              # misfit evaluations of the line search
    accepted: bool


def relative_direction(model: Model, grads: Model, params: Sequence[str]) -> Model:
    """s_p = m_p g_p / max |m g| over all inverted parameters and cells."""
    scale = max(float(np.abs(model[p].astype(np.float64) * grads[p]).max()) for p in params)
    if not scale > 0.0:
        return {p: np.zeros_like(model[p], dtype=np.float64) for p in params}
    return {p: model[p].astype(np.float64) * grads[p] / scale for p in params}


def apply_step(model: Model, s: Model, alpha: float) -> Model:
    out = dict(model)
    for p, sp in s.items():
        out[p] = (model[p].astype(np.float64) * (1.0 - alpha * sp)).astype(np.float32)
    return out


@dataclass
class Descent:
    evaluate: Callable[[Model], float]
    gradient: Callable[[Model], Tuple[float, Model]]
    params: Sequence[str] = ("vp", "vs")
    alpha0: float = 0.02
    shrink: float = 0.5
    grow: float = 1.5
    max_trials: int = 6
    c1: float = 1e-4
    alpha_max: float = 0.1
    history: List[StepRecord] = field(default_factory=list)

    def step(self, model: Model) -> Model:
        """One descent step from `model`; returns the (possibly unchanged) model."""
        J, g = self.gradient(model)
        s = relative_direction(model, g, self.params)
        alpha = min(self.alpha0, self.alpha_max)
        for trial in range(1, self.max_trials + 1):
            cand = apply_step(model, s, alpha)
            slope = sum(float((g[p] * (cand[p].astype(np.float64) - model[p])).sum()) for p in self.params)
            Jn = self.evaluate(cand)
            if np.isfinite(Jn) and Jn <= J + self.c1 * slope:
                self.history.append(StepRecord(len(self.history), J, Jn, alpha, trial, True))
                # next step starts a little larger after an acceptance at the first try
                self.alpha0 = min(alpha * (self.grow if trial == 1 else 1.0), self.alpha_max)
                return cand
            alpha *= self.shrink
        self.history.append(StepRecord(len(self.history), J, J, 0.0, self.max_trials, False))
        self.alpha0 = alpha
        return model

    def run(self, model: Model, iterations: int) -> Model:
        for _ in range(iterations):
            model = self.step(model)
        return model


class ShotInversion:
    """Inversion of one problem (a configs.Workload-like description: nx, nz,
    nt, dx, dz, dt, flags, sources, rec_i, rec_j, make_sim) over its shots.

    obs[s] are the observed traces of shot s, [ncomp][nrec][nt] in the
    receiver components of the physics (ux, uz for PSV; uy for SH)."""

    def __init__(self, workload, obs, params: Sequence[str] = ("vp", "vs"), smooth_sigma: float = 0.0,
                 **descent_kw):
        self.w = workload
        self.obs = [np.ascontiguousarray(o, np.float32) for o in obs]
        self.psv = bool(workload.flags.get("psv", True))
        self.comps = [0, 2] if self.psv else [1]
        self.sim = workload.make_sim()
        self.smooth_sigma = float(smooth_sigma)
        self.descent = Descent(self.evaluate, self.gradient, params=params, **descent_kw)
        self.evaluations = 0

    # -- model upload ---------------------------------------------------------
    def _upload(self, model: Model):
        for k in ("vp", "vs", "rho"):
            self.sim.upload_model(k, model[k])
        self.sim.prepare()

    # -- misfit and gradient ----------------------------------------------------
    def evaluate(self, model: Model) -> float:
        from . import l2_misfit

        self._upload(model)
        J = 0.0
        for s in range(len(self.w.sources)):
            self.sim.forward(s)
            J += l2_misfit(self.sim.traces()[self.comps], self.obs[s], self.w.dt)[0]
        self.evaluations += 1
        return J

    def gradient(self, model: Model) -> Tuple[float, Model]:
        from . import l2_misfit, velocity_gradients

        self._upload(model)
        self.sim.gradient_clear()
        J = 0.0
        for s in range(len(self.w.sources)):
            self.sim.forward_op(s, 0)
            Js, adj = l2_misfit(self.sim.traces()[self.comps], self.obs[s], self.w.dt)
            J += Js
            self.sim.backward_op(adj)
        g = {p: self.sim.gradient(p) for p in ("lambda", "mu", "buoyancy")}
        gvp, gvs, grho = velocity_gradients(g["lambda"], g["mu"], g["buoyancy"], model["vp"], model["vs"],
                                            model["rho"])
        out = {"vp": gvp, "vs": gvs, "rho": grho}
        if self.smooth_sigma > 0.0:
            out = {k: self._smooth(v) for k, v in out.items()}
        self.evaluations += 1
        return J, out

    def _smooth(self, a: np.ndarray) -> np.ndarray:
        import torch

        from . import smooth_noalloc

        src = torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()
        dst = torch.empty_like(src)
        smooth_noalloc(src.data_ptr(), dst.data_ptr(), a.shape[0], a.shape[1], self.smooth_sigma,
                       torch.cuda.current_stream().cuda_stream)
        torch.cuda.current_stream().synchronize()
        return dst.cpu().numpy()

    # -- driver -------------------------------------------------------------------
    def run(self, model: Optional[Model] = None, iterations: int = 5) -> Model:
        m = {k: np.ascontiguousarray(v, np.float32) for k, v in (model or self.w.model).items()}
        return self.descent.run(m, iterations)

    @property
    def history(self) -> List[StepRecord]:
        return self.descent.history

    def close(self):
        self.sim.close()
