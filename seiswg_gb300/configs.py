"""Seeded synthetic workloads of the five benchmark configurations.

The reference generates its example models with src/bin/gen_model.rs; the
benchmark configurations are larger and synthetic, so they are generated
here, in the reference's conventions (k = i*nz + j, vp/vs/rho or Lame
fields, Ricker sources):

  c1  SH forward 200 x 200, homogeneous, the size of the reference's example
  c2  PSV forward 4096 x 4096, vp gradient + Gaussian-filtered perturbation
  c3  PSV + micropolar spin 2048 x 2048, homogeneous Cosserat medium
  c4  PSV adjoint gradient 2048 x 2048, 8 shots, Gaussian anomaly (true model)
  c5  48 independent problems of uneven size, SH or PSV, 1-4 shots each

Every random draw uses numpy.random.default_rng(seed).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Dict, List, Tuple

import numpy as np


@dataclass
class Workload:
    name: str
    nx: int
    nz: int
    nt: int
    dx: float
    dz: float
    dt: float
    flags: Dict[str, object]
    model: Dict[str, np.ndarray]
    sources: List[Tuple[int, int, float, float, float, float]]  # (i, j, f0, t0, ang, amp)
    rec_i: np.ndarray
    rec_j: np.ndarray
    extra: Dict[str, object] = field(default_factory=dict)

    @property
    def cells(self) -> int:
        return self.nx * self.nz

    def stf(self):
        """[3][nsrc][nt] Ricker table (solver.rs:721-733)."""
        from . import ricker

        return np.stack([ricker(self.nt, self.dt, f0, t0, ang, amp) for (_, _, f0, t0, ang, amp) in self.sources],
                        axis=1)

    def make_sim(self, model=None, **options):
        """A seiswg_gb300.Sim with the model, sources and receivers uploaded."""
        from . import Sim

        sim = Sim(self.nx, self.nz, self.nt, self.dx, self.dz, self.dt, **self.flags)
        for k, v in options.items():
            sim.set_option(k, v)
        for k, v in (model or self.model).items():
            sim.upload_model(k, v)
        sim.prepare()
        sim.set_sources([s[0] for s in self.sources], [s[1] for s in self.sources], self.stf())
        sim.set_receivers(self.rec_i, self.rec_j)
        return sim


def _f32(a):
    return np.ascontiguousarray(a, np.float32)


def _elastic(vp, rho=None):
    vp = _f32(vp)
    vs = _f32(vp / np.float32(math.sqrt(3.0)))
    rho = _f32(np.float32(310.0) * vp ** np.float32(0.25)) if rho is None else _f32(rho)
    return dict(vp=vp, vs=vs, rho=rho)


def gradient_model(nx, nz, dz, rng, amp=0.05, sigma=20.0, background_only=False):
    """vp = 2000 + 600 * depth_km, times (1 + p) with p a Gaussian-filtered
    random field scaled to max |p| = amp."""
    depth_km = (np.arange(nz, dtype=np.float32) * np.float32(dz) / np.float32(1000.0))[None, :]
    vp = np.float32(2000.0) + np.float32(600.0) * depth_km + np.zeros((nx, 1), np.float32)
    if not background_only:
        from scipy.ndimage import gaussian_filter

        p = gaussian_filter(rng.standard_normal((nx, nz)).astype(np.float32), sigma)
        p *= np.float32(amp / np.abs(p).max())
        vp = vp * (np.float32(1.0) + p)
    return vp.astype(np.float32)


def c1_sh_forward() -> Workload:
    nx = nz = 200
    dx = 10.0
    n = (nx, nz)
    model = dict(vp=np.full(n, 3000.0, np.float32), vs=np.full(n, 1732.0, np.float32),
                 rho=np.full(n, 2600.0, np.float32))
    xs = np.linspace(100.0, 1900.0, 25)
    rec_i = np.floor(xs / dx + 0.5).astype(np.int32)   # round half away (solver.rs:748)
    rec_j = np.full(25, 20, np.int32)                   # z = 200 m
    flags = dict(sh=True, psv=False, abs_left=True, abs_right=True, abs_bottom=True, abs_top=True, abs_width=20,
                 abs_alpha=0.015)
    return Workload("c1: SH forward 200x200 homogeneous, nt=1000", nx, nz, 1000, dx, dx, 1e-3, flags, model,
                    [(100, 100, 10.0, 0.12, 0.0, 1.0e10)], rec_i, rec_j, dict(snap_every=100))


def c2_psv_forward(nx=4096, nz=4096, nt=4000, seed=0) -> Workload:
    dx = 5.0
    rng = np.random.default_rng(seed)
    vp = gradient_model(nx, nz, dx, rng)
    model = _elastic(vp)
    dt = float(np.float32(0.3 * dx / float(vp.max())))
    w = 40
    rec_i = np.round(np.linspace(0, nx - 1, 256)).astype(np.int32)
    flags = dict(sh=False, psv=True, abs_left=True, abs_right=True, abs_bottom=True, abs_top=True, abs_width=w,
                 abs_alpha=0.015)
    return Workload(f"c2: PSV forward heterogeneous {nx}x{nz}, nt={nt}", nx, nz, nt, dx, dx, dt, flags, model,
                    [(nx // 2, w + 10, 15.0, 0.1, 90.0, 1.0e10)], rec_i, np.zeros(256, np.int32))


def c3_spin_forward(n=2048, nt=3000) -> Workload:
    dx = 5.0
    rho, lam = 2000.0, 4.5e9
    mu, nu = lam, 0.05 * lam
    jj = rho * (0.5 * dx) ** 2
    cc = 0.1 * mu * dx * dx
    vp = math.sqrt((lam + 2 * mu) / rho)
    dt = 0.25 * dx / vp
    # Stability check before the run: P-wave CFL, rotational frequency, couple-wave speed.
    omega0 = math.sqrt(4.0 * nu / jj)
    v_couple = math.sqrt((cc + cc) / jj)
    assert vp * dt / dx <= 0.3 and omega0 * dt < 1.0 and v_couple * dt / dx <= 0.3
    shape = (n, n)
    full = lambda v: np.full(shape, v, np.float32)  # noqa: E731
    model = {"rho": full(rho), "lambda": full(lam), "mu": full(mu), "nu": full(nu), "j": full(jj),
             "lambda_c": full(cc), "mu_c": full(cc), "nu_c": full(cc)}
    w = 30
    rec_i = np.round(np.linspace(w, n - 1 - w, 64)).astype(np.int32)
    flags = dict(sh=False, psv=True, spin=True, abs_left=True, abs_right=True, abs_bottom=True, abs_top=True,
                 abs_width=w, abs_alpha=0.015)
    return Workload(f"c3: PSV + spin {n}x{n} homogeneous, nt={nt}", n, n, nt, dx, dx, float(np.float32(dt)), flags,
                    model, [(n // 2, n // 2, 12.0, 1.2 / 12.0, 45.0, 1.0e10)], rec_i, np.full(64, n // 2, np.int32),
                    dict(stability=dict(cfl=vp * dt / dx, omega0_dt=omega0 * dt, couple_cfl=v_couple * dt / dx)))


def c4_psv_adjoint(n=2048, nt=3000, shots=8) -> Workload:
    """True model: homogeneous with a +10 % vp/vs Gaussian anomaly of radius 40
    cells, placed at depth nz/4 so that the top receivers see it within nt
    steps (a centred anomaly at 5.1 km depth is not illuminated in 3000 steps
    at any stable dt); initial model homogeneous."""
    dx = 5.0
    w = 20
    ii, jj = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    r2 = (ii - n // 2) ** 2 + (jj - n // 4) ** 2
    bump = (1.0 + 0.1 * np.exp(-r2 / 40.0 ** 2)).astype(np.float32)
    true = dict(vp=_f32(3000.0 * bump), vs=_f32(1732.0 * bump), rho=np.full((n, n), 2600.0, np.float32))
    init = dict(vp=np.full((n, n), 3000.0, np.float32), vs=np.full((n, n), 1732.0, np.float32),
                rho=np.full((n, n), 2600.0, np.float32))
    dt = float(np.float32(0.45 * dx / float(true["vp"].max())))
    src_i = np.round(np.linspace(w + 10, n - 1 - w - 10, shots)).astype(int)
    rec_i = np.round(np.linspace(0, n - 1, 256)).astype(np.int32)
    flags = dict(sh=False, psv=True, abs_left=True, abs_right=True, abs_bottom=True, abs_top=True, abs_width=w,
                 abs_alpha=0.015)
    return Workload(f"c4: PSV adjoint {n}x{n}, {shots} shots, nt={nt}", n, n, nt, dx, dx, dt, flags, init,
                    [(int(i), w + 5, 12.0, 0.1, 0.0, 1.0e10) for i in src_i], rec_i, np.full(256, w, np.int32),
                    dict(true_model=true, smooth_sigma=5.0))


def c5_batch(seed=0, count=48, lo=256, hi=1536, nt_lo=1000, nt_hi=3000) -> List[Workload]:
    """Independent problems: nx, nz ~ U[lo, hi], nt ~ U[nt_lo, nt_hi], SH or
    PSV 50/50, 1-4 shots near the top, 32-128 receivers on the line j = w;
    true model from the c2 generator, initial model its smooth background."""
    rng = np.random.default_rng(seed)
    out = []
    dx = 5.0
    for p in range(count):
        nx, nz = (int(v) for v in rng.integers(lo, hi + 1, 2))
        nt = int(rng.integers(nt_lo, nt_hi + 1))
        sh = bool(rng.integers(0, 2))
        nshot = int(rng.integers(1, 5))
        nrec = int(rng.integers(32, 129))
        w = 20
        true_vp = gradient_model(nx, nz, dx, rng)
        init_vp = gradient_model(nx, nz, dx, rng, background_only=True)
        true, init = _elastic(true_vp), _elastic(init_vp)
        dt = float(np.float32(0.4 * dx / float(true_vp.max())))
        src_i = np.round(np.linspace(w + 5, nx - 1 - w - 5, nshot + 2)[1:-1]).astype(int)
        rec_i = np.round(np.linspace(w, nx - 1 - w, nrec)).astype(np.int32)
        flags = dict(sh=sh, psv=not sh, abs_left=True, abs_right=True, abs_bottom=True, abs_top=True, abs_width=w,
                     abs_alpha=0.015)
        out.append(Workload(f"c5[{p}]: {'SH' if sh else 'PSV'} {nx}x{nz}, nt={nt}, {nshot} shots", nx, nz, nt, dx,
                            dx, dt, flags, init, [(int(i), w + 5, 15.0, 0.1, 0.0, 1.0e10) for i in src_i], rec_i,
                            np.full(nrec, w, np.int32), dict(true_model=true)))
    return out
