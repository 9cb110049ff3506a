"""TEST INFRASTRUCTURE ONLY -- ctypes front end of the CPU oracle.

`oracle/fd2d_oracle.cpp` restates seiswg's `shaders/fd2d.wgsl` and the
numeric parts of `src/solver.rs`; this module adds the host-side set-up the
reference performs before its time loop, restated in numpy:

* grid inference from the coordinate files      (solver.rs:646-656)
* source / station cell location                (solver.rs:709-719, 742-751)
* the Ricker STF table                           (solver.rs:350-356, 721-733)

Only tests/, the smoke check and the CPU-baseline leg of bench.py import
this.  The product never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")

# Field slots (fd2d.wgsl:53-105).
F = dict(
    VY=0, UY=1, SXY=2, SZY=3, DSY=4, DVYDX=5, DVYDZ=6,
    VX=7, VZ=8, UX=9, UZ=10, SXX=11, SZZ=12, SXZ=13, DSX=14, DSZ=15,
    DVXDX=16, DVXDZ=17, DVZDX=18, DVZDZ=19,
    VY_C=20, UY_C=21, SYX_C=22, SYY_C=23, SYZ_C=24, DSY_C=25, DVYDX_C=26, DVYDZ_C=27,
    DUZDX=28, DUXDZ=29,
    LAM=30, MU=31, NU=32, J=33, LAM_C=34, MU_C=35, NU_C=36, RHO=37, BOUND=38,
    K_LAM=39, K_MU=40, K_RHO=41, GSUM=42, GTMP=43,
)
# Observation components (fd2d.wgsl:110-114).
OBS = dict(X=0, Y=1, Z=2, YI=3, YC=4)


class OracleParams(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int32), ("nz", ctypes.c_int32), ("nt", ctypes.c_int32),
        ("dx", ctypes.c_double), ("dz", ctypes.c_double), ("dt", ctypes.c_double),
        ("sh", ctypes.c_int32), ("psv", ctypes.c_int32), ("spin", ctypes.c_int32),
        ("abs_left", ctypes.c_int32), ("abs_right", ctypes.c_int32),
        ("abs_bottom", ctypes.c_int32), ("abs_top", ctypes.c_int32),
        ("abs_width", ctypes.c_int32), ("abs_alpha", ctypes.c_double),
        ("nsrc", ctypes.c_int32), ("nrec", ctypes.c_int32),
    ]


_lib = None


def build():
    """Compile liboracle.so with the committed Makefile."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        vp, dp, ip = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int32)
        L.oracle_create.restype = vp
        L.oracle_create.argtypes = [ctypes.POINTER(OracleParams), ctypes.c_int]
        L.oracle_destroy.argtypes = [vp]
        for name in ("oracle_set_field", "oracle_get_field"):
            getattr(L, name).argtypes = [vp, ctypes.c_int, dp]
        L.oracle_set_sources.argtypes = [vp, ip, dp]
        L.oracle_set_receivers.argtypes = [vp, ip]
        for name in ("oracle_init_model", "oracle_clear_dynamic", "oracle_clear_obs"):
            getattr(L, name).argtypes = [vp]
        L.oracle_forward_step.argtypes = [vp, ctypes.c_int, ctypes.c_int]
        L.oracle_adjoint_step.argtypes = [vp, ctypes.c_int]
        L.oracle_imaging.argtypes = [vp, dp, ctypes.c_double]
        L.oracle_smooth.argtypes = [vp, ctypes.c_double]
        L.oracle_get_obs.argtypes = [vp, ctypes.c_int, dp]
        L.oracle_set_obs.argtypes = [vp, ctypes.c_int, dp]
        L.oracle_run_forward.restype = ctypes.c_int
        L.oracle_run_forward.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ip, dp]
        L.oracle_run_adjoint.restype = ctypes.c_int
        L.oracle_run_adjoint.argtypes = [vp, ctypes.c_int, ip, dp, ctypes.c_int, ctypes.c_double, dp]
        L.oracle_ricker_f32.argtypes = [ctypes.c_int] + [ctypes.c_float] * 5 + [ctypes.POINTER(ctypes.c_float)]
        L.oracle_ricker_f64.argtypes = [ctypes.c_int] + [ctypes.c_double] * 5 + [dp]
        L.oracle_misfit_f32.restype = ctypes.c_double
        L.oracle_misfit_f32.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                        ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float),
                                        ctypes.POINTER(ctypes.c_float)]
        L.oracle_num_threads.restype = ctypes.c_int
        L.oracle_exact_gradient.restype = ctypes.c_int
        L.oracle_exact_gradient.argtypes = [vp, ctypes.c_int, dp, dp, dp, dp]
        _lib = L
    return _lib


def _dptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _iptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))


def _fptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


# ---------------------------------------------------------------------------
# Host-side set-up restated from solver.rs
# ---------------------------------------------------------------------------

def round_half_away(x):
    """Rust's f32::round: halfway cases away from zero."""
    x = np.asarray(x)
    return np.sign(x) * np.floor(np.abs(x) + x.dtype.type(0.5))


def infer_grid(x, z):
    """solver.rs:646-656: nx, nz from the coordinate extents (f64 sqrt, f32 dx).
    The extents fold f32::max / f32::min from -/+infinity (solver.rs:647-650),
    which pass over NaN elements: nanmax / nanmin."""
    x = np.asarray(x, np.float32)
    z = np.asarray(z, np.float32)
    npt = x.size
    lx = np.float32(np.nanmax(x) - np.nanmin(x))
    lz = np.float32(np.nanmax(z) - np.nanmin(z))
    nx = int(round_half_away(np.float64(np.sqrt(np.float64(npt) * np.float64(lx) / np.float64(lz)))))
    nz = int(round_half_away(np.float64(np.sqrt(np.float64(npt) * np.float64(lz) / np.float64(lx)))))
    dx = np.float32(lx / np.float32(nx - 1))
    dz = np.float32(lz / np.float32(nz - 1))
    return nx, nz, float(dx), float(dz)


def locate(xs, zs, dx, dz, nz):
    """solver.rs:716-718 / 748-750: k = round(x/dx)*nz + round(z/dz), in f32."""
    xs = np.asarray(xs, np.float32)
    zs = np.asarray(zs, np.float32)
    ix = round_half_away(xs / np.float32(dx)).astype(np.int64)
    iz = round_half_away(zs / np.float32(dz)).astype(np.int64)
    return (ix * nz + iz).astype(np.int32)


def parse_table(text):
    """solver.rs:248-255: whitespace table, '#' comments, bad numbers -> 0."""
    rows = []
    for line in text.splitlines():
        t = line.strip()
        if not t or t.startswith("#"):
            continue
        row = []
        for tok in t.split():
            try:
                row.append(float(tok))
            except ValueError:
                row.append(0.0)
        rows.append(row)
    return rows


def source_params(rows):
    """solver.rs:709-715: (x, z, f0, t0, ang, amp) with the reference defaults."""
    out = []
    for r in rows:
        g = lambda i, d: r[i] if len(r) > i else d  # noqa: E731
        out.append((g(0, 0.0), g(1, 0.0), g(3, 10.0), g(4, 0.1), g(5, 0.0), g(6, 1.0e10)))
    return out


def ricker(nt, dt, f0, t0, ang, amp, precision=32):
    """[3][nt] STF (x, y, z) of one source, solver.rs:350-356."""
    L = lib()
    if precision == 32:
        out = np.zeros(3 * nt, np.float32)
        L.oracle_ricker_f32(nt, dt, f0, t0, ang, amp, _fptr(out))
    else:
        out = np.zeros(3 * nt, np.float64)
        L.oracle_ricker_f64(nt, dt, f0, t0, ang, amp, _dptr(out))
    return out.reshape(3, nt)


def stf_table(srcs, nt, dt, precision=32):
    """[3][nsrc][nt] table, solver.rs:721-733."""
    tab = np.zeros((3, len(srcs), nt), np.float64)
    for s, (_, _, f0, t0, ang, amp) in enumerate(srcs):
        tab[:, s, :] = ricker(nt, dt, f0, t0, ang, amp, precision)
    return tab


def misfit_f32(syn, ref, dt):
    syn = np.ascontiguousarray(syn, np.float32)
    ref = np.ascontiguousarray(ref, np.float32)
    nrec, nt = syn.shape
    ad = np.zeros_like(syn)
    m = lib().oracle_misfit_f32(nrec, nt, dt, _fptr(syn), _fptr(ref), _fptr(ad))
    return m, ad


# ---------------------------------------------------------------------------
# The stencil oracle
# ---------------------------------------------------------------------------

@dataclass
class Setup:
    nx: int
    nz: int
    nt: int
    dx: float
    dz: float
    dt: float
    sh: bool = False
    psv: bool = True
    spin: bool = False
    abs_left: bool = False
    abs_right: bool = False
    abs_bottom: bool = False
    abs_top: bool = False
    abs_width: int = 20
    abs_alpha: float = 0.015


class FD2DOracle:
    """One reference-layout solver instance (44 fields x npt) on the CPU."""

    def __init__(self, s: Setup, src_k, stf, rec_k, precision=32):
        self.s = s
        self.npt = s.nx * s.nz
        self.nsrc = len(src_k)
        self.nrec = len(rec_k)
        p = OracleParams(s.nx, s.nz, s.nt, s.dx, s.dz, s.dt, int(s.sh), int(s.psv), int(s.spin),
                         int(s.abs_left), int(s.abs_right), int(s.abs_bottom), int(s.abs_top),
                         int(s.abs_width), s.abs_alpha, self.nsrc, self.nrec)
        self._h = lib().oracle_create(ctypes.byref(p), precision)
        if not self._h:
            raise ValueError("oracle_create rejected the parameters")
        k = np.ascontiguousarray(src_k, np.int32)
        st = np.ascontiguousarray(stf, np.float64).reshape(-1)
        assert st.size == 3 * self.nsrc * s.nt
        lib().oracle_set_sources(self._h, _iptr(k), _dptr(st))
        r = np.ascontiguousarray(rec_k, np.int32)
        lib().oracle_set_receivers(self._h, _iptr(r))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().oracle_destroy(h)
            self._h = None

    def set_field(self, name, data):
        a = np.ascontiguousarray(data, np.float64).reshape(-1)
        assert a.size == self.npt
        lib().oracle_set_field(self._h, F[name], _dptr(a))

    def field(self, name):
        out = np.zeros(self.npt, np.float64)
        lib().oracle_get_field(self._h, F[name], _dptr(out))
        return out.reshape(self.s.nx, self.s.nz)

    def init_model(self):
        lib().oracle_init_model(self._h)

    def obs(self, comp):
        out = np.zeros(self.nrec * self.s.nt, np.float64)
        lib().oracle_get_obs(self._h, OBS[comp], _dptr(out))
        return out.reshape(self.nrec, self.s.nt)

    def set_obs(self, comp, data):
        a = np.ascontiguousarray(data, np.float64).reshape(-1)
        lib().oracle_set_obs(self._h, OBS[comp], _dptr(a))

    def forward_step(self, it, isrc=-1):
        lib().oracle_forward_step(self._h, it, isrc)

    def adjoint_step(self, it):
        lib().oracle_adjoint_step(self._h, it)

    def imaging(self, fw, ndt):
        a = np.ascontiguousarray(fw, np.float64).reshape(-1)
        lib().oracle_imaging(self._h, _dptr(a), ndt)

    def smooth(self, sigma):
        lib().oracle_smooth(self._h, sigma)

    def clear_dynamic(self):
        lib().oracle_clear_dynamic(self._h)

    def run_forward(self, isrc=-1, snap_every=0, snap_fields=()):
        s = self.s
        nsnap = 0
        if snap_every > 0:
            nsnap = sum(1 for it in range(1, s.nt) if it % snap_every == 0)
        fids = np.array([F[n] for n in snap_fields], np.int32)
        snaps = np.zeros(max(1, nsnap * len(fids) * self.npt), np.float64)
        n = lib().oracle_run_forward(self._h, isrc, snap_every, len(fids), _iptr(fids), _dptr(snaps))
        assert n == nsnap
        return snaps[: nsnap * len(fids) * self.npt].reshape(nsnap, len(fids), s.nx, s.nz)

    def run_adjoint(self, run_isrc, obs_y, adj_interval=10, sigma=5.0):
        runs = np.ascontiguousarray(run_isrc, np.int32)
        o = np.ascontiguousarray(obs_y, np.float64).reshape(-1)
        assert o.size == len(runs) * self.nrec * self.s.nt
        mis = np.zeros(len(runs), np.float64)
        rc = lib().oracle_run_adjoint(self._h, len(runs), _iptr(runs), _dptr(o), adj_interval, sigma, _dptr(mis))
        if rc != 0:
            raise ValueError("adj_interval >= nt")
        return mis


    def exact_gradient(self, adj, isrc=-1):
        """(g_lambda, g_mu, g_buoyancy) of J for the adjoint source `adj` = dJ/dd
        ([2][nrec][nt] ux, uz for PSV; [1][nrec][nt] uy for SH)."""
        a = np.ascontiguousarray(adj, np.float64).reshape(-1)
        gl = np.zeros(self.npt)
        gm = np.zeros(self.npt)
        gb = np.zeros(self.npt)
        rc = lib().oracle_exact_gradient(self._h, isrc, _dptr(a), _dptr(gl), _dptr(gm), _dptr(gb))
        if rc != 0:
            raise ValueError("exact gradient is defined for SH or PSV without spin")
        shp = (self.s.nx, self.s.nz)
        return gl.reshape(shp), gm.reshape(shp), gb.reshape(shp)


def misfit_taper(nt, dt):
    """The cosine taper of solver.rs:442-459, in float64."""
    t = np.arange(nt) * dt
    t_end = (nt - 1) * dt
    tw = t_end / 10.0
    tau = np.ones(nt)
    lo, hi = t <= tw, t >= t_end - tw
    tau[lo] = 0.5 + 0.5 * np.cos(np.pi * (tw - t[lo]) / tw)
    tau[hi] = 0.5 + 0.5 * np.cos(np.pi * ((t_end - tw) - t[hi]) / tw)
    return tau


def l2_misfit(syn, obs, dt):
    """J = sum (taper * (syn - obs))^2 over traces and samples, and dJ/dsyn."""
    tau = misfit_taper(syn.shape[-1], dt)
    d = (np.asarray(syn, np.float64) - np.asarray(obs, np.float64)) * tau
    return float((d * d).sum()), 2.0 * d * tau


def lame_to_velocity_gradients(g_lam, g_mu, g_b, vp, vs, rho):
    """Chain rule through lambda = rho (vp^2 - 2 vs^2) (0 where vp <= vs),
    mu = rho vs^2, B = 1/rho (fd2d.wgsl:188-201)."""
    vp, vs, rho = (np.asarray(a, np.float64) for a in (vp, vs, rho))
    live = vp > vs
    g_vp = np.where(live, g_lam * 2.0 * rho * vp, 0.0)
    g_vs = np.where(live, g_lam * (-4.0 * rho * vs), 0.0) + g_mu * 2.0 * rho * vs
    g_rho = np.where(live, g_lam * (vp * vp - 2.0 * vs * vs), 0.0) + g_mu * vs * vs - g_b / (rho * rho)
    return g_vp, g_vs, g_rho


def num_threads():
    return lib().oracle_num_threads()
