"""seiswg_gb300 -- Python binding of the GB300 (sm_103a) seiswg engine.

A thin ctypes layer over the C ABI in include/seiswg.h, which is what the
reference's host API (Rust) would bind over FFI.  Everything numeric runs in
libseiswg.so: CUDA kernels for the stencil, C++ for the host workflows.  If
the library has not been built, importing this package still works but every
call raises `SeiswgError` (there is no fallback implementation).

    cfg = Config.load("examples/forward/config.ini")
    with Solver(cfg) as s:
        out = s.run_forward()          # dict path -> bytes, like the reference's Vfs
"""
from __future__ import annotations

import ctypes
import os
from typing import Dict, Iterable, Optional, Sequence

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libseiswg.so")
CLI_PATH = os.path.join(_HERE, "_lib", "seiswg")

OK, EINVAL, EIO, ECUDA, EINTERNAL, ENUMERIC, ETIMEOUT = 0, 1, 2, 3, 4, 5, 6
OBS_X, OBS_Y, OBS_Z, OBS_YI, OBS_YC = range(5)


class SeiswgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"[{code}] {msg}")
        self.code = code


class SimDesc(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int32), ("nz", ctypes.c_int32), ("nt", ctypes.c_int32),
        ("dx", ctypes.c_float), ("dz", ctypes.c_float), ("dt", ctypes.c_float),
        ("sh", ctypes.c_int32), ("psv", ctypes.c_int32), ("spin", ctypes.c_int32),
        ("abs_left", ctypes.c_int32), ("abs_right", ctypes.c_int32),
        ("abs_bottom", ctypes.c_int32), ("abs_top", ctypes.c_int32),
        ("abs_width", ctypes.c_int32), ("abs_alpha", ctypes.c_float),
    ]


_lib = None

# (name, restype, argtypes) for every symbol of include/seiswg.h.
_c_int, _vp, _sz, _i32, _f32 = ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int32, ctypes.c_float
_pf = ctypes.POINTER(ctypes.c_float)
_pi = ctypes.POINTER(ctypes.c_int32)
_cp = ctypes.c_char_p
PROTOTYPES = [
    ("seiswg_last_error", _cp, []),
    ("seiswg_version", _cp, []),
    ("seiswg_vfs_new", _vp, []),
    ("seiswg_vfs_free", None, [_vp]),
    ("seiswg_vfs_insert", _c_int, [_vp, _cp, _vp, _sz]),
    ("seiswg_vfs_get", _c_int, [_vp, _cp, ctypes.POINTER(_vp), ctypes.POINTER(_sz)]),
    ("seiswg_vfs_size", _sz, [_vp]),
    ("seiswg_vfs_key", _cp, [_vp, _sz]),
    ("seiswg_config_load", _c_int, [_cp, ctypes.POINTER(_vp)]),
    ("seiswg_config_load_str", _c_int, [_cp, _cp, ctypes.POINTER(_vp)]),
    ("seiswg_config_free", None, [_vp]),
    ("seiswg_config_get", _c_int, [_vp, _cp, ctypes.c_char_p, _sz]),
    ("seiswg_solver_new", _c_int, [_vp, _vp, ctypes.POINTER(_vp)]),
    ("seiswg_solver_set_write_files", _c_int, [_vp, _c_int]),
    ("seiswg_solver_run_forward", _c_int, [_vp, _vp]),
    ("seiswg_solver_run_adjoint", _c_int, [_vp, _vp, _vp]),
    ("seiswg_solver_run_inversion", _c_int, [_vp, _vp, _vp]),
    ("seiswg_solver_info", _c_int, [_vp, _pi, _pi, _pf, _pf, _pi, _pi]),
    ("seiswg_solver_total_misfit", ctypes.c_double, [_vp]),
    ("seiswg_solver_sim", _vp, [_vp]),
    ("seiswg_solver_free", None, [_vp]),
    ("seiswg_sim_create", _c_int, [ctypes.POINTER(SimDesc), _vp, ctypes.POINTER(_vp)]),
    ("seiswg_sim_free", None, [_vp]),
    ("seiswg_sim_upload_model", _c_int, [_vp, _cp, _pf, _sz]),
    ("seiswg_sim_prepare", _c_int, [_vp]),
    ("seiswg_sim_stability", _c_int, [_vp, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]),
    ("seiswg_sim_set_sources", _c_int, [_vp, _i32, _pi, _pi, _pf]),
    ("seiswg_sim_set_receivers", _c_int, [_vp, _i32, _pi, _pi]),
    ("seiswg_sim_forward", _c_int, [_vp, _i32, _i32, _i32, ctypes.POINTER(_cp), _pf, _i32]),
    ("seiswg_sim_traces", _c_int, [_vp, _pf]),
    ("seiswg_sim_state", _c_int, [_vp, _cp, _pf]),
    ("seiswg_sim_kernel_clear", _c_int, [_vp]),
    ("seiswg_sim_adjoint_forward", _c_int, [_vp, _i32, _i32]),
    ("seiswg_sim_adjoint_backward", _c_int, [_vp, _pf, _i32]),
    ("seiswg_sim_kernel_smooth", _c_int, [_vp, _f32]),
    ("seiswg_sim_kernel", _c_int, [_vp, _pf]),
    ("seiswg_sim_gradient_clear", _c_int, [_vp]),
    ("seiswg_sim_forward_op", _c_int, [_vp, _i32, _i32]),
    ("seiswg_sim_backward_op", _c_int, [_vp, _pf]),
    ("seiswg_sim_checkpoint_interval", _i32, [_vp]),
    ("seiswg_sim_checkpoint_plan", _c_int, [_vp, _pi, _pi, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(_sz)]),
    ("seiswg_sim_set_observed", _c_int, [_vp, _pf]),
    ("seiswg_sim_misfit_op", _c_int, [_vp, ctypes.POINTER(ctypes.c_double)]),
    ("seiswg_sim_backward_op_device", _c_int, [_vp]),
    ("seiswg_sim_gradient", _c_int, [_vp, _cp, _pf]),
    ("seiswg_sim_release_workspace", _c_int, [_vp]),
    ("seiswg_sim_set_option", _c_int, [_vp, _cp, ctypes.c_int64]),
    ("seiswg_sim_synchronize", _c_int, [_vp]),
    ("seiswg_sim_launches", ctypes.c_uint64, [_vp]),
    ("seiswg_sim_stream", _vp, [_vp]),
    ("seiswg_sim_device_bytes", _sz, [_vp]),
    ("seiswg_ricker", _c_int, [_i32, _f32, _f32, _f32, _f32, _f32, _pf]),
    ("seiswg_waveform_misfit", _c_int, [_pf, _pf, _i32, _i32, _f32, _pf, ctypes.POINTER(ctypes.c_double)]),
    ("seiswg_npy_encode", _c_int, [_pf, _sz, _sz, _vp, ctypes.POINTER(_sz)]),
    ("seiswg_infer_grid", _c_int, [_pf, _pf, _sz, _pi, _pi, _pf, _pf]),
    ("seiswg_smooth_noalloc", _c_int, [_vp, _vp, _i32, _i32, _f32, _vp]),
    ("seiswg_batch_create", _c_int, [ctypes.POINTER(_vp), ctypes.POINTER(_pf), _i32, _i32, _vp, ctypes.POINTER(_vp)]),
    ("seiswg_batch_run", _c_int, [_vp]),
    ("seiswg_batch_set_option", _c_int, [_vp, _cp, ctypes.c_int64]),
    ("seiswg_batch_chunk_rows", _i32, [_vp]),
    ("seiswg_batch_two_step", _i32, [_vp]),
    ("seiswg_batch_concurrent", _i32, [_vp]),
    ("seiswg_batch_stream_groups", _i32, [_vp]),
    ("seiswg_batch_tma_jobs", _i32, [_vp]),
    ("seiswg_batch_queue", _i32, [_vp, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(_i32), ctypes.POINTER(_i32)]),
    ("seiswg_batch_checkpoint_plan", _c_int, [_vp, _pi, ctypes.POINTER(ctypes.c_int64)]),
    ("seiswg_batch_gradient", _c_int, [_vp, _i32, _cp, _pf]),
    ("seiswg_batch_misfit", ctypes.c_double, [_vp, _i32]),
    ("seiswg_batch_info", _c_int, [_vp, _pi, _pi, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(_sz)]),
    ("seiswg_batch_stream", _vp, [_vp]),
    ("seiswg_batch_free", None, [_vp]),
    ("seiswg_l2_misfit", _c_int, [_pf, _pf, _i32, _i32, _f32, _pf, ctypes.POINTER(ctypes.c_double)]),
    ("seiswg_velocity_gradients", _c_int, [_pf, _pf, _pf, _pf, _pf, _pf, _sz, _pf, _pf, _pf]),
]


def lib():
    """The loaded libseiswg.so; raises SeiswgError when it was never built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise SeiswgError(EINTERNAL, f"{LIB_PATH} is missing: build it with "
                                         "`python -m seiswg_gb300.build` (no CPU fallback exists)")
        L = ctypes.CDLL(LIB_PATH)
        for name, res, args in PROTOTYPES:
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _check(rc):
    if rc != OK:
        raise SeiswgError(rc, lib().seiswg_last_error().decode(errors="replace"))


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _fp(a):
    return a.ctypes.data_as(_pf)


def _ip(a):
    return a.ctypes.data_as(_pi)


# ---------------------------------------------------------------------------
# VFS, config, solver (the reference's host API)
# ---------------------------------------------------------------------------

class Vfs:
    """`Vfs = HashMap<String, Vec<u8>>` (solver.rs:15) held in the library."""

    def __init__(self, entries: Optional[Dict[str, bytes]] = None):
        self._h = lib().seiswg_vfs_new()
        for k, v in (entries or {}).items():
            self[k] = v

    def __setitem__(self, key: str, data: bytes):
        b = bytes(data)
        _check(lib().seiswg_vfs_insert(self._h, key.encode(), b, len(b)))

    def __getitem__(self, key: str) -> bytes:
        p, n = _vp(), _sz()
        _check(lib().seiswg_vfs_get(self._h, key.encode(), ctypes.byref(p), ctypes.byref(n)))
        return ctypes.string_at(p, n.value) if n.value else b""

    def keys(self):
        return [lib().seiswg_vfs_key(self._h, i).decode() for i in range(lib().seiswg_vfs_size(self._h))]

    def to_dict(self) -> Dict[str, bytes]:
        return {k: self[k] for k in self.keys()}

    def __len__(self):
        return lib().seiswg_vfs_size(self._h)

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.seiswg_vfs_free(self._h)
            self._h = None


class Config:
    """config::Config (config.rs:53-57); only parsed values are exposed."""

    def __init__(self, handle):
        self._h = handle

    @classmethod
    def load(cls, path: str) -> "Config":
        h = _vp()
        _check(lib().seiswg_config_load(path.encode(), ctypes.byref(h)))
        return cls(h)

    @classmethod
    def from_str(cls, text: str, base_dir: str = "") -> "Config":
        h = _vp()
        _check(lib().seiswg_config_load_str(text.encode(), base_dir.encode(), ctypes.byref(h)))
        return cls(h)

    def get(self, key: str) -> str:
        buf = ctypes.create_string_buffer(4096)
        _check(lib().seiswg_config_get(self._h, key.encode(), buf, len(buf)))
        return buf.value.decode()

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.seiswg_config_free(self._h)
            self._h = None


class Solver:
    """Solver (solver.rs:194): new / run_forward / run_adjoint."""

    def __init__(self, cfg: Config, vfs: Optional[Vfs] = None, write_files: bool = True):
        h = _vp()
        _check(lib().seiswg_solver_new(cfg._h, vfs._h if vfs else None, ctypes.byref(h)))
        self._h = h
        self._cfg = cfg
        _check(lib().seiswg_solver_set_write_files(h, int(write_files)))

    def run_forward(self) -> Dict[str, bytes]:
        out = Vfs()
        _check(lib().seiswg_solver_run_forward(self._h, out._h))
        return out.to_dict()

    def run_adjoint(self, vfs: Optional[Vfs] = None) -> Dict[str, bytes]:
        out = Vfs()
        _check(lib().seiswg_solver_run_adjoint(self._h, vfs._h if vfs else None, out._h))
        return out.to_dict()

    def run_inversion(self, vfs: Optional[Vfs] = None) -> Dict[str, bytes]:
        """`mode = inversion` (seiswg_solver_run_inversion): the final model
        files and inversion_misfit.txt."""
        out = Vfs()
        _check(lib().seiswg_solver_run_inversion(self._h, vfs._h if vfs else None, out._h))
        return out.to_dict()

    def info(self):
        nx, nz, nsrc, nrec = _i32(), _i32(), _i32(), _i32()
        dx, dz = ctypes.c_float(), ctypes.c_float()
        _check(lib().seiswg_solver_info(self._h, ctypes.byref(nx), ctypes.byref(nz), ctypes.byref(dx),
                                        ctypes.byref(dz), ctypes.byref(nsrc), ctypes.byref(nrec)))
        return dict(nx=nx.value, nz=nz.value, dx=dx.value, dz=dz.value, nsrc=nsrc.value, nrec=nrec.value)

    @property
    def total_misfit(self) -> float:
        return lib().seiswg_solver_total_misfit(self._h)

    @property
    def sim(self) -> "Sim":
        return Sim._borrowed(lib().seiswg_solver_sim(self._h), self)

    def close(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.seiswg_solver_free(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        self.close()


# ---------------------------------------------------------------------------
# Simulation operator (kernel-level interface)
# ---------------------------------------------------------------------------

class Sim:
    """One simulation on the GPU: model, sources, receivers, wavefield."""

    def __init__(self, nx, nz, nt, dx, dz, dt, sh=False, psv=True, spin=False, abs_left=False,
                 abs_right=False, abs_bottom=False, abs_top=False, abs_width=20, abs_alpha=0.015,
                 stream=None):
        d = SimDesc(nx, nz, nt, dx, dz, dt, int(sh), int(psv), int(spin), int(abs_left), int(abs_right),
                    int(abs_bottom), int(abs_top), int(abs_width), abs_alpha)
        h = _vp()
        _check(lib().seiswg_sim_create(ctypes.byref(d), stream, ctypes.byref(h)))
        self._h, self._owner = h, None
        self.nx, self.nz, self.nt = nx, nz, nt
        self.sh, self.psv, self.spin = sh, psv, spin
        self.nrec = 0

    @classmethod
    def _borrowed(cls, handle, owner):
        s = cls.__new__(cls)
        s._h, s._owner = handle, owner
        info = owner.info()
        s.nx, s.nz = info["nx"], info["nz"]
        s.nt = int(owner._cfg.get("solver.nt"))
        s.nrec = info["nrec"]
        return s

    def upload_model(self, name: str, data):
        a = _f32(data).reshape(-1)
        _check(lib().seiswg_sim_upload_model(self._h, name.encode(), _fp(a), a.size))

    def prepare(self):
        _check(lib().seiswg_sim_prepare(self._h))

    def stability(self):
        """(wave, spin) stability numbers of the last prepare(); above 1 is unstable."""
        w, s = ctypes.c_double(), ctypes.c_double()
        _check(lib().seiswg_sim_stability(self._h, ctypes.byref(w), ctypes.byref(s)))
        return w.value, s.value

    def set_sources(self, i: Sequence[int], j: Sequence[int], stf_xyz):
        i = np.ascontiguousarray(i, np.int32)
        j = np.ascontiguousarray(j, np.int32)
        s = _f32(stf_xyz).reshape(-1)
        assert s.size == 3 * i.size * self.nt, "stf must be [3][nsrc][nt]"
        _check(lib().seiswg_sim_set_sources(self._h, i.size, _ip(i), _ip(j), _fp(s)))

    def set_receivers(self, i: Sequence[int], j: Sequence[int]):
        i = np.ascontiguousarray(i, np.int32)
        j = np.ascontiguousarray(j, np.int32)
        _check(lib().seiswg_sim_set_receivers(self._h, i.size, _ip(i), _ip(j)))
        self.nrec = int(i.size)

    def forward(self, isrc: int = -1, snap_every: int = 0, fields: Iterable[str] = (), sync: bool = True):
        """Runs nt steps.  Returns snapshots [nsnap][nfields][nx][nz] when requested."""
        fields = list(fields)
        if snap_every > 0 and fields:
            nsnap = sum(1 for it in range(1, self.nt) if it % snap_every == 0)
            out = np.zeros((nsnap, len(fields), self.nx, self.nz), np.float32)
            arr = (ctypes.c_char_p * len(fields))(*[f.encode() for f in fields])
            _check(lib().seiswg_sim_forward(self._h, isrc, snap_every, len(fields), arr, _fp(out), 1))
            return out
        _check(lib().seiswg_sim_forward(self._h, isrc, 0, 0, None, None, int(sync)))
        return None

    def traces(self):
        out = np.zeros((5, self.nrec, self.nt), np.float32)
        _check(lib().seiswg_sim_traces(self._h, _fp(out)))
        return out

    def state(self, field: str):
        out = np.zeros((self.nx, self.nz), np.float32)
        _check(lib().seiswg_sim_state(self._h, field.encode(), _fp(out)))
        return out

    def kernel_clear(self):
        _check(lib().seiswg_sim_kernel_clear(self._h))

    def adjoint_forward(self, isrc: int, adj_interval: int):
        _check(lib().seiswg_sim_adjoint_forward(self._h, isrc, adj_interval))

    def adjoint_backward(self, adstf, adj_interval: int):
        a = _f32(adstf).reshape(-1)
        _check(lib().seiswg_sim_adjoint_backward(self._h, _fp(a), adj_interval))

    def kernel_smooth(self, sigma: float):
        _check(lib().seiswg_sim_kernel_smooth(self._h, sigma))

    def kernel(self):
        out = np.zeros((self.nx, self.nz), np.float32)
        _check(lib().seiswg_sim_kernel(self._h, _fp(out)))
        return out

    # -- exact adjoint ---------------------------------------------------
    def gradient_clear(self):
        _check(lib().seiswg_sim_gradient_clear(self._h))

    def forward_op(self, isrc: int = -1, ckpt_every: int = 0):
        """Forward run storing checkpoints; traces via traces()."""
        _check(lib().seiswg_sim_forward_op(self._h, isrc, ckpt_every))

    def backward_op(self, adj):
        """Reverse sweep for dJ/dd, [ncomp][nrec][nt] (SH: uy; PSV: ux, uz)."""
        a = _f32(adj).reshape(-1)
        _check(lib().seiswg_sim_backward_op(self._h, _fp(a)))

    @property
    def checkpoint_interval(self) -> int:
        """Checkpoint interval of the last forward_op."""
        return int(lib().seiswg_sim_checkpoint_interval(self._h))

    def checkpoint_plan(self):
        """Of the last forward_op: dict(slots = binomial checkpointing slots
        (0: uniform), interval, recomputed = forward steps the reverse sweep
        recomputes, bytes = device memory of the checkpoints)."""
        s, k, r, b = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int64(), ctypes.c_size_t()
        _check(lib().seiswg_sim_checkpoint_plan(self._h, ctypes.byref(s), ctypes.byref(k), ctypes.byref(r),
                                                ctypes.byref(b)))
        return dict(slots=s.value, interval=k.value, recomputed=r.value, bytes=b.value)

    def set_observed(self, obs):
        """Observed traces [ncomp][nrec][nt] for misfit_op (kept on the device)."""
        a = _f32(obs).reshape(-1)
        _check(lib().seiswg_sim_set_observed(self._h, _fp(a)))

    def misfit_op(self) -> float:
        """L2 waveform misfit of the last forward_op on the device; keeps its
        adjoint source there for backward_op_device()."""
        J = ctypes.c_double(0.0)
        _check(lib().seiswg_sim_misfit_op(self._h, ctypes.byref(J)))
        return J.value

    def backward_op_device(self):
        """Reverse sweep with the adjoint source left by misfit_op()."""
        _check(lib().seiswg_sim_backward_op_device(self._h))

    def gradient(self, param: str):
        out = np.zeros((self.nx, self.nz), np.float32)
        _check(lib().seiswg_sim_gradient(self._h, param.encode(), _fp(out)))
        return out

    def release_workspace(self):
        _check(lib().seiswg_sim_release_workspace(self._h))

    def set_option(self, key: str, value: int):
        """The options of seiswg_sim_set_option (include/seiswg.h): "graphs", "chunk_rows", "loader",
        "two_step", "two_step_rows", "two_step_producer", "reverse_producer", "cluster", "tma", "pdl", "autotune", "stability_check",
        "checkpoint_slots", "checkpoint_budget_mb", "wait_polls", "test_arm_extra"."""
        _check(lib().seiswg_sim_set_option(self._h, key.encode(), int(value)))

    def synchronize(self):
        _check(lib().seiswg_sim_synchronize(self._h))

    @property
    def launches(self) -> int:
        return lib().seiswg_sim_launches(self._h)

    @property
    def stream(self) -> int:
        return lib().seiswg_sim_stream(self._h) or 0

    @property
    def device_bytes(self) -> int:
        return lib().seiswg_sim_device_bytes(self._h)

    def close(self):
        if getattr(self, "_h", None) and self._owner is None and _lib is not None:
            _lib.seiswg_sim_free(self._h)
        self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        self.close()


class Batch:
    """Gradients of many independent problems in grouped launches under one
    CUDA graph.  sims: prepared Sim objects (SH or PSV, sources = shots);
    obs[p]: observed traces [nshot][ncomp][nrec][nt] of problem p."""

    def __init__(self, sims, obs, ckpt_every: int = 0, stream=None):
        self._sims = list(sims)   # the problems must outlive the batch
        self._obs = [_f32(o).reshape(-1) for o in obs]
        hs = (_vp * len(sims))(*[s._h for s in sims])
        ps = (_pf * len(sims))(*[_fp(o) for o in self._obs])
        h = _vp()
        _check(lib().seiswg_batch_create(hs, ps, len(sims), ckpt_every, stream, ctypes.byref(h)))
        self._h = h

    def run(self):
        _check(lib().seiswg_batch_run(self._h))

    def set_option(self, key: str, value: int):
        """"chunk_rows" (0: per-problem model), "two_step" (0/1), "reverse_producer" (0/1: grouped PSV
        reverse launches with rows from producer warps), "two_step_recompute" (0/1: the
        intervals' states recomputed two steps per grouped launch), "concurrent" (0, 1, 2: grouped
        launches in that order; 3: one persistent launch over a device queue), "stream_groups" (1..4),
        "tma" (0/1: rows of the two-step and reverse marches by tensor copies or bulk copies), "pdl" (0/1:
        programmatic dependent launch of the grouped launches),
        "queue_wait_us" (bound of a queue dependency wait), "queue_band" (slots per band of the queue's
        order, 0: slot-major), "test_queue_need_extra" (test hook),
        "checkpoint_slots" or "autotune" (slots per timing window)."""
        _check(lib().seiswg_batch_set_option(self._h, key.encode(), int(value)))

    def gradient(self, problem: int, param: str):
        s = self._sims[problem]
        out = np.zeros((s.nx, s.nz), np.float32)
        _check(lib().seiswg_batch_gradient(self._h, problem, param.encode(), _fp(out)))
        return out

    def misfit(self, problem: int) -> float:
        return lib().seiswg_batch_misfit(self._h, problem)

    def info(self):
        j, s, l, b = _i32(), _i32(), ctypes.c_uint64(), _sz()
        _check(lib().seiswg_batch_info(self._h, ctypes.byref(j), ctypes.byref(s), ctypes.byref(l), ctypes.byref(b)))
        return dict(jobs=j.value, slots=s.value, launches_per_run=l.value, device_bytes=b.value,
                    chunk_rows=int(lib().seiswg_batch_chunk_rows(self._h)),
                    two_step=bool(lib().seiswg_batch_two_step(self._h)),
                    concurrent=int(lib().seiswg_batch_concurrent(self._h)),
                    stream_groups=int(lib().seiswg_batch_stream_groups(self._h)),
                    tma_jobs=int(lib().seiswg_batch_tma_jobs(self._h)), **self.queue(), **self.checkpoint_plan())

    def queue(self):
        """dict(queue_units = units in the device queue, queue_blocks = CTAs of the persistent launch
        (both 0 outside launch order 3), queue_band = slots per band of the queue's order)."""
        u, b, k = ctypes.c_int64(), _i32(), _i32()
        _check(lib().seiswg_batch_queue(self._h, ctypes.byref(u), ctypes.byref(b), ctypes.byref(k)))
        return dict(queue_units=u.value, queue_blocks=b.value, queue_band=k.value)

    def checkpoint_plan(self):
        """dict(checkpoint_slots = binomial slots per job (0: uniform),
        recomputed_steps = forward steps recomputed per run over all jobs)."""
        s, r = _i32(), ctypes.c_int64()
        _check(lib().seiswg_batch_checkpoint_plan(self._h, ctypes.byref(s), ctypes.byref(r)))
        return dict(checkpoint_slots=s.value, recomputed_steps=r.value)

    @property
    def stream(self) -> int:
        return lib().seiswg_batch_stream(self._h) or 0

    def close(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.seiswg_batch_free(self._h)
            self._h = None

    def __del__(self):
        self.close()


# ---------------------------------------------------------------------------
# Host numerics of the reference
# ---------------------------------------------------------------------------

def ricker(nt: int, dt: float, f0: float, t0: float, ang: float = 0.0, amp: float = 1.0e10):
    """[3][nt] Ricker STF (x, y, z), solver.rs:350-356."""
    out = np.zeros(3 * nt, np.float32)
    _check(lib().seiswg_ricker(nt, dt, f0, t0, ang, amp, _fp(out)))
    return out.reshape(3, nt)


def waveform_misfit(syn, obs, dt: float):
    """(misfit, adstf) of solver.rs:432-467."""
    s, o = _f32(syn), _f32(obs)
    nrec, nt = s.shape
    ad = np.zeros_like(s)
    m = ctypes.c_double()
    _check(lib().seiswg_waveform_misfit(_fp(s), _fp(o), nrec, nt, dt, _fp(ad), ctypes.byref(m)))
    return m.value, ad


def npy_encode(a) -> bytes:
    a = _f32(a)
    assert a.ndim == 2
    n = _sz()
    _check(lib().seiswg_npy_encode(_fp(a), a.shape[0], a.shape[1], None, ctypes.byref(n)))
    buf = ctypes.create_string_buffer(n.value)
    _check(lib().seiswg_npy_encode(_fp(a), a.shape[0], a.shape[1], buf, ctypes.byref(n)))
    return buf.raw[: n.value]


def smooth_noalloc(in_ptr: int, out_ptr: int, nx: int, nz: int, sigma: float, stream: int = 0):
    """Gaussian smoothing of a device field without device allocation
    (seiswg_smooth_noalloc): in_ptr/out_ptr are device addresses of nx*nz
    float32 arrays owned by the caller."""
    _check(lib().seiswg_smooth_noalloc(in_ptr, out_ptr, nx, nz, sigma, stream or None))


def l2_misfit(syn, obs, dt: float):
    """(J, dJ/dsyn) of J = sum (taper (syn - obs))^2; syn/obs [..., nt]."""
    s, o = _f32(syn), _f32(obs)
    nt = s.shape[-1]
    ntr = s.size // nt
    adj = np.zeros_like(s)
    J = ctypes.c_double()
    _check(lib().seiswg_l2_misfit(_fp(s), _fp(o), ntr, nt, dt, _fp(adj), ctypes.byref(J)))
    return J.value, adj


def velocity_gradients(g_lam, g_mu, g_b, vp, vs, rho):
    """(g_vp, g_vs, g_rho) from gradients with respect to lambda, mu, 1/rho."""
    arrs = [_f32(a).reshape(-1) for a in (g_lam, g_mu, g_b, vp, vs, rho)]
    n = arrs[0].size
    outs = [np.zeros(n, np.float32) for _ in range(3)]
    _check(lib().seiswg_velocity_gradients(*[_fp(a) for a in arrs], n, *[_fp(o) for o in outs]))
    shp = np.shape(g_lam)
    return tuple(o.reshape(shp) for o in outs)


def infer_grid(x, z):
    x, z = _f32(x).reshape(-1), _f32(z).reshape(-1)
    nx, nz, dx, dz = _i32(), _i32(), ctypes.c_float(), ctypes.c_float()
    _check(lib().seiswg_infer_grid(_fp(x), _fp(z), x.size, ctypes.byref(nx), ctypes.byref(nz),
                                   ctypes.byref(dx), ctypes.byref(dz)))
    return nx.value, nz.value, dx.value, dz.value


__all__ = ["SeiswgError", "Vfs", "Config", "Solver", "Sim", "Batch", "SimDesc", "ricker", "waveform_misfit",
           "npy_encode", "infer_grid", "smooth_noalloc", "l2_misfit", "velocity_gradients", "lib", "LIB_PATH", "CLI_PATH", "PROTOTYPES"]
