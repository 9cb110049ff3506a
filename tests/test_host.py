"""Host-side behaviour of the drop-in API, no GPU needed: INI semantics
(config.rs), file formats, Ricker STF, misfit, grid inference, and the error
behaviour of Solver::new on bad inputs (solver.rs:220-267, 578-751)."""
import io
import os

import numpy as np
import pytest

import seiswg_gb300 as sw
from oracle import oracle as O
from tests.examples import golden, write_example

FORWARD_INI = """[workflow]
mode = Forward

[solver]
nt = 1200
dt = 0.015
abs_bottom = YES
abs_left = yes
abs_right = no
abs_width = 15
save_snapshot = 100
combine_sources = yes
threads_per_block = abc

[path]
output        = output
output_traces = output/traces
model_init    = model
sources       = sources.dat
stations      = /abs/stations.dat
"""


def test_config_defaults_and_booleans():
    c = sw.Config.from_str(FORWARD_INI, "/base")
    assert c.get("workflow") == "forward"            # trimmed and lower-cased
    assert c.get("solver.nt") == "1200"
    assert float(c.get("solver.dt")) == np.float32(0.015)
    assert c.get("solver.sh") == "no"                 # default no   (config.rs:163)
    assert c.get("solver.psv") == "yes"               # default yes  (config.rs:164)
    assert c.get("solver.spin") == "no"
    assert c.get("solver.abs_bottom") == "yes"        # "YES" -> yes after lower-casing
    assert c.get("solver.abs_right") == "no"
    assert c.get("solver.abs_top") == "no"
    assert c.get("solver.abs_width") == "15"
    assert float(c.get("solver.abs_alpha")) == np.float32(0.015)
    assert c.get("solver.threads_per_block") == "128"  # unparsable -> default (config.rs:85-89)
    assert c.get("solver.adj_interval") == "10"
    assert float(c.get("solver.smooth")) == 5.0
    assert c.get("solver.save_snapshot") == "100"
    assert c.get("solver.combine_sources") == "yes"


def test_config_paths_resolve_against_base():
    c = sw.Config.from_str(FORWARD_INI, "/base")
    assert c.get("path.output") == "/base/output"
    assert c.get("path.output_traces") == "/base/output/traces"
    assert c.get("path.model_init") == "/base/model"
    assert c.get("path.stations") == "/abs/stations.dat"
    with pytest.raises(sw.SeiswgError):
        c.get("path.traces")                          # unset optional key
    with pytest.raises(sw.SeiswgError):
        c.get("path.model_true")


def test_config_load_from_file_uses_its_directory(tmp_path):
    p = tmp_path / "sub" / "config.ini"
    p.parent.mkdir()
    p.write_text(FORWARD_INI)
    c = sw.Config.load(str(p))
    assert c.get("path.output") == str(tmp_path / "sub" / "output")


@pytest.mark.parametrize("text,msg", [
    ("[solver]\nnt=1\ndt=1\n[path]\noutput=o\nsources=s\nstations=t\n", "[workflow] mode is required"),
    ("[workflow]\nmode=forward\n[solver]\ndt=1\n[path]\noutput=o\nsources=s\nstations=t\n", "[solver] nt is required"),
    ("[workflow]\nmode=forward\n[solver]\nnt=x\ndt=1\n[path]\noutput=o\nsources=s\nstations=t\n",
     "[solver] nt must be an integer"),
    ("[workflow]\nmode=forward\n[solver]\nnt=5\ndt=fast\n[path]\noutput=o\nsources=s\nstations=t\n",
     "[solver] dt must be a float"),
    ("[workflow]\nmode=forward\n[solver]\nnt=5\ndt=1\n[path]\nsources=s\nstations=t\n", "[path] output is required"),
    ("[workflow]\nmode=forward\n[solver]\nnt=5\ndt=1\n[path]\noutput=o\nstations=t\n", "[path] sources is required"),
])
def test_config_errors(text, msg):
    with pytest.raises(sw.SeiswgError) as e:
        sw.Config.from_str(text, "")
    assert msg in str(e.value)


def test_config_missing_file():
    with pytest.raises(sw.SeiswgError) as e:
        sw.Config.load("/nonexistent/config.ini")
    assert e.value.code == sw.EIO


def test_config_comments_and_case():
    c = sw.Config.from_str("; comment\n# another\n[WORKFLOW]\nMODE : adjoint\n[Solver]\nNT=7\ndt = 2.5 ; tail\n"
                           "[path]\noutput=o\nsources=s\nstations=t\ntraces = obs\n", "b")
    assert c.get("workflow") == "adjoint"
    assert c.get("solver.nt") == "7"
    assert float(c.get("solver.dt")) == 2.5
    assert c.get("path.traces") == "b/obs"


def test_ricker_matches_oracle_bitwise():
    for (nt, dt, f0, t0, ang, amp) in [(1200, 0.015, 1.0, 1.0, 0.0, 1e10), (300, 1e-4, 50.0, 0.05, 30.0, 1e10),
                                        (4000, 1.0131627e-4, 15.0, 0.1, 90.0, 1e10)]:
        got = sw.ricker(nt, dt, f0, t0, ang, amp)
        ref = O.ricker(nt, dt, f0, t0, ang, amp, 32)
        assert np.array_equal(got, ref)
    # angle 90: x = stf, z = -stf*cos(pi/2) ~ 0 (solver.rs:355)
    s = sw.ricker(100, 1e-3, 20.0, 0.05, 90.0, 1.0)
    assert np.allclose(s[0], s[1]) and np.abs(s[2]).max() < 1e-6 * np.abs(s[1]).max()


def test_misfit_matches_oracle_bitwise():
    rng = np.random.default_rng(3)
    syn = rng.standard_normal((7, 501)).astype(np.float32)
    obs = rng.standard_normal((7, 501)).astype(np.float32)
    m, ad = sw.waveform_misfit(syn, obs, 0.06)
    m_ref, ad_ref = O.misfit_f32(syn, obs, 0.06)
    assert m == m_ref
    assert np.array_equal(ad, ad_ref)
    # time-reversed adjoint source, zero taper at both ends (solver.rs:450-463)
    assert ad[0, 0] == 0.0 and ad[0, -1] == 0.0
    assert m > 0


@pytest.mark.parametrize("shape", [(13, 1200), (1, 1), (144, 4800), (0, 5), (7, 2000)])
def test_npy_encoding(shape):
    a = np.arange(np.prod(shape), dtype=np.float32).reshape(shape)
    b = sw.npy_encode(a)
    assert b[:8] == b"\x93NUMPY\x01\x00"
    hl = int.from_bytes(b[8:10], "little")
    assert (10 + hl) % 64 == 10 % 64 or hl % 64 == 0   # header (dict + '\n') padded to 64 (solver.rs:275)
    assert hl % 64 == 0
    assert b[10 + hl - 1:10 + hl] == b"\n"
    r = np.load(io.BytesIO(b))
    assert r.dtype == np.float32 and r.shape == shape and np.array_equal(r, a)
    dict_txt = f"{{'descr': '<f4', 'fortran_order': False, 'shape': ({shape[0]}, {shape[1]}), }}"
    assert b[10:10 + len(dict_txt)].decode() == dict_txt


def test_fixture_npy_headers_match_our_encoder():
    """The reference's own .npy fixtures carry exactly our header bytes."""
    g = golden("forward")
    ref = g["fix_uy_000000"]
    b = sw.npy_encode(ref)
    assert np.array_equal(np.load(io.BytesIO(b)), ref)


def test_infer_grid_matches_oracle():
    for name, pre in (("forward", "model_"), ("spin", "model_"), ("adjoint", "init_")):
        g = golden(name)
        assert sw.infer_grid(g[pre + "x"], g[pre + "z"]) == O.infer_grid(g[pre + "x"], g[pre + "z"])
    # non-square grid with dx == dz
    x = np.repeat(np.arange(30, dtype=np.float32) * 7.0, 50)
    z = np.tile(np.arange(50, dtype=np.float32) * 7.0, 30)
    assert sw.infer_grid(x, z) == (30, 50, 7.0, 7.0)
    # The reference infers nx from the extents' aspect ratio, which assumes
    # dx == dz; with dx != dz it gets nx*nz != npt.  Rectangular cells are
    # read from the coordinate layout instead.
    z3 = np.tile(np.arange(50, dtype=np.float32) * 3.0, 30)
    assert O.infer_grid(x, z3)[:2] == (46, 33)
    assert sw.infer_grid(x, z3) == (30, 50, 7.0, 3.0)
    # a coincidental nx*nz == npt under the aspect-ratio rule still defers to the layout
    xs = np.repeat(np.arange(40, dtype=np.float32) * 10.0, 90)
    zs = np.tile(np.arange(90, dtype=np.float32) * 1.0, 40)
    nx_ref, nz_ref = O.infer_grid(xs, zs)[:2]
    assert nx_ref * nz_ref != 3600 or (nx_ref, nz_ref) != (40, 90)
    assert sw.infer_grid(xs, zs) == (40, 90, 10.0, 1.0)
    # a large grid (its extents scanned by several threads), origin off zero
    xl = np.repeat(np.float32(-1234.5) + np.arange(2048, dtype=np.float32) * np.float32(12.5), 2048)
    zl = np.tile(np.float32(77.25) + np.arange(2048, dtype=np.float32) * np.float32(12.5), 2048)
    assert sw.infer_grid(xl, zl) == O.infer_grid(xl, zl)
    assert sw.infer_grid(xl, zl)[:2] == (2048, 2048)
    # extents as the reference folds them (f32::max / f32::min from
    # -/+infinity): a NaN anywhere is passed over, the first element included
    zn = zl.copy()
    zn[zn.size * 5 // 7] = np.nan
    assert sw.infer_grid(xl, zn) == sw.infer_grid(xl, zl)
    zn[0] = np.nan
    assert sw.infer_grid(xl, zn) == sw.infer_grid(xl, zl)
    xn = xl.copy()
    xn[0] = np.nan            # the smallest x, also held by the rest of the first column
    assert sw.infer_grid(xn, zl) == O.infer_grid(xn, zl)
    with pytest.raises(sw.SeiswgError):
        sw.infer_grid(np.full(16, np.nan, np.float32), zl[:16])
    # square cells that the layout check cannot read, which the reference
    # accepts by its aspect-ratio rule: coordinates stored z first, and x
    # values jittered by rounding within a column
    xz = np.tile(np.arange(30, dtype=np.float32) * 7.0, 50)
    zz = np.repeat(np.arange(50, dtype=np.float32) * 7.0, 30)
    assert sw.infer_grid(xz, zz) == O.infer_grid(xz, zz) == (30, 50, 7.0, 7.0)
    xj = x + (np.random.default_rng(1).random(x.size).astype(np.float32) - 0.5) * np.float32(1e-3)
    xj[0], xj[-1] = x[0], x[-1]
    assert sw.infer_grid(xj, z) == O.infer_grid(xj, z)
    # coordinates that form no grid: errors
    with pytest.raises(sw.SeiswgError) as e:
        sw.infer_grid(x, np.random.default_rng(0).random(x.size).astype(np.float32) * 100)
    assert "rectangular grid" in str(e.value)
    with pytest.raises(sw.SeiswgError):
        sw.infer_grid(np.zeros(10, np.float32), np.zeros(10, np.float32))


# ---- Solver::new input errors (raised before any GPU work) -----------------

def _example(tmp_path, name="forward"):
    return write_example(name, str(tmp_path / name))


def test_solver_missing_model_file(tmp_path):
    cfg = _example(tmp_path)
    os.remove(os.path.join(os.path.dirname(cfg), "model", "proc000000_vs.bin"))
    with pytest.raises(sw.SeiswgError) as e:
        sw.Solver(sw.Config.load(cfg))
    assert e.value.code == sw.EIO and "proc000000_vs.bin" in str(e.value)


def test_solver_truncated_model_file(tmp_path):
    cfg = _example(tmp_path)
    p = os.path.join(os.path.dirname(cfg), "model", "proc000000_vp.bin")
    b = open(p, "rb").read()
    open(p, "wb").write(b[:1000])
    with pytest.raises(sw.SeiswgError) as e:
        sw.Solver(sw.Config.load(cfg))
    assert "too short" in str(e.value)


def test_solver_station_outside_grid(tmp_path):
    cfg = _example(tmp_path)
    with open(os.path.join(os.path.dirname(cfg), "stations.dat"), "a") as f:
        f.write("1.0e9 100.0\n")
    with pytest.raises(sw.SeiswgError) as e:
        sw.Solver(sw.Config.load(cfg))
    assert "outside the grid" in str(e.value)


def test_solver_no_model_path(tmp_path):
    c = sw.Config.from_str("[workflow]\nmode=forward\n[solver]\nnt=5\ndt=1\n[path]\noutput=o\nsources=s\n"
                           "stations=t\n", str(tmp_path))
    with pytest.raises(sw.SeiswgError) as e:
        sw.Solver(c)
    assert "No model path" in str(e.value)


def test_solver_reads_inputs_from_vfs_first(tmp_path):
    """VFS entries shadow the disk (solver.rs:236-267): a VFS stations table with
    an out-of-grid station fails although the file on disk is valid."""
    cfg = _example(tmp_path)
    st = os.path.join(os.path.dirname(cfg), "stations.dat")
    v = sw.Vfs({st: b"1.0e9 0.0\n"})
    with pytest.raises(sw.SeiswgError) as e:
        sw.Solver(sw.Config.load(cfg), v)
    assert "outside the grid" in str(e.value)


def test_vfs_roundtrip():
    v = sw.Vfs({"a/b.bin": b"\x00\x01\x02", "c": b""})
    assert v["a/b.bin"] == b"\x00\x01\x02"
    assert v["c"] == b""
    assert sorted(v.keys()) == ["a/b.bin", "c"]
    with pytest.raises(sw.SeiswgError):
        v["missing"]


def test_gpu_paths_fail_loudly_without_a_gpu():
    """No CPU fallback: without a usable GPU the engine reports a CUDA error."""
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(sw.SeiswgError) as e:
        sw.Sim(16, 16, 4, 1.0, 1.0, 1e-3)
    assert e.value.code == sw.ECUDA
