"""Parity report: the GPU results against the reference's WGSL fixtures and
against the FP32 and FP64 oracles, as a markdown table (needs a GPU).

    python tests/parity_report.py

Rows: the reference's three examples through the drop-in host API (fixtures
are WGSL-path outputs), and seeded oracle cases for each kernel family (the
step kernels, the two-step PSV and SH kernels, the cluster kernel for small SH grids,
the spin kernel).  Columns: relative L2 and max|d|/peak against the fixture
(where there is one), relative L2 against the FP32 oracle (reference operation
order) and the FP64 oracle, and the FP32 oracle's own distance from FP64.
"""
import os
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from tests.examples import golden, max_rel, oracle_example, rel_l2, write_example  # noqa: E402
from tests.test_gpu_parity import _model, _run_pair  # noqa: E402


def _fmt(v):
    return "—" if v is None else f"{v:.1e}"


def examples(rows):
    import seiswg_gb300 as sw

    tmp = tempfile.mkdtemp()
    # forward example (SH 200 x 200): snapshot at it=100 and uy traces
    cfg = write_example("forward", os.path.join(tmp, "forward"))
    g = golden("forward")
    with sw.Solver(sw.Config.load(cfg)) as s:
        s.run_forward()
    out = os.path.join(tmp, "forward", "output")
    snap = np.fromfile(os.path.join(out, "proc000100_vy.bin"), "<f4")
    uy = np.load(os.path.join(out, "traces", "uy_000000.npy"))
    refs = {}
    for prec in (32, 64):
        o, s_, _, _ = oracle_example("forward", prec)
        snaps = o.run_forward(-1, 100, ["VY"])
        refs[prec] = dict(snap=snaps[0, 0].reshape(-1), uy=o.obs("Y"))
    for name, ours, fix, key in (("forward example: vy at it=100", snap, g["fix_proc000100_vy"], "snap"),
                                 ("forward example: uy traces", uy, g["fix_uy_000000"], "uy")):
        rows.append((name, rel_l2(ours, fix), max_rel(ours, fix), rel_l2(ours, refs[32][key]),
                     rel_l2(ours, refs[64][key]), rel_l2(refs[32][key], refs[64][key])))
    # spin example (PSV + micropolar 200 x 200): vx at it=200 and ry traces
    cfg = write_example("spin", os.path.join(tmp, "spin"))
    g = golden("spin")
    with sw.Solver(sw.Config.load(cfg)) as s:
        s.run_forward()
    out = os.path.join(tmp, "spin", "output")
    vx = np.fromfile(os.path.join(out, "proc000200_vx.bin"), "<f4")
    ry = np.load(os.path.join(out, "ry_000000.npy"))
    refs = {}
    for prec in (32, 64):
        o, s_, _, _ = oracle_example("spin", prec)
        snaps = o.run_forward(-1, 200, ["VX"])
        refs[prec] = dict(vx=snaps[0, 0].reshape(-1), ry=o.obs("Y"))  # ry: the spin run's y trace
    for name, ours, fix, key in (("spin example: vx at it=200", vx, g["fix_proc000200_vx"], "vx"),
                                 ("spin example: ry traces", ry, g["fix_ry_000000"], "ry")):
        rows.append((name, rel_l2(ours, fix), max_rel(ours, fix), rel_l2(ours, refs[32][key]),
                     rel_l2(ours, refs[64][key]), rel_l2(refs[32][key], refs[64][key])))


def oracle_cases(rows):
    import seiswg_gb300 as sw

    cases = [
        ("SH 200 x 200, cluster kernel (whole run on chip)", 200, 200, 600, 10.0, 1.0e-3,
         [(100, 100, 10.0, 0.12, 0.0)], [(i, 20) for i in range(10, 191, 15)],
         dict(sh=True, psv=False, abs_left=True, abs_right=True, abs_bottom=True, abs_top=True, abs_width=20), {}),
        ("SH 600 x 520, two-step kernel", 600, 520, 400, 10.0, 1.0e-3,
         [(300, 260, 15.0, 0.08, 0.0)], [(i, 300) for i in range(240, 361, 15)],
         dict(sh=True, psv=False, abs_left=True, abs_right=True, abs_bottom=True, abs_top=True, abs_width=20), {}),
        ("SH 600 x 520, one-step kernel", 600, 520, 400, 10.0, 1.0e-3,
         [(300, 260, 15.0, 0.08, 0.0)], [(i, 300) for i in range(240, 361, 15)],
         dict(sh=True, psv=False, abs_left=True, abs_right=True, abs_bottom=True, abs_top=True, abs_width=20),
         {"two_step": 0}),
        ("PSV 512 x 480, two-step kernel", 512, 480, 400, 5.0, 4.0e-4,
         [(256, 50, 15.0, 0.05, 90.0)], [(i, 0) for i in range(0, 512, 32)] + [(256, 240)],
         dict(psv=True, abs_left=True, abs_right=True, abs_bottom=True, abs_top=True, abs_width=40), {}),
        ("PSV 512 x 480, one-step kernel", 512, 480, 400, 5.0, 4.0e-4,
         [(256, 50, 15.0, 0.05, 90.0)], [(i, 0) for i in range(0, 512, 32)] + [(256, 240)],
         dict(psv=True, abs_left=True, abs_right=True, abs_bottom=True, abs_top=True, abs_width=40),
         {"two_step": 0}),
        ("PSV + spin 300 x 260", 300, 260, 500, 1.0, 1.0e-4,
         [(150, 130, 50.0, 0.024, 45.0)], [(i, 130) for i in range(30, 271, 30)],
         dict(psv=True, spin=True, abs_left=True, abs_right=True, abs_bottom=True, abs_top=True, abs_width=30), {}),
    ]
    comps = {"x": 0, "y": 1, "z": 2, "yi": 3, "yc": 4}
    for name, nx, nz, nt, dx, dt, src, rec, flags, opts in cases:
        orig = sw.Sim.prepare

        def prepare(self, _o=opts):
            orig(self)
            for k, v in _o.items():
                self.set_option(k, v)

        sw.Sim.prepare = prepare
        try:
            gpu, ref = _run_pair(nx, nz, nt, dx, dt, src, rec, _model(nx, nz, 11, spin=flags.get("spin", False),
                                                                       dx=dx), **flags)
        finally:
            sw.Sim.prepare = orig
        names = (["y"] if flags.get("sh") else []) + (["x", "z"] if flags.get("psv", True) else []) + \
                (["yi", "yc"] if flags.get("spin") else [])
        for c in names:
            k = comps[c]
            rows.append((f"{name}: u{c} traces", None, None, rel_l2(gpu["traces"][k], ref[32]["obs"][k]),
                         rel_l2(gpu["traces"][k], ref[64]["obs"][k]), rel_l2(ref[32]["obs"][k], ref[64]["obs"][k])))
        for f, a in gpu["state"].items():
            rows.append((f"{name}: final {f}", None, None, rel_l2(a, ref[32]["state"][f]),
                         rel_l2(a, ref[64]["state"][f]), rel_l2(ref[32]["state"][f], ref[64]["state"][f])))


def main():
    rows = []
    examples(rows)
    oracle_cases(rows)
    print("| result | rel L2 vs fixture | max|d|/peak vs fixture | rel L2 vs FP32 oracle | rel L2 vs FP64 oracle "
          "| FP32 oracle vs FP64 |")
    print("|---|---|---|---|---|---|")
    for r in rows:
        print(f"| {r[0]} | " + " | ".join(_fmt(v) for v in r[1:]) + " |")


if __name__ == "__main__":
    main()
