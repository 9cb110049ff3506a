"""Benchmark: PSV forward, heterogeneous, 4096 x 4096, nt = 4000 (the HBM-bound
headline workload), in Gcell-updates/s on one GB300.

A step is one complete forward simulation (4000 time steps of the fused
velocity+stress kernel over 16.8 M cells, plus receiver traces).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--nt NT]

value  device throughput: model, sources and receivers resident in HBM; CUDA
       events on the engine's stream around K forward runs.
e2e    the reference-facing C ABI with host buffers: per step
       seiswg_solver_new (INI text + model files in a VFS, uploaded to the GPU)
       + seiswg_solver_run_forward (traces copied back as .npy bytes).
--impl reference  the CPU oracle (a restatement of the reference's WGSL
       kernels; the WGSL itself has no CPU path here) on all host cores, on a
       bounded sample of the same workload.
N > 1: independent replicas, one per GPU (shots are independent; no
       collective on the data path); value = total cell-updates / max time.
other_configs  (N = 1) after the headline, C1, C3, C4 and C5 each measured by
       its own `bench.py --workload cX --no-cpu` process and summarised in the
       same line (--no-others skips them).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Gcell-updates/s"
BYTES_PER_CELL = {"sh": 32, "psv": 52, "spin": 96}  # algorithmic bytes per cell-update


# ---------------------------------------------------------------------------
# Workload: PSV forward, heterogeneous, 4096^2 (seeded synthetic model)
# ---------------------------------------------------------------------------
def make_workload(nx=4096, nz=4096, nt=4000, seed=0):
    from scipy.ndimage import gaussian_filter

    dx = dz = 5.0
    rng = np.random.default_rng(seed)
    p = gaussian_filter(rng.standard_normal((nx, nz)).astype(np.float32), 20.0)
    p *= np.float32(0.05 / np.abs(p).max())
    depth_km = (np.arange(nz, dtype=np.float32) * np.float32(dz) / np.float32(1000.0))[None, :]
    vp = ((np.float32(2000.0) + np.float32(600.0) * depth_km) * (np.float32(1.0) + p)).astype(np.float32)
    vs = (vp / np.float32(math.sqrt(3.0))).astype(np.float32)
    rho = (np.float32(310.0) * vp ** np.float32(0.25)).astype(np.float32)
    dt = float(np.float32(0.3 * dx / float(vp.max())))
    w = 40
    src = dict(i=nx // 2, j=w + 10, f0=15.0, t0=0.1, ang=90.0, amp=1.0e10)
    rec_i = np.round(np.linspace(0, nx - 1, 256)).astype(np.int32)  # 256 receivers on the top row
    rec_j = np.zeros(256, np.int32)
    return dict(nx=nx, nz=nz, nt=nt, dx=dx, dz=dz, dt=dt, vp=vp, vs=vs, rho=rho, w=w, alpha=0.015, src=src,
                rec_i=rec_i, rec_j=rec_j)


def workload_config(W, nt, physics="psv"):
    return {"workload": f"{physics.upper()} forward, heterogeneous {W['nx']}x{W['nz']}, nt={nt}",
            "grid": [W["nx"], W["nz"]], "nt": nt, "dx_m": W["dx"], "dt_s": W["dt"],
            "physics": physics, "abs_width": W["w"], "receivers": int(W["rec_i"].size),
            "source": "Ricker f0=15 Hz t0=0.1 s angle 90 at (nx/2, w+10)",
            "model": "vp=2000+600*depth_km, Gaussian-filtered (sigma 20) +-5% perturbation, seed 0; "
                     "vs=vp/sqrt(3); rho=310*vp^0.25",
            "l2": "state+model 8 x 67 MB > 129 MB L2 (no flush needed)",
            "parallelism": "replicas"}


# ---------------------------------------------------------------------------
# Clock sampling during the timed region
# ---------------------------------------------------------------------------
class Clocks:
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for n, v in zip(names, f[4:8]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def _traffic(kernel, nx, nz):
    """DRAM bytes per launch of `kernel` from the committed ncu summary, scaled
    to nx*nz cells; None when no capture is recorded."""
    path = os.path.join(ROOT, "profiles", "traffic.txt")
    try:
        for ln in open(path):
            f = ln.split()
            if len(f) >= 3 and f[0] == kernel:
                return float(f[1]) * (nx * nz) / float(f[2])
    except OSError:
        pass
    return None


def cpu_oracle_rate(W, nt_sample, physics="psv"):
    """FP32 oracle (reference operation order, OpenMP) on the full grid for
    nt_sample steps; returns (Gcell/s, seconds, threads)."""
    from oracle import oracle as O

    s = O.Setup(W["nx"], W["nz"], nt_sample, W["dx"], W["dz"], W["dt"], sh=physics == "sh", psv=physics == "psv",
                abs_left=True, abs_right=True, abs_bottom=True, abs_top=True, abs_width=W["w"],
                abs_alpha=W["alpha"])
    sr = W["src"]
    stf = O.stf_table([(0, 0, sr["f0"], sr["t0"], sr["ang"], sr["amp"])], nt_sample, W["dt"], 32)
    o = O.FD2DOracle(s, [sr["i"] * W["nz"] + sr["j"]], stf, W["rec_i"] * W["nz"] + W["rec_j"], 32)
    o.set_field("LAM", W["vp"])
    o.set_field("MU", W["vs"])
    o.set_field("RHO", W["rho"])
    o.init_model()
    t0 = time.perf_counter()
    o.run_forward(-1)
    dtm = time.perf_counter() - t0
    return W["nx"] * W["nz"] * nt_sample / dtm / 1e9, dtm, O.num_threads()


_ORACLE_SLOT = {"vp": "LAM", "vs": "MU", "rho": "RHO", "lambda": "LAM", "mu": "MU", "nu": "NU", "j": "J",
                "lambda_c": "LAM_C", "mu_c": "MU_C", "nu_c": "NU_C"}


def workload_oracle(W, nt, model=None, precision=32):
    """The oracle set up with a configs.Workload's grid, flags, model, sources
    and receivers, for `nt` steps."""
    from oracle import oracle as O

    f = W.flags
    s = O.Setup(W.nx, W.nz, nt, W.dx, W.dz, W.dt, sh=f.get("sh", False), psv=f.get("psv", True),
                spin=f.get("spin", False), abs_left=f.get("abs_left", False), abs_right=f.get("abs_right", False),
                abs_bottom=f.get("abs_bottom", False), abs_top=f.get("abs_top", False),
                abs_width=f.get("abs_width", 20), abs_alpha=f.get("abs_alpha", 0.015))
    stf = O.stf_table([(0, 0, f0, t0, ang, amp) for (_, _, f0, t0, ang, amp) in W.sources], nt, W.dt, precision)
    o = O.FD2DOracle(s, [i * W.nz + j for (i, j, *_) in W.sources], stf,
                     np.asarray(W.rec_i, np.int64) * W.nz + np.asarray(W.rec_j, np.int64), precision)
    for k, v in (model or W.model).items():
        o.set_field(_ORACLE_SLOT[k], v)
    o.init_model()
    return o


def cpu_forward_rate(W, nt_sample):
    """FP32 oracle forward of shot 0 for nt_sample steps on the full grid:
    (Gcell/s, seconds, threads)."""
    from oracle import oracle as O

    o = workload_oracle(W, nt_sample)
    t0 = time.perf_counter()
    o.run_forward(0)
    dtm = time.perf_counter() - t0
    return W.cells * nt_sample / dtm / 1e9, dtm, O.num_threads()


def cpu_gradient_rate(W, nt_sample):
    """FP32 oracle exact gradient (forward with every step's strains kept, then
    the reverse sweep) of shot 0 for nt_sample steps on the full grid: counted
    cell-updates (2 per cell and step) per second, seconds, threads."""
    from oracle import oracle as O

    o = workload_oracle(W, nt_sample)
    ncomp = 2 if W.flags.get("psv", True) else 1
    adj = np.random.default_rng(0).standard_normal((ncomp, W.rec_i.size, nt_sample)) * 1e-12
    t0 = time.perf_counter()
    o.exact_gradient(adj, 0)
    dtm = time.perf_counter() - t0
    return 2.0 * W.cells * nt_sample / dtm / 1e9, dtm, O.num_threads()


def run_reference(args, rank):
    if rank != 0:
        return
    W = make_workload(nx=args.grid, nz=args.grid, nt=args.nt)
    phys = args.physics
    rates = []
    for _ in range(args.warmup):
        cpu_oracle_rate(W, 2, phys)
    for _ in range(args.steps):
        r, dtm, thr = cpu_oracle_rate(W, args.ref_sample, phys)
        rates.append(r)
    val = float(np.median(rates))
    line = {
        "impl": "reference", "metric": METRIC, "value": val, "unit": METRIC, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup,
        # one step of this arm is the bounded sample (ref_sample of the nt
        # time steps on the full grid); the whole run by linear extrapolation:
        "ms_per_step": dtm * 1e3,
        "extrapolated_ms_per_full_run": dtm * 1e3 * args.nt / args.ref_sample,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(W, args.nt, phys),
        "cpu_baseline": {"value": val, "unit": METRIC, "cores": thr, "kind": "port",
                         "sample": f"full {W['nx']}x{W['nz']} grid, {args.ref_sample} of {args.nt} steps per "
                                   f"step (FP32 oracle restating fd2d.wgsl, OpenMP)"},
        "e2e": {"value": val, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args, rank, world):
    import seiswg_gb300 as sw

    dist = world > 1
    if dist:
        import torch
        import torch.distributed as tdist
    import torch

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    W = make_workload(nx=args.grid, nz=args.grid, nt=args.nt)
    nx, nz, nt = W["nx"], W["nz"], W["nt"]
    sr = W["src"]
    stf = sw.ricker(nt, W["dt"], sr["f0"], sr["t0"], sr["ang"], sr["amp"])[:, None, :]

    # ---- device-resident throughput --------------------------------------
    phys = args.physics
    sim = sw.Sim(nx, nz, nt, W["dx"], W["dz"], W["dt"], sh=phys == "sh", psv=phys == "psv", abs_left=True,
                 abs_right=True, abs_bottom=True, abs_top=True, abs_width=W["w"], abs_alpha=W["alpha"])
    if args.chunk_rows:
        sim.set_option("chunk_rows", args.chunk_rows)
    if args.two_step >= 0:
        sim.set_option("two_step", args.two_step)
    if args.two_step_rows:
        sim.set_option("two_step_rows", args.two_step_rows)
    if args.tma >= 0:
        sim.set_option("tma", args.tma)
    if args.pdl >= 0:
        sim.set_option("pdl", args.pdl)
    if args.two_step_producer >= 0 and phys == "psv":
        sim.set_option("two_step_producer", args.two_step_producer)
    two_step = args.two_step != 0   # the engine's default for PSV alone and SH alone is on
    sim.upload_model("vp", W["vp"])
    sim.upload_model("vs", W["vs"])
    sim.upload_model("rho", W["rho"])
    sim.prepare()
    sim.set_sources([sr["i"]], [sr["j"]], stf)
    sim.set_receivers(W["rec_i"], W["rec_j"])
    stream = torch.cuda.ExternalStream(sim.stream)
    for _ in range(args.warmup):
        sim.forward(0, sync=False)
    sim.synchronize()
    if dist:
        tdist.barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    l0 = sim.launches
    with Clocks(local) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            sim.forward(0, sync=False)
        ev1.record(stream)
        ev1.synchronize()
    sim.synchronize()
    torch.cuda.synchronize()
    launches = sim.launches - l0
    ms = ev0.elapsed_time(ev1)
    tr = sim.traces()
    finite = bool(np.isfinite(tr).all())
    sim.close()
    if dist:
        t = torch.tensor([ms], device="cuda")
        tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
        ms = float(t.item())
        tdist.barrier()

    cells = float(nx) * nz * nt
    ms_per_step = ms / args.steps
    value = world * cells * args.steps / (ms / 1e3) / 1e9
    # Dominant kernel: one launch per time step (one-step kernel) or per two
    # steps (two-step kernel, nt even and no snapshots here); its average
    # duration is the timed region over its launches (memsets and the trace
    # kernel are < 0.1 % of it; see the launch lists under profiles/).
    # Algorithmic bytes of a launch: one pass over the state (read and
    # written) and the material (read), 52 B (PSV) or 32 B (SH) per cell,
    # whether the launch advances one step or two.
    # (two-step rows are fetched by tensor copies unless --tma 0)
    kernel = (f"{phys}_step2_tma_kernel" if args.tma != 0 else f"{phys}_step2_kernel") if two_step \
        else f"{phys}_step_kernel"
    if two_step and args.tma != 0 and args.two_step_producer != 0 and phys == "psv":
        kernel = "psv_step2_pc_kernel"   # the default: rows from producer warps
    per_launch = 2 if two_step else 1
    launch_s = ms_per_step / 1e3 / (nt / per_launch)
    achieved = BYTES_PER_CELL[phys] * nx * nz / launch_s / 1e9
    peak, peak_kind = _peaks()
    traffic = _traffic(kernel, nx, nz)

    # ---- parity outside the timed region: a short run against the FP32 oracle
    parity = None
    if rank == 0 and not args.no_parity:
        parity = short_parity(W, phys, args.parity_nt)

    # ---- end to end through the reference-facing C ABI ---------------------
    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(args, W, stf)
        if dist:
            t = torch.tensor([e2e["seconds"]], device="cuda")
            tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
            e2e["seconds"] = float(t.item())

    cpu = None
    if rank == 0 and not args.no_cpu:
        r, dtm, thr = cpu_oracle_rate(W, args.ref_sample, phys)
        cpu = {"value": r, "unit": METRIC, "cores": thr, "kind": "port",
               "sample": f"full {nx}x{nz} grid, {args.ref_sample} of {nt} steps (FP32 oracle restating "
                         f"fd2d.wgsl, OpenMP), {dtm:.1f} s"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": workload_config(W, nt, phys),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "traffic_source": "profile: dram__bytes_read.sum + dram__bytes_write.sum of one ncu "
                                           "capture of this kernel (profiles/traffic.txt), scaled to the grid; "
                                           "not measured in this run" if traffic else None,
                         "kernel": kernel, "algorithmic_bytes_per_launch": BYTES_PER_CELL[phys] * nx * nz,
                         "bytes_per_cell": BYTES_PER_CELL[phys], "cells_per_launch": nx * nz,
                         "time_steps_per_launch": per_launch, "launch_us": launch_s * 1e6,
                         "peak_source": peak_kind},
            "gpu_launches": int(launches),
            "clocks": clk.summary(),
            "traces_finite": finite,
        }
        if e2e:
            line["e2e"] = {"value": world * cells * args.e2e_steps / e2e["seconds"] / 1e9, "unit": METRIC,
                           "h2d_bytes_per_step": e2e["h2d"], "d2h_bytes_per_step": e2e["d2h"],
                           "api": "seiswg_config_load_str + seiswg_solver_new + seiswg_solver_run_forward"}
        if cpu:
            line["cpu_baseline"] = cpu
        if parity:
            line["parity"] = parity
        if world == 1 and not args.no_others:
            line["other_configs"] = run_others()
        print(json.dumps(line), flush=True)


# The other configurations, measured after the headline in the same run (one
# process each, outside the headline's timed region): C1 and C3 forward, the
# C4 gradient, the C5 batch (autotuned) against its plain per-shot path.
OTHERS = [("c1", ["--steps", "5", "--warmup", "3"], 300),
          ("c3", ["--steps", "2", "--warmup", "3"], 300),
          ("c4", ["--steps", "1", "--warmup", "2"], 600),
          ("c5", ["--steps", "1", "--warmup", "2", "--autotune"], 900)]


def run_others():
    out = {}
    for name, extra, limit in OTHERS:
        cmd = [sys.executable, os.path.abspath(__file__), "--workload", name, "--no-cpu"] + extra
        try:
            r = subprocess.run(cmd, capture_output=True, text=True, timeout=limit)
            lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
            if r.returncode != 0 or not lines:
                out[name] = {"error": f"exit {r.returncode}: " + (r.stderr or r.stdout)[-300:]}
                continue
            d = json.loads(lines[-1])
        except Exception as e:  # noqa: BLE001 - a failed secondary must not lose the headline line
            out[name] = {"error": repr(e)[-300:]}
            continue
        keep = ("metric", "value", "unit", "ms_per_step", "steps", "warmup", "speedup", "max_rel_l2_mu_vs_plain",
                "gcell_updates_per_s", "clocks")
        o = {k: d[k] for k in keep if k in d}
        o["workload"] = d.get("config", {}).get("workload")
        if "roofline" in d:
            o["roofline_frac"] = d["roofline"].get("frac")
        if "plain" in d:
            o["plain_problem_gradients_per_s"] = d["plain"].get("problem_gradients_per_s")
        o["command"] = "bench.py --workload " + name + " --no-cpu " + " ".join(extra)
        out[name] = o
    return out


def short_parity(W, phys, nt_p):
    """The same grid, model, source and receivers for nt_p steps on the GPU and
    in the FP32 oracle (reference operation order): relative L2 of the final
    state fields (the top-row receivers' traces stay zero in both; the row is
    decoupled by the edge rule)."""
    import seiswg_gb300 as sw
    from oracle import oracle as O

    nx, nz = W["nx"], W["nz"]
    sr = W["src"]
    stf = sw.ricker(nt_p, W["dt"], sr["f0"], sr["t0"], sr["ang"], sr["amp"])[:, None, :]
    flags = dict(sh=phys == "sh", psv=phys == "psv", abs_left=True, abs_right=True, abs_bottom=True, abs_top=True,
                 abs_width=W["w"], abs_alpha=W["alpha"])
    fields = ("vy", "sxy", "szy") if phys == "sh" else ("vx", "vz", "sxx", "szz", "sxz")
    slots = dict(vy="VY", sxy="SXY", szy="SZY", vx="VX", vz="VZ", sxx="SXX", szz="SZZ", sxz="SXZ")
    with sw.Sim(nx, nz, nt_p, W["dx"], W["dz"], W["dt"], **flags) as sim:
        sim.upload_model("vp", W["vp"])
        sim.upload_model("vs", W["vs"])
        sim.upload_model("rho", W["rho"])
        sim.prepare()
        sim.set_sources([sr["i"]], [sr["j"]], stf)
        sim.set_receivers(W["rec_i"], W["rec_j"])
        sim.forward(0)
        got = {f: sim.state(f) for f in fields}
        tr = sim.traces()
    s = O.Setup(nx, nz, nt_p, W["dx"], W["dz"], W["dt"], **flags)
    o = O.FD2DOracle(s, [sr["i"] * nz + sr["j"]], stf.astype(np.float64), W["rec_i"] * nz + W["rec_j"], 32)
    o.set_field("LAM", W["vp"])
    o.set_field("MU", W["vs"])
    o.set_field("RHO", W["rho"])
    o.init_model()
    o.run_forward(0)
    errs = {f: float(np.linalg.norm(got[f] - o.field(slots[f])) / max(np.linalg.norm(o.field(slots[f])), 1e-300))
            for f in fields}
    comps = (1,) if phys == "sh" else (0, 2)
    zero = bool(all(not np.any(tr[c]) and not np.any(o.obs(("X", "Y", "Z")[c])) for c in comps))
    return {"rel_l2": max(errs.values()), "per_field": errs, "nt": nt_p, "against": "FP32 oracle",
            "top_row_traces_zero_in_both": zero}


def run_e2e(args, W, stf):
    """Reference-facing API with host buffers: INI + model files in a VFS."""
    import seiswg_gb300 as sw

    nx, nz, nt = W["nx"], W["nz"], W["nt"]
    x = np.repeat(np.arange(nx, dtype=np.float32) * np.float32(W["dx"]), nz)
    z = np.tile(np.arange(nz, dtype=np.float32) * np.float32(W["dz"]), nx)

    def mbin(a):
        a = np.ascontiguousarray(a, np.float32).reshape(-1)
        return np.array([a.size], np.int32).tobytes() + a.tobytes()

    vfs = sw.Vfs({"m/proc000000_x.bin": mbin(x), "m/proc000000_z.bin": mbin(z),
                  "m/proc000000_vp.bin": mbin(W["vp"]), "m/proc000000_vs.bin": mbin(W["vs"]),
                  "m/proc000000_rho.bin": mbin(W["rho"])})
    sr = W["src"]
    vfs["sources.dat"] = (f"{sr['i'] * W['dx']} {sr['j'] * W['dz']} 0 {sr['f0']} {sr['t0']} {sr['ang']} "
                          f"{sr['amp']}\n").encode()
    vfs["stations.dat"] = "".join(f"{i * W['dx']} {j * W['dz']}\n" for i, j in
                                  zip(W["rec_i"], W["rec_j"])).encode()
    sh = args.physics == "sh"
    ini = (f"[workflow]\nmode = forward\n[solver]\nsh = {'yes' if sh else 'no'}\npsv = {'no' if sh else 'yes'}\n"
           f"nt = {nt}\ndt = {W['dt']!r}\n"
           f"abs_top = yes\nabs_bottom = yes\nabs_left = yes\nabs_right = yes\nabs_width = {W['w']}\n"
           f"abs_alpha = {W['alpha']}\ncombine_sources = yes\n[path]\noutput = out\nmodel_init = m\n"
           f"sources = sources.dat\nstations = stations.dat\n")
    cfg = sw.Config.from_str(ini, "")
    h2d = 3 * nx * nz * 4 + 3 * nt * 4 + 2 * 256 * 4
    d2h = (1 if sh else 2) * len(W["rec_i"]) * nt * 4  # the trace components written out (uy; ux, uz)

    def one():
        s = sw.Solver(cfg, vfs, write_files=False)
        out = s.run_forward()
        s.close()
        return out

    one()  # warm-up (context, allocator)
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        out = one()
    sec = time.perf_counter() - t0
    assert any(k.endswith(("uy_000000.npy" if sh else "ux_000000.npy")) for k in out)
    return {"seconds": sec, "h2d": h2d, "d2h": d2h}


def _timed(stream, fn, reps):
    import torch

    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        fn()
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1) / reps


def run_secondary(args):
    """The other benchmark configurations, one JSON line each (not the headline)."""
    import torch

    import seiswg_gb300 as sw
    from seiswg_gb300 import configs

    peak, peak_kind = _peaks()
    out = {"impl": "ours", "workload_key": args.workload, "warmup": args.warmup, "steps": args.steps,
           "dtype": "f32", "data": "synthetic", "n_gpus": 1}
    if args.workload in ("c1", "c3"):
        W = configs.c1_sh_forward() if args.workload == "c1" else configs.c3_spin_forward(nt=args.nt or 3000)
        sim = W.make_sim()
        if args.pdl >= 0:
            sim.set_option("pdl", args.pdl)
        if args.autotune:
            sim.set_option("autotune", 50)
        stream = torch.cuda.ExternalStream(sim.stream)
        snap = W.extra.get("snap_every", 0)
        run = (lambda: sim.forward(0, snap, ["vy"])) if snap else (lambda: sim.forward(0, sync=False))
        for _ in range(args.warmup):
            run()
        sim.synchronize()
        l0 = sim.launches
        with Clocks(0) as clk:
            ms = _timed(stream, run, args.steps)
        sim.synchronize()
        bpc = BYTES_PER_CELL["sh" if args.workload == "c1" else "spin"]
        achieved = bpc * W.cells * W.nt / (ms / 1e3) / 1e9
        out.update(metric=METRIC, value=W.cells * W.nt / (ms / 1e3) / 1e9, unit=METRIC, ms_per_step=ms,
                   higher_is_better=True, config={"workload": W.name, **{k: v for k, v in W.extra.items()
                                                                          if k != "true_model"}},
                   roofline={"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                             "frac": achieved / peak, "bytes_per_cell_update": bpc, "peak_source": peak_kind,
                             "note": "L2-resident grid (3 state + 2 model fields x 160 KB)" if args.workload == "c1"
                             else None},
                   gpu_launches=int((sim.launches - l0) / args.steps), clocks=clk.summary(),
                   traces_finite=bool(np.isfinite(sim.traces()).all()))
        sim.close()
        if not args.no_cpu:
            ns = W.nt if args.workload == "c1" else min(W.nt, 300)
            r, dtm, thr = cpu_forward_rate(W, ns)
            out["cpu_baseline"] = {"value": r, "unit": METRIC, "cores": thr, "kind": "port",
                                   "sample": f"full grid, {ns} of {W.nt} steps (FP32 oracle, OpenMP), {dtm:.1f} s"}
    elif args.workload == "c4":
        W = configs.c4_psv_adjoint(nt=args.nt or 3000)
        sim_t = W.make_sim(model=W.extra["true_model"])
        obs = []
        for s in range(len(W.sources)):
            sim_t.forward(s)
            obs.append(sim_t.traces()[[0, 2]])
        sim_t.close()
        sim = W.make_sim()
        if args.tma >= 0:
            sim.set_option("tma", args.tma)
        if args.pdl >= 0:
            sim.set_option("pdl", args.pdl)
        if args.reverse_producer >= 0:
            sim.set_option("reverse_producer", args.reverse_producer)
        if args.checkpoint_slots:
            sim.set_option("checkpoint_slots", args.checkpoint_slots)
        if args.checkpoint_budget_mb:
            sim.set_option("checkpoint_budget_mb", args.checkpoint_budget_mb)
        stream = torch.cuda.ExternalStream(sim.stream)
        Js = []

        def gradient():
            # Per shot: the observed traces uploaded, the forward operator,
            # the misfit and its adjoint source on the device, the reverse
            # sweep (host misfit: --host-misfit).
            sim.gradient_clear()
            Js.clear()
            for s in range(len(W.sources)):
                if args.host_misfit:
                    sim.forward_op(s, 0)
                    J, adj = sw.l2_misfit(sim.traces()[[0, 2]], obs[s], W.dt)
                    Js.append(J)
                    sim.backward_op(adj)
                else:
                    sim.set_observed(obs[s])
                    sim.forward_op(s, 0)
                    Js.append(sim.misfit_op())
                    sim.backward_op_device()

        for _ in range(max(1, args.warmup)):
            gradient()
        sim.synchronize()
        with Clocks(0) as clk:
            t0 = time.perf_counter()
            ms = _timed(stream, gradient, args.steps)
            wall = (time.perf_counter() - t0) / args.steps
        g = {p: sim.gradient(p) for p in ("lambda", "mu", "buoyancy")}
        gvp, gvs, grho = sw.velocity_gradients(g["lambda"], g["mu"], g["buoyancy"], W.model["vp"], W.model["vs"],
                                               W.model["rho"])
        nshot = len(W.sources)
        cell_updates = 2.0 * W.cells * W.nt * nshot   # forward + adjoint; recomputation not counted
        out.update(metric="gradients/s", value=1000.0 / ms, unit="gradients/s", ms_per_step=ms,
                   higher_is_better=True, wall_s_per_gradient=wall,
                   gcell_updates_per_s=cell_updates / (ms / 1e3) / 1e9,
                   config={"workload": W.name, "checkpoint_interval": sim.checkpoint_interval,
                           "checkpoint_plan": {**sim.checkpoint_plan(),
                                               "scheme": "binomial (revolve)" if sim.checkpoint_plan()["slots"]
                                               else "uniform",
                                               "recomputed_per_shot_of_nt": sim.checkpoint_plan()["recomputed"] / W.nt,
                                               "budget_mb": args.checkpoint_budget_mb or None},
                           "misfit": "L2 waveform, ux+uz, " + ("host" if args.host_misfit else "on the device"),
                           "J_per_shot": list(Js),
                           "receivers": int(W.rec_i.size), "shots": nshot},
                   gradient_finite=bool(np.isfinite(gvp).all() and np.isfinite(gvs).all()),
                   gradient_vs_peak_cell=[int(v) for v in np.unravel_index(np.argmax(np.abs(gvs)), gvs.shape)],
                   clocks=clk.summary())
        # Outputs: the vp, vs, rho kernels smoothed with sigma = 5 cells on the device (after the timed region).
        sig = float(W.extra.get("smooth_sigma", 5.0))
        smoothed = {}
        for name, a in (("vp", gvp), ("vs", gvs), ("rho", grho)):
            src_t = torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()
            dst_t = torch.empty_like(src_t)
            sw.smooth_noalloc(src_t.data_ptr(), dst_t.data_ptr(), W.nx, W.nz, sig,
                              torch.cuda.current_stream().cuda_stream)
            smoothed[name] = dst_t.cpu().numpy()
        out["smoothed_kernels"] = {"sigma_cells": sig, "finite": bool(all(np.isfinite(v).all()
                                                                             for v in smoothed.values()))}
        if args.fd_check:
            # Central finite differences of the misfit on seeded cells among the
            # strongest vp sensitivities of the illuminated zone: away (40
            # cells) from the source and receiver lines, whose near field
            # makes the misfit strongly nonlinear in a single cell, and from
            # the absorbing edges.
            rng = np.random.default_rng(1)
            w = int(W.flags["abs_width"])
            zone = np.abs(gvp).copy()
            zone[:, : int(W.sources[0][1]) + 40] = 0.0
            zone[:, W.nz // 2:] = 0.0
            zone[: w + 40, :] = 0.0
            zone[W.nx - w - 40:, :] = 0.0
            strong = np.argsort(zone.ravel())[-2000:]
            cells = [int(c) for c in rng.choice(strong, args.fd_check, replace=False)]

            def misfit(vp):
                sim.upload_model("vp", vp)
                sim.upload_model("vs", W.model["vs"])
                sim.upload_model("rho", W.model["rho"])
                sim.prepare()
                J = 0.0
                for s_ in range(len(W.sources)):
                    sim.forward(s_)
                    J += sw.l2_misfit(sim.traces()[[0, 2]], obs[s_], W.dt)[0]
                return J

            errs = []
            for c in cells:
                i, j = divmod(c, W.nz)
                h = args.fd_h * float(W.model["vp"][i, j])
                vp_p = W.model["vp"].copy()
                vp_p[i, j] += h
                vp_m = W.model["vp"].copy()
                vp_m[i, j] -= h
                fd = (misfit(vp_p) - misfit(vp_m)) / (2 * h)
                errs.append(abs(float(gvp[i, j]) - fd) / max(abs(fd), 1e-300))
            # Directional derivative along the true anomaly's vp shape (many
            # cells at once).  FP32 rounding of the traces makes the misfit
            # noisy in the model at small steps (single-cell differences at
            # this size are limited by it); the directional difference
            # converges as eps grows (at 512^2: 22 %, 3.5 %, 1.6 %, 0.5 % off
            # for eps 1e-3, 3e-3, 1e-2, 3e-2, against a gradient that matches
            # the FP64 oracle's exact gradient to 2e-4).
            dm = (W.extra["true_model"]["vp"].astype(np.float64) - W.model["vp"]).astype(np.float64)
            eps = 3e-2
            jp = misfit((W.model["vp"] + eps * dm).astype(np.float32))
            jm = misfit((W.model["vp"] - eps * dm).astype(np.float32))
            fd_dir = (jp - jm) / (2 * eps)
            g_dir = float((gvp.astype(np.float64) * dm).sum())
            out["fd_check"] = {"cells": len(cells), "h": f"{100 * args.fd_h:g} % of vp", "max_rel_err": float(max(errs)),
                               "median_rel_err": float(np.median(errs)),
                               "zone": "top |g_vp| cells 40+ cells from sources, receivers and absorbing edges",
                               "directional": {"direction": "true vp anomaly", "eps": eps, "fd": fd_dir,
                                               "gradient": g_dir,
                                               "rel_err": abs(g_dir - fd_dir) / max(abs(fd_dir), 1e-300)}}
        sim.close()
        if not args.no_cpu:
            ns = 24
            r, dtm, thr = cpu_gradient_rate(W, ns)
            out["cpu_baseline"] = {"value": r * 1e9 / cell_updates, "unit": "gradients/s", "cores": thr,
                                   "kind": "port", "gcell_updates_per_s": r,
                                   "sample": f"full grid, one shot, {ns} of {W.nt} steps (FP32 oracle exact "
                                             f"gradient, every step's strains kept, OpenMP), {dtm:.1f} s; "
                                             f"extrapolated to {nshot} shots x {W.nt} steps by cell-updates"}
    elif args.workload == "c5":
        problems = configs.c5_batch(count=args.count, lo=min(256, args.c5_hi), hi=args.c5_hi,
                                    nt_lo=min(1000, args.c5_nt_hi), nt_hi=args.c5_nt_hi)
        comps = [[0, 2] if w.flags["psv"] else [1] for w in problems]
        obs = []
        for w, c in zip(problems, comps):   # observed data from the true models (untimed)
            st = w.make_sim(model=w.extra["true_model"])
            o = []
            for s in range(len(w.sources)):
                st.forward(s)
                o.append(st.traces()[c])
            st.close()
            obs.append(np.array(o))
        sims = [w.make_sim() for w in problems]
        nshots = sum(len(w.sources) for w in problems)
        # plain path: one problem and one shot at a time, host misfit (as the
        # reference's solver.rs:432-467); each problem once untimed (graph
        # capture, buffers), then timed.
        plain = []
        plain_s = 0.0
        for w, sim, o, c in zip(problems, sims, obs, comps):
            for rep in range(2):
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                sim.gradient_clear()
                for s in range(len(w.sources)):
                    sim.forward_op(s, 0)
                    _, adj = sw.l2_misfit(sim.traces()[c], o[s], w.dt)
                    sim.backward_op(adj)
                sim.synchronize()
                if rep == 1:
                    plain_s += time.perf_counter() - t0
            plain.append(sim.gradient("mu"))
            sim.release_workspace()
        batch = sw.Batch(sims, obs)
        if args.concurrent >= 0:
            batch.set_option("concurrent", args.concurrent)
        if args.stream_groups > 0:
            batch.set_option("stream_groups", args.stream_groups)
        if args.tma >= 0:
            batch.set_option("tma", args.tma)
        if args.queue_band >= 0:
            batch.set_option("queue_band", args.queue_band)
        if args.pdl >= 0:
            batch.set_option("pdl", args.pdl)
        if args.checkpoint_slots:
            batch.set_option("checkpoint_slots", args.checkpoint_slots)
        if args.two_step_recompute >= 0:
            batch.set_option("two_step_recompute", args.two_step_recompute)
        if args.reverse_producer >= 0:
            batch.set_option("reverse_producer", args.reverse_producer)
        tune_ms = None
        if args.autotune:
            t0 = time.perf_counter()
            batch.set_option("autotune", 48)
            tune_ms = (time.perf_counter() - t0) * 1e3
        elif args.chunk_rows:
            batch.set_option("chunk_rows", args.chunk_rows)
        stream = torch.cuda.ExternalStream(batch.stream)
        t0 = time.perf_counter()
        batch.run()                       # captures and instantiates the graph
        first_s = time.perf_counter() - t0
        for _ in range(max(0, args.warmup - 1)):
            batch.run()
        with Clocks(0) as clk:
            t0 = time.perf_counter()
            ms = _timed(stream, batch.run, args.steps)
            wall = (time.perf_counter() - t0) / args.steps
        errs = [rel_err for rel_err in (float(np.linalg.norm(batch.gradient(i, "mu") - plain[i]) /
                                              max(np.linalg.norm(plain[i]), 1e-30)) for i in range(len(problems)))]
        info = batch.info()
        cells = sum(2.0 * w.cells * w.nt * len(w.sources) for w in problems)
        out.update(metric="gradients/s", value=len(problems) / (wall), unit="problem-gradients/s",
                   ms_per_step=wall * 1e3, higher_is_better=True,
                   batched={"problem_gradients_per_s": len(problems) / wall, "shot_gradients_per_s": nshots / wall,
                            "gcell_updates_per_s": cells / wall / 1e9, "seconds": wall, "event_ms": ms,
                            "first_run_s_with_graph_capture": first_s},
                   plain={"problem_gradients_per_s": len(problems) / plain_s, "shot_gradients_per_s": nshots / plain_s,
                          "gcell_updates_per_s": cells / plain_s / 1e9, "seconds": plain_s},
                   speedup=plain_s / wall, max_rel_l2_mu_vs_plain=max(errs),
                   config={"workload": f"c5: {len(problems)} problems, {min(256, args.c5_hi)}..{args.c5_hi} per axis, "
                                       f"nt {min(1000, args.c5_nt_hi)}..{args.c5_nt_hi}, SH/PSV, "
                                       "1-4 shots",
                           "jobs": info["jobs"], "slots": info["slots"], "launches_per_run": info["launches_per_run"],
                           "device_bytes": info["device_bytes"],
                           "checkpoints": (f"binomial (revolve), {info['checkpoint_slots']} states per job"
                                           if info["checkpoint_slots"] else "ceil(sqrt(nt)) per job"),
                           "recomputed_steps_per_run": info["recomputed_steps"],
                           "chunk_rows": info.get("chunk_rows"), "two_step_recording": info.get("two_step"),
                           "concurrent": info.get("concurrent"), "stream_groups": info.get("stream_groups"),
                           "queue_units": info.get("queue_units"), "queue_blocks": info.get("queue_blocks"),
                           "queue_band": info.get("queue_band"),
                           "tma_jobs": info.get("tma_jobs"), "autotune_ms": tune_ms},
                   clocks=clk.summary())
        if not args.no_cpu:
            small = min(range(len(problems)), key=lambda q: problems[q].cells)
            ns = min(problems[small].nt, 300)
            r, dtm, thr = cpu_gradient_rate(problems[small], ns)
            out["cpu_baseline"] = {"value": r * 1e9 / cells * len(problems), "unit": "problem-gradients/s",
                                   "cores": thr, "kind": "port", "gcell_updates_per_s": r,
                                   "sample": f"smallest problem ({problems[small].nx}x{problems[small].nz}), one "
                                             f"shot, {ns} of {problems[small].nt} steps (FP32 oracle exact "
                                             f"gradient, OpenMP), {dtm:.1f} s; extrapolated to all {len(problems)} problems "
                                             f"by cell-updates"}
        batch.close()
        for s in sims:
            s.close()
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--nt", type=int, default=4000)
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--ref-sample", type=int, default=600, help="oracle steps in the CPU sample (~10 s)")
    ap.add_argument("--chunk-rows", type=int, default=0)
    ap.add_argument("--grid", type=int, default=4096, help="grid edge (4096 = the headline workload)")
    ap.add_argument("--physics", default="psv", choices=["psv", "sh"],
                    help="c2 grid and model with the SH system instead (the SH step kernel at scale)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-parity", action="store_true")
    ap.add_argument("--no-others", action="store_true",
                    help="c2: skip the other configurations' lines embedded after the headline (other_configs)")
    ap.add_argument("--parity-nt", type=int, default=60, help="c2: steps of the parity run outside the timed region")
    ap.add_argument("--autotune", action="store_true", help="empirical loader/chunk tuning before timing")
    ap.add_argument("--two-step", type=int, default=-1,
                    help="c2: two time steps per launch (1), one (0), or the engine's default (-1: two)")
    ap.add_argument("--two-step-rows", type=int, default=0)
    ap.add_argument("--two-step-producer", type=int, default=-1,
                    help="c2 (PSV): two-step rows fetched by producer warps (1, the default) or by every march (0)")
    ap.add_argument("--reverse-producer", type=int, default=-1,
                    help="c4, c5: PSV reverse-step rows fetched by producer warps (1; the default for c4, not c5) "
                         "or by every march (0)")
    ap.add_argument("--two-step-recompute", type=int, default=-1,
                    help="c5: grouped launches recompute two steps per operation (1) or one (0); -1: the default")
    ap.add_argument("--tma", type=int, default=-1,
                    help="c2, c4, c5: rows of the two-step and reverse kernels by tensor copies (1) or bulk copies (0)")
    ap.add_argument("--pdl", type=int, default=-1,
                    help="c2-c5: step launches may start while the previous one finishes (1, the engine's "
                         "default) or not (0)")
    ap.add_argument("--count", type=int, default=48, help="c5: number of problems (48 = the configuration)")
    ap.add_argument("--c5-hi", type=int, default=1536,
                    help="c5: largest grid edge (1536 = the configuration; smaller for profiling captures)")
    ap.add_argument("--c5-nt-hi", type=int, default=3000,
                    help="c5: most time steps (3000 = the configuration; smaller for profiling captures)")
    ap.add_argument("--queue-band", type=int, default=-1,
                    help="c5: slots per band of the device queue's order (0 slot-major; -1: the default)")
    ap.add_argument("--stream-groups", type=int, default=0, help="c5: job groups with their own streams (0: default)")
    ap.add_argument("--concurrent", type=int, default=-1,
                    help="c5: 0 serial grouped launches, 1 a slot's kinds on forked streams, 2 one stream per "
                         "kind, 3 one persistent launch over a device queue (-1: the default, 2)")
    ap.add_argument("--fd-check", type=int, default=0, help="c4: finite-difference check on this many cells")
    ap.add_argument("--checkpoint-slots", type=int, default=0,
                    help="c4, c5: binomial checkpointing with this many stored states (per shot / per job)")
    ap.add_argument("--checkpoint-budget-mb", type=int, default=0,
                    help="c4: the memory the default checkpoint choice may use (binomial below sqrt(nt) states)")
    ap.add_argument("--host-misfit", action="store_true", help="c4: misfit and adjoint source on the host")
    ap.add_argument("--fd-h", type=float, default=1e-3, help="c4: relative vp step of the finite differences")
    ap.add_argument("--workload", default="c2", choices=["c1", "c2", "c3", "c4", "c5"],
                    help="c2 (default) is the headline; the others print their own line")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.warmup < 3:
        print("warning: fewer than 3 warm-up steps", file=sys.stderr)
    if args.impl == "reference":
        run_reference(args, rank)
        return
    if args.workload != "c2":
        if args.nt == 4000:
            args.nt = 0  # each configuration's own nt
        run_secondary(args)
        return
    if world > 1:
        import torch.distributed as tdist

        tdist.init_process_group("nccl")
    try:
        run_ours(args, rank, world)
    finally:
        if world > 1:
            import torch.distributed as tdist

            tdist.destroy_process_group()


if __name__ == "__main__":
    main()
