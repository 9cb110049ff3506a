"""Exact discrete adjoint on the GPU (fd_adjoint.cu, checkpointed reverse
sweep) against the FP64 oracle adjoint, finite differences of the FP32
misfit, and invariance under the checkpoint interval."""
import numpy as np
import pytest

from tests.examples import rel_l2

pytestmark = pytest.mark.gpu

NX, NZ, NT, DX, DT = 70, 150, 260, 10.0, 1.5e-3


def _problem(phys, seed=0):
    rng = np.random.default_rng(seed)
    vp = (3000 * (1 + 0.05 * np.tanh(rng.standard_normal((NX, NZ))))).astype(np.float32)
    vs = (vp / np.sqrt(3)).astype(np.float32)
    rho = (2500 * (1 + 0.03 * np.tanh(rng.standard_normal((NX, NZ))))).astype(np.float32)
    flags = dict(sh=phys == "sh", psv=phys == "psv", abs_left=True, abs_right=True, abs_bottom=True, abs_width=12)
    src = [(20, 40, 25.0, 0.04, 30.0), (50, 100, 20.0, 0.05, 60.0)]
    rec = [(i, 20) for i in range(4, 67, 7)] + [(60, 140), (10, 130)]
    return vp, vs, rho, flags, src, rec


def _sim(vp, vs, rho, flags, src, rec):
    import seiswg_gb300 as sw

    sim = sw.Sim(NX, NZ, NT, DX, DX, DT, **flags)
    sim.upload_model("vp", vp)
    sim.upload_model("vs", vs)
    sim.upload_model("rho", rho)
    sim.prepare()
    stf = np.stack([sw.ricker(NT, DT, s[2], s[3], s[4], 1.0e10) for s in src], axis=1)
    sim.set_sources([s[0] for s in src], [s[1] for s in src], stf)
    sim.set_receivers([r[0] for r in rec], [r[1] for r in rec])
    return sim, stf


def _comps(flags):
    return [0, 2] if flags["psv"] else [1]


def _observed(vp, vs, rho, flags, src, rec, isrc):
    sim, _ = _sim(vp * 1.02, vs * 0.98, rho, flags, src, rec)
    sim.forward(isrc)
    obs = sim.traces()[_comps(flags)]
    sim.close()
    return obs


def _gpu_gradient(sim, flags, obs, isrc, ckpt):
    import seiswg_gb300 as sw

    sim.gradient_clear()
    sim.forward_op(isrc, ckpt)
    syn = sim.traces()[_comps(flags)]
    J, adj = sw.l2_misfit(syn, obs, DT)
    sim.backward_op(adj)
    return J, adj, {p: sim.gradient(p) for p in ("lambda", "mu", "buoyancy")}


@pytest.mark.parametrize("phys", ["psv", "sh"])
def test_gradient_matches_fp64_oracle(phys):
    from oracle import oracle as O

    vp, vs, rho, flags, src, rec = _problem(phys)
    obs = _observed(vp, vs, rho, flags, src, rec, 0)
    sim, stf = _sim(vp, vs, rho, flags, src, rec)
    J, adj, g = _gpu_gradient(sim, flags, obs, 0, 0)
    sim.close()
    s = O.Setup(NX, NZ, NT, DX, DX, DT, **flags)
    o = O.FD2DOracle(s, np.array([x[0] * NZ + x[1] for x in src]), stf.astype(np.float64),
                     np.array([r[0] * NZ + r[1] for r in rec], np.int32), 64)
    o.set_field("LAM", vp)
    o.set_field("MU", vs)
    o.set_field("RHO", rho)
    o.init_model()
    o.run_forward(0)
    syn64 = np.stack([o.obs(c) for c in (("X", "Z") if flags["psv"] else ("Y",))])
    J64, adj64 = O.l2_misfit(syn64, obs, DT)
    gl, gm, gb = o.exact_gradient(adj64, 0)
    assert abs(J - J64) <= 1e-4 * J64
    assert rel_l2(g["mu"], gm) <= 1e-4
    assert rel_l2(g["buoyancy"], gb) <= 1e-4
    if flags["psv"]:
        assert rel_l2(g["lambda"], gl) <= 1e-4


@pytest.mark.parametrize("phys", ["psv", "sh"])
def test_checkpoint_interval_does_not_change_the_gradient(phys):
    """With one-step forward launches the recorded and the recomputed states
    are the same bits whatever the interval, so the gradient is bitwise equal.
    The default records two steps per launch (multiply-add contraction)
    between checkpoints, which changes the states by rounding only."""
    vp, vs, rho, flags, src, rec = _problem(phys, 1)
    obs = _observed(vp, vs, rho, flags, src, rec, -1)
    sim, _ = _sim(vp, vs, rho, flags, src, rec)
    sim.set_option("two_step", 0)
    ref = _gpu_gradient(sim, flags, obs, -1, 1)[2]       # every state stored
    for k in (2, 7, 0, NT):                             # 2 and 7 steps, the default, one interval
        g = _gpu_gradient(sim, flags, obs, -1, k)[2]
        for p in g:
            assert np.array_equal(g[p], ref[p]), (k, p)
    sim.set_option("two_step", 1)
    for k in (2, 7, 0, NT):
        g = _gpu_gradient(sim, flags, obs, -1, k)[2]
        for p in (("lambda", "mu", "buoyancy") if phys == "psv" else ("mu", "buoyancy")):
            assert rel_l2(g[p], ref[p]) <= 1e-5, (k, p)
    sim.close()


@pytest.mark.parametrize("phys,nt", [("psv", 259), ("psv", 260), ("sh", 259)])
def test_every_state_kept_by_the_two_step_recording(phys, nt):
    """Every state kept (k = 1) with two steps per recording launch: the
    launches store the state between their two steps, an odd last step runs
    alone, nothing is recomputed, and the gradient is the one of one-step
    recording with every state kept to FP32 rounding (the two-step kernel
    contracts multiply-adds), the same bits on a second run."""
    import seiswg_gb300 as sw

    vp, vs, rho, flags, src, rec = _problem(phys, 3)
    stf = np.stack([sw.ricker(nt, DT, s[2], s[3], s[4], 1.0e10) for s in src], axis=1)
    sim = sw.Sim(NX, NZ, nt, DX, DX, DT, **flags)
    for k, v in (("vp", vp), ("vs", vs), ("rho", rho)):
        sim.upload_model(k, v)
    sim.prepare()
    sim.set_sources([s[0] for s in src], [s[1] for s in src], stf)
    sim.set_receivers([r[0] for r in rec], [r[1] for r in rec])
    sim.forward(-1)
    obs = 0.8 * sim.traces()[_comps(flags)]
    out = {}
    for two in (0, 1, 1):
        sim.set_option("two_step", two)
        sim.gradient_clear()
        sim.forward_op(-1, 1)
        plan = sim.checkpoint_plan()
        assert plan["interval"] == 1 and plan["recomputed"] == 0, plan
        _, adj = sw.l2_misfit(sim.traces()[_comps(flags)], obs, DT)
        sim.backward_op(adj)
        g = {p: sim.gradient(p) for p in (("lambda", "mu", "buoyancy") if phys == "psv" else ("mu", "buoyancy"))}
        if two in out:
            for p in g:
                assert np.array_equal(g[p], out[two][p]), p
        out[two] = g
    sim.close()
    for p, ref in out[0].items():
        assert np.abs(ref).max() > 0
        assert rel_l2(out[1][p], ref) <= 1e-5, (p, rel_l2(out[1][p], ref))


def test_checkpoint_allocation_failure_falls_back_to_a_smaller_scheme():
    """A budget above the device's memory: the every-state scheme of a 2048^2
    PSV run of 4000 steps (about 344 GB) fails to allocate -- an error return
    of the allocator, nothing on the device -- and forward_op takes the next
    scheme that fits (every second state, about 172 GB); the reverse sweep
    then runs on it."""
    import seiswg_gb300 as sw

    n, nt, dt = 2048, 4000, 5e-4
    sim = sw.Sim(n, n, nt, 5.0, 5.0, dt, psv=True, abs_left=True, abs_right=True, abs_bottom=True, abs_width=20)
    try:
        sim.upload_model("vp", np.full((n, n), 3000.0, np.float32))
        sim.upload_model("vs", np.full((n, n), 1732.0, np.float32))
        sim.upload_model("rho", np.full((n, n), 2600.0, np.float32))
        sim.prepare()
        sim.set_sources([n // 2], [60], sw.ricker(nt, dt, 15.0, 0.08, 0.0, 1.0e10)[:, None, :])
        sim.set_receivers(list(range(100, n - 100, 64)), [40] * len(range(100, n - 100, 64)))
        sim.set_option("checkpoint_budget_mb", 10 << 20)  # 10 TiB
        sim.gradient_clear()
        sim.forward_op(0, 0)
        plan = sim.checkpoint_plan()
        assert plan["interval"] == 2 and plan["slots"] == 0, plan
        syn = sim.traces()[[0, 2]]
        assert np.isfinite(syn).all() and np.abs(syn).max() > 0
        _, adj = sw.l2_misfit(syn, 0.5 * syn, dt)
        sim.backward_op(adj)
        g = sim.gradient("mu")
        assert np.isfinite(g).all() and np.abs(g).max() > 0
    finally:
        sim.close()


def test_psv_gradient_matches_finite_differences_of_fp32_misfit():
    import seiswg_gb300 as sw

    vp, vs, rho, flags, src, rec = _problem("psv", 2)
    obs = _observed(vp, vs, rho, flags, src, rec, 1)
    sim, _ = _sim(vp, vs, rho, flags, src, rec)
    _, _, g = _gpu_gradient(sim, flags, obs, 1, 0)
    sim.close()
    gvp, gvs, grho = sw.velocity_gradients(g["lambda"], g["mu"], g["buoyancy"], vp, vs, rho)
    grads = dict(vp=gvp, vs=gvs, rho=grho)
    rng = np.random.default_rng(5)
    # cells where the sensitivity is large (illuminated), seeded
    mag = np.abs(gvs)
    cand = np.argwhere(mag > 0.2 * mag.max())
    picks = cand[rng.choice(len(cand), 16, replace=False)]
    for q, (i, j) in enumerate(picks):
        name = ("vp", "vs", "rho")[q % 3]
        base = dict(vp=vp, vs=vs, rho=rho)
        h = np.float32(2e-3) * base[name][i, j]

        def J_of(sign):
            m = {k: v.copy() for k, v in base.items()}
            m[name][i, j] += sign * h
            s, _ = _sim(m["vp"], m["vs"], m["rho"], flags, src, rec)
            s.forward(1)
            syn = s.traces()[[0, 2]]
            s.close()
            return sw.l2_misfit(syn, obs, DT)[0]

        fd = (J_of(1) - J_of(-1)) / (2 * float(h))
        assert abs(grads[name][i, j] - fd) <= 2e-2 * abs(fd), (name, i, j, grads[name][i, j], fd)


def test_gradients_accumulate_over_shots_and_scale_linearly():
    vp, vs, rho, flags, src, rec = _problem("psv", 3)
    sim, _ = _sim(vp, vs, rho, flags, src, rec)
    rng = np.random.default_rng(4)
    adj = [rng.standard_normal((2, len(rec), NT)).astype(np.float32) for _ in range(2)]
    parts = []
    for s in range(2):
        sim.gradient_clear()
        sim.forward_op(s, 0)
        sim.backward_op(adj[s])
        parts.append(sim.gradient("mu"))
    sim.gradient_clear()
    for s in range(2):
        sim.forward_op(s, 0)
        sim.backward_op(adj[s])
    both = sim.gradient("mu")
    assert rel_l2(both, parts[0] + parts[1]) <= 1e-6
    sim.gradient_clear()
    sim.forward_op(0, 0)
    sim.backward_op(2.0 * adj[0])
    assert rel_l2(sim.gradient("mu"), 2.0 * parts[0]) <= 1e-6
    sim.close()


@pytest.mark.parametrize("phys", ["psv", "sh"])
def test_device_misfit_matches_host_misfit(phys):
    """misfit_op + backward_op_device (traces and adjoint source stay on the
    GPU) against l2_misfit on downloaded traces + backward_op."""
    vp, vs, rho, flags, src, rec = _problem(phys, seed=5)
    obs = _observed(vp, vs, rho, flags, src, rec, 1)
    sim, _ = _sim(vp, vs, rho, flags, src, rec)
    try:
        J_host, _, g_host = _gpu_gradient(sim, flags, obs, 1, 0)
        sim.set_observed(obs)
        sim.gradient_clear()
        sim.forward_op(1, 0)
        J_dev = sim.misfit_op()
        sim.backward_op_device()
        g_dev = {p: sim.gradient(p) for p in ("lambda", "mu", "buoyancy")}
        with pytest.raises(Exception):
            sim.forward_op(1, 0)
            sim.backward_op_device()   # no misfit_op since the last forward_op
    finally:
        sim.close()
    assert abs(J_dev - J_host) <= 1e-12 * abs(J_host)
    for p in ("lambda", "mu") if phys == "psv" else ("mu", "buoyancy"):
        assert rel_l2(g_dev[p], g_host[p]) <= 1e-6, p


def test_exact_gradient_agrees_with_the_reference_imaging_kernel(tmp_path):
    """The reference's adjoint example (SH, 12 shots; its K_MU fixture is the
    WGSL imaging-condition kernel, smoothed with sigma 5) against our exact
    gradient of the same tapered L2 misfit with respect to mu, smoothed the
    same way.  The two are different discretisations of the same sensitivity
    (the reference correlates velocity derivatives every adj_interval steps),
    so the test asks for the same spatial pattern, not equal values."""
    import torch

    import seiswg_gb300 as sw
    from tests.examples import golden, write_example

    d = tmp_path / "adjoint"
    write_example("adjoint", str(d))
    g = golden("adjoint")
    with sw.Solver(sw.Config.load(str(d / "config_true.ini"))) as s:
        s.run_forward()
    with sw.Solver(sw.Config.load(str(d / "config.ini"))) as s:
        sim = s.sim
        nshot, dt = s.info()["nsrc"], float(np.float32(0.06))
        sim.gradient_clear()
        for shot in range(nshot):
            sim.forward_op(shot, 0)
            syn = sim.traces()[[1]]
            obs = np.load(d / "obs_traces" / f"uy_{shot:06d}.npy")[None]
            _, adj = sw.l2_misfit(syn, obs, dt)
            sim.backward_op(adj)
        g_mu = sim.gradient("mu")
    nx, nz = g_mu.shape
    src = torch.from_numpy(np.ascontiguousarray(g_mu)).cuda()
    dst = torch.empty_like(src)
    sw.smooth_noalloc(src.data_ptr(), dst.data_ptr(), nx, nz, 5.0, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    ours = dst.cpu().numpy().astype(np.float64).ravel()
    ref = g["fix_proc000000_kmu"].astype(np.float64).ravel()
    corr = abs(float(ours @ ref / (np.linalg.norm(ours) * np.linalg.norm(ref))))
    print(f"corr(exact g_mu, reference K_MU) = {corr:.3f}")
    assert corr > 0.9, corr  # measured 0.948


def test_gradient_matches_fp64_oracle_in_the_c4_geometry():
    """The C4 set-up (PSV, absorbing on all edges, sources and receivers near
    the top, Gaussian anomaly in the true model) at 320^2, 600 steps, 2
    shots: GPU exact gradient against the FP64 oracle's exact gradient, cell
    by cell and along the anomaly's direction."""
    import seiswg_gb300 as sw
    from oracle import oracle as O
    from seiswg_gb300 import configs
    import bench

    W = configs.c4_psv_adjoint(n=320, nt=600, shots=2)
    st = W.make_sim(model=W.extra["true_model"])
    obs = []
    for s in range(len(W.sources)):
        st.forward(s)
        obs.append(st.traces()[[0, 2]])
    st.close()
    sim = W.make_sim()
    sim.gradient_clear()
    for s in range(len(W.sources)):
        sim.forward_op(s, 0)
        _, adj = sw.l2_misfit(sim.traces()[[0, 2]], obs[s], W.dt)
        sim.backward_op(adj)
    g = {p: sim.gradient(p) for p in ("lambda", "mu", "buoyancy")}
    sim.close()
    ours = sw.velocity_gradients(g["lambda"], g["mu"], g["buoyancy"], W.model["vp"], W.model["vs"], W.model["rho"])
    gl = gm = gb = 0.0
    for s in range(len(W.sources)):
        o = bench.workload_oracle(W, W.nt, precision=64)
        o.run_forward(s)
        syn = np.stack([o.obs("X"), o.obs("Z")])
        _, adj = O.l2_misfit(syn, obs[s].astype(np.float64), W.dt)
        a, b, c = o.exact_gradient(adj, s)
        gl, gm, gb = gl + a, gm + b, gb + c
    ref = O.lame_to_velocity_gradients(gl, gm, gb, W.model["vp"], W.model["vs"], W.model["rho"])
    for k, name in enumerate(("vp", "vs", "rho")):
        assert rel_l2(ours[k], ref[k]) <= 1e-3, name
    dm = W.extra["true_model"]["vp"].astype(np.float64) - W.model["vp"]
    d_ours, d_ref = float((ours[0] * dm).sum()), float((ref[0] * dm).sum())
    assert abs(d_ours - d_ref) <= 1e-3 * abs(d_ref)


def test_exact_gradient_and_reference_adjoint_share_a_sim():
    """The exact gradient, then the reference's SH imaging-condition adjoint
    (its forward store sized by adj_interval), then the exact gradient again
    on the same Sim: the workspaces of one path leave the other's intact, so
    the two exact gradients are the same bits."""
    import seiswg_gb300 as sw

    vp, vs, rho, flags, src, rec = _problem("sh", 3)
    obs = _observed(vp, vs, rho, flags, src, rec, 0)
    sim, _ = _sim(vp, vs, rho, flags, src, rec)
    try:
        first = _gpu_gradient(sim, flags, obs, 0, 0)[2]
        for adj_interval in (5, 7):   # two store sizes: the store is resized once
            sim.kernel_clear()
            sim.adjoint_forward(0, adj_interval)
            _, adstf = sw.waveform_misfit(sim.traces()[1], obs[0], DT)   # uy against the observed uy
            sim.adjoint_backward(adstf, adj_interval)
            assert np.isfinite(sim.kernel()).all()
        again = _gpu_gradient(sim, flags, obs, 0, 0)[2]
        for p in first:
            assert np.array_equal(first[p], again[p]), p
    finally:
        sim.close()


def test_reverse_step_tensor_copies_give_the_same_gradient():
    """The PSV reverse step (and the two-step recording) with rows fetched by
    tensor copies or by one bulk copy per field: the same bits."""
    vp, vs, rho, flags, src, rec = _problem("psv", 4)
    obs = _observed(vp, vs, rho, flags, src, rec, -1)
    sim, _ = _sim(vp, vs, rho, flags, src, rec)
    try:
        g = []
        for tma in (1, 0):
            sim.set_option("tma", tma)
            g.append(_gpu_gradient(sim, flags, obs, -1, 0)[2])
        for p in g[0]:
            assert np.abs(g[0][p]).max() > 0
            assert np.array_equal(g[0][p], g[1][p]), p
    finally:
        sim.close()


def _revolve_cost(n, s):
    """F(n, s) of binomial checkpointing (Griewank and Walther's revolve):
    forward steps that reverse n steps from the first state with s more
    free slots."""
    from math import comb

    if n <= 1:
        return 0
    if s <= 0:
        return n * (n - 1) // 2
    r = 0
    while comb(s + 1 + r, r) < n:
        r += 1
    return r * n - comb(s + 1 + r, r - 1)


@pytest.mark.parametrize("phys", ["psv", "sh"])
def test_binomial_checkpointing_gives_the_uniform_gradient(phys):
    """With one-step recording every stored or recomputed state is the same
    bits whatever the schedule, so binomial checkpointing with any number of
    slots gives the gradient of uniform checkpoints bit for bit, recomputing
    exactly F(nt, S-1) - (nt - 1) steps.  With the default two-step recording
    the states differ by rounding only."""
    vp, vs, rho, flags, src, rec = _problem(phys, 3)
    obs = _observed(vp, vs, rho, flags, src, rec, -1)
    sim, _ = _sim(vp, vs, rho, flags, src, rec)
    sim.set_option("two_step", 0)
    ref = _gpu_gradient(sim, flags, obs, -1, 1)[2]
    params = ("lambda", "mu", "buoyancy") if phys == "psv" else ("mu", "buoyancy")
    for S in (1, 2, 3, 7, 40, NT):
        sim.set_option("checkpoint_slots", S)
        g = _gpu_gradient(sim, flags, obs, -1, 0)[2]
        plan = sim.checkpoint_plan()
        assert plan["slots"] == S and plan["interval"] == 0
        assert plan["recomputed"] == _revolve_cost(NT, S - 1) - (NT - 1), (S, plan)
        for p in params:
            assert np.array_equal(g[p], ref[p]), (S, p)
    sim.set_option("two_step", 1)
    for S in (2, 13):
        sim.set_option("checkpoint_slots", S)
        g = _gpu_gradient(sim, flags, obs, -1, 0)[2]
        for p in params:
            assert rel_l2(g[p], ref[p]) <= 1e-5, (S, p)
    sim.close()


def test_checkpoint_budget_selects_the_scheme():
    """The default scheme under a memory budget: every state where nt + 1
    fit (nothing recomputed; the two-step launches store the state between
    their steps), every second step where that fits, every ceil(sqrt(nt))
    steps where that fits, else binomial checkpointing with as many states as
    fit (the same gradient)."""
    vp, vs, rho, flags, src, rec = _problem("psv", 4)
    obs = _observed(vp, vs, rho, flags, src, rec, 0)
    sim, _ = _sim(vp, vs, rho, flags, src, rec)
    ref = _gpu_gradient(sim, flags, obs, 0, 1)[2]
    g0 = _gpu_gradient(sim, flags, obs, 0, 0)[2]
    plan = sim.checkpoint_plan()
    assert plan["interval"] == 1 and plan["slots"] == 0 and plan["recomputed"] == 0, plan  # every state fits
    state = plan["bytes"] / (NT + 1)
    for states, want in ((NT // 2 + 8, "second"), (40, "sqrt"), (12, "binomial")):
        sim.set_option("checkpoint_budget_mb", max(1, int(states * state) >> 20))
        g = _gpu_gradient(sim, flags, obs, 0, 0)[2]
        plan = sim.checkpoint_plan()
        if want == "second":
            assert plan["interval"] == 2 and plan["slots"] == 0, plan
        elif want == "sqrt":
            assert plan["interval"] == int(np.ceil(np.sqrt(NT))) and plan["slots"] == 0, plan
        else:
            assert plan["slots"] >= 1 and plan["interval"] == 0 and plan["bytes"] <= states * state, plan
        for p in ("lambda", "mu", "buoyancy"):
            assert rel_l2(g[p], ref[p]) <= 1e-5 and rel_l2(g0[p], ref[p]) <= 1e-5
    sim.close()
