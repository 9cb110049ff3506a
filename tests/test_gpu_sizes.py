"""The CUDA path against the oracles at the benchmark configurations' own grid
sizes, with fewer time steps so that the CPU oracles finish in seconds:

  C2  PSV forward 4096 x 4096 (heterogeneous, absorbing width 40, the
      headline two-step kernel with tensor copies), 400 steps
  C3  PSV + spin 2048 x 2048 (the spin kernel), 100 steps
  C4  PSV exact gradient 2048 x 2048, one shot, 60 steps, checkpointed: the
      gradient against the FP64 oracle's exact gradient, and the vp / vs /
      rho gradients against central differences of the FP64 misfit on 16
      seeded cells of the illuminated zone

and, at the full sizes and step counts, properties that need no oracle: the
whole C2 run is deterministic and linear in the source, and one whole C4
shot gradient is deterministic.

Traces and final states are held to relative L2 <= 1e-5 against the FP32
oracle (the spin rotation yi to 3x the oracle's own distance from FP64,
tests/test_gpu_parity.py); the distance from the FP64 oracle is reported.
The metric follows the reference's own comparison of a run against its
fixtures (tests/integration.rs:153-190)."""
import numpy as np
import pytest

from tests.examples import rel_l2
from tests.test_gpu_parity import _check_plain, _STATE, _ORACLE_SLOT

pytestmark = pytest.mark.gpu


def _oracle(w, prec, rec_i, rec_j, isrc=-1, model=None):
    from oracle import oracle as O

    s = O.Setup(w.nx, w.nz, w.nt, w.dx, w.dz, w.dt, **w.flags)
    src_k = np.array([x[0] * w.nz + x[1] for x in w.sources])
    o = O.FD2DOracle(s, src_k, w.stf().astype(np.float64), np.asarray(rec_i) * w.nz + np.asarray(rec_j), prec)
    for k, v in (model or w.model).items():
        o.set_field(_ORACLE_SLOT[k], v)
    o.init_model()
    o.run_forward(isrc)
    return o


def _pair(w, rec_i, rec_j, fields):
    import seiswg_gb300 as sw  # noqa: F401

    sim = w.make_sim()
    sim.set_receivers(rec_i, rec_j)
    sim.forward(-1)
    gpu = dict(traces=sim.traces(), state={f: sim.state(f) for f in fields})
    sim.close()
    ref = {}
    for prec in (32, 64):
        o = _oracle(w, prec, rec_i, rec_j)
        ref[prec] = dict(obs=np.stack([o.obs(c) for c in ("X", "Y", "Z", "YI", "YC")]),
                         state={f: o.field(_STATE[f]) for f in fields})
        del o
    return gpu, ref


def test_c2_full_grid():
    """4096 x 4096.  The configuration's 256 receivers lie on the top row,
    which the edge rule decouples from the grid: their traces stay exactly
    zero, on the GPU as in the oracle.  Sixteen receivers on a line ten cells
    below the source record the first arrivals within the 400 steps."""
    from seiswg_gb300 import configs

    w = configs.c2_psv_forward(nt=400)
    si, sj = w.sources[0][0], w.sources[0][1]
    deep_i = np.arange(si - 30, si + 34, 4, dtype=np.int32)
    rec_i = np.concatenate([w.rec_i, deep_i])
    rec_j = np.concatenate([w.rec_j, np.full(deep_i.size, sj + 10, np.int32)])
    gpu, ref = _pair(w, rec_i, rec_j, ("vx", "vz", "sxx", "szz", "sxz"))
    top = slice(0, w.rec_i.size)
    for c in (0, 2):
        assert not np.any(gpu["traces"][c][top]) and not np.any(ref[64]["obs"][c][top])
        assert np.abs(gpu["traces"][c][top.stop:]).max() > 0
    _check_plain(gpu, ref, w.flags)


def test_c3_full_grid():
    """2048 x 2048 PSV + spin: ux, uz, ry, yi, yc traces of the configuration's
    64 receivers at mid-depth (the two nearest the source see the first
    arrivals within 100 steps) and all nine state fields."""
    from seiswg_gb300 import configs

    w = configs.c3_spin_forward(nt=100)
    gpu, ref = _pair(w, w.rec_i, w.rec_j, ("vx", "vz", "sxx", "szz", "sxz", "vyc", "syx", "syy", "syz"))
    assert np.abs(gpu["traces"][0]).max() > 0
    _check_plain(gpu, ref, w.flags)


def test_c4_full_grid_gradient():
    """2048 x 2048, the first shot, 60 steps, checkpoints every second step
    (the default where HBM allows it).  Observed traces from the true model
    (oracle, FP64); the GPU gradient of the L2 misfit against the FP64
    oracle's exact gradient for the same adjoint source, and against central
    differences of the FP64 misfit."""
    import seiswg_gb300 as sw
    from oracle import oracle as O
    from seiswg_gb300 import configs

    w = configs.c4_psv_adjoint(nt=60, shots=8)
    w.sources = w.sources[:1]
    # Within 60 steps the waves reach about 30 cells: the observed data come
    # from a model perturbed there (+5 % vp and vs in a Gaussian of radius 20
    # cells between the source and the first receivers), not from the
    # configuration's deep anomaly, which no wave reaches that soon.
    si, sj = w.sources[0][0], w.sources[0][1]
    ii, jj = np.meshgrid(np.arange(w.nx), np.arange(w.nz), indexing="ij")
    bump = (1.0 + 0.05 * np.exp(-((ii - si - 15) ** 2 + (jj - sj - 10) ** 2) / 20.0 ** 2)).astype(np.float32)
    near = dict(vp=(w.model["vp"] * bump).astype(np.float32), vs=(w.model["vs"] * bump).astype(np.float32),
                rho=w.model["rho"])
    obs_o = _oracle(w, 64, w.rec_i, w.rec_j, model=near)
    obs = np.stack([obs_o.obs("X"), obs_o.obs("Z")]).astype(np.float32)
    del obs_o

    sim = w.make_sim()
    sim.gradient_clear()
    sim.forward_op(0, 0)
    syn = sim.traces()[[0, 2]]
    J, adj = sw.l2_misfit(syn, obs, w.dt)
    sim.backward_op(adj)
    g = {p: sim.gradient(p) for p in ("lambda", "mu", "buoyancy")}
    ck = sim.checkpoint_interval
    sim.close()
    assert J > 0 and ck >= 1

    o = _oracle(w, 64, w.rec_i, w.rec_j)
    syn64 = np.stack([o.obs("X"), o.obs("Z")])
    J64, adj64 = O.l2_misfit(syn64, obs, w.dt)
    assert abs(J - J64) <= 1e-4 * J64
    gl, gm, gb = o.exact_gradient(adj64, 0)
    del o
    for name, a, b in (("lambda", g["lambda"], gl), ("mu", g["mu"], gm), ("buoyancy", g["buoyancy"], gb)):
        assert rel_l2(a, b) <= 1e-4, (name, rel_l2(a, b))

    # central differences of the FP64 misfit on 16 seeded cells where the
    # gradient of the perturbed parameter is at least 0.2 of its largest
    vp, vs, rho = (w.model[k] for k in ("vp", "vs", "rho"))
    gvp, gvs, grho = sw.velocity_gradients(g["lambda"], g["mu"], g["buoyancy"], vp, vs, rho)
    grads = dict(vp=gvp, vs=gvs, rho=grho)
    rng = np.random.default_rng(7)
    errs = []
    for q in range(16):
        name = ("vp", "vs", "rho")[q % 3]
        mag = np.abs(grads[name])
        cand = np.argwhere(mag >= 0.2 * mag.max())
        i, j = cand[rng.integers(len(cand))]
        h = 1e-3 * float(w.model[name][i, j])

        def J_of(sign):
            m = {k: v.astype(np.float64) for k, v in w.model.items()}
            m[name][i, j] += sign * h
            oo = _oracle(w, 64, w.rec_i, w.rec_j, model=m)
            return O.l2_misfit(np.stack([oo.obs("X"), oo.obs("Z")]), obs, w.dt)[0]

        fd = (J_of(1) - J_of(-1)) / (2 * h)
        errs.append(abs(fd - grads[name][i, j]) / abs(fd))
    errs = np.array(errs)
    assert np.median(errs) <= 2e-3 and errs.max() <= 2e-2, errs


def test_c2_full_run_is_deterministic_and_linear_in_the_source():
    """The whole C2 run (4096 x 4096, nt = 4000, the headline two-step kernel)
    checked by properties that need no oracle at this size: two runs give the
    same bits (no race between warps or launches), and the wavefield is linear
    in the source.  With the amplitude doubled every operation on normal
    numbers doubles its result exactly, but the leading edge of a wavefield
    passes through the subnormal range, where a doubled value keeps more
    significant bits, and traces of weak first arrivals carry that difference
    (measured: 4.2e-7 on the deep receivers' ux): the doubled run is held to
    2x the first to the parity tolerance, relative L2 1e-5."""
    from seiswg_gb300 import configs

    w = configs.c2_psv_forward()
    si, sj = w.sources[0][0], w.sources[0][1]
    deep_i = np.arange(si - 600, si + 601, 40, dtype=np.int32)
    rec_i = np.concatenate([w.rec_i, deep_i])
    rec_j = np.concatenate([w.rec_j, np.full(deep_i.size, sj + 300, np.int32)])
    fields = ("vx", "vz", "sxx", "szz", "sxz")

    def run(workload):
        sim = workload.make_sim()
        sim.set_receivers(rec_i, rec_j)
        sim.forward(-1)
        out = [sim.traces()[0], sim.traces()[2]] + [sim.state(f) for f in fields]
        sim.close()
        return out

    a, b = run(w), run(w)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    assert np.abs(a[0][w.rec_i.size:]).max() > 0          # the deep line records the wavefield
    w2 = configs.c2_psv_forward()
    w2.sources = [s[:5] + (2.0 * s[5],) for s in w2.sources]
    d = run(w2)
    for x, y in zip(a, d):
        assert np.all(np.isfinite(y))
        assert rel_l2(y, 2.0 * x) <= 1e-5


def test_c4_full_shot_gradient_is_deterministic():
    """One shot of the C4 gradient at full size (2048 x 2048, nt = 3000:
    two-step recording, checkpoints every second step, recomputation and
    3000 reverse steps): two runs give the same bits."""
    import seiswg_gb300 as sw
    from seiswg_gb300 import configs

    w = configs.c4_psv_adjoint()
    w.sources = w.sources[:1]
    st = w.make_sim(model=w.extra["true_model"])
    st.forward(0)
    obs = st.traces()[[0, 2]]
    st.close()
    sim = w.make_sim()
    grads = []
    for _ in range(2):
        sim.gradient_clear()
        sim.forward_op(0, 0)
        _, adj = sw.l2_misfit(sim.traces()[[0, 2]], obs, w.dt)
        sim.backward_op(adj)
        grads.append([sim.gradient(p) for p in ("lambda", "mu", "buoyancy")])
    sim.close()
    for x, y in zip(*grads):
        assert np.abs(x).max() > 0
        assert np.array_equal(x, y)


def test_c3_full_run_is_deterministic_and_linear_in_the_source():
    """The whole C3 run (2048 x 2048 PSV + spin, nt = 3000, the spin kernel):
    two runs give the same bits, and doubling the source amplitude doubles the
    ux and uz traces and the final vx, vz, sxx and vy_c to the parity
    tolerance (as for C2).  The rotation-related results are left out of the
    linearity check: yi and the couple stress syy are differences of two
    nearly equal quantities (the rotation against half the curl), so the
    leading edge's subnormal-range differences reach them amplified (3e-4 and
    8e-5 measured)."""
    from seiswg_gb300 import configs

    fields = ("vx", "vz", "sxx", "vyc")

    def run(workload):
        sim = workload.make_sim()
        sim.forward(-1)
        tr = sim.traces()
        out = [tr[c] for c in range(tr.shape[0])] + [sim.state(f) for f in fields]
        sim.close()
        return out

    w = configs.c3_spin_forward()
    a, b = run(w), run(w)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    assert np.abs(a[0]).max() > 0
    w2 = configs.c3_spin_forward()
    w2.sources = [s[:5] + (2.0 * s[5],) for s in w2.sources]
    d = run(w2)
    ntr = len(a) - len(fields)
    for k, (x, y) in enumerate(zip(a, d)):
        assert np.all(np.isfinite(y))
        if (k in (0, 2) or k >= ntr) and np.any(x):   # ux, uz, and the state fields
            assert rel_l2(y, 2.0 * x) <= 1e-5, k
