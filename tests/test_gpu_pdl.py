"""Programmatic dependent launch (the "pdl" option of a Sim and of a Batch,
default on): a step or reverse launch may start while the previous launch in
its stream finishes; its CTAs set up their row pipelines on the SMs that
launch leaves and wait for it to complete before their first read of state.
Only the timing may change: forward traces and final state (one- and
two-step kernels, PSV, SH and spin), the exact gradient (recording,
recomputation and reverse steps) and a batch's gradients (grouped launches in
every launch order) are bitwise equal with the option on and off."""
import numpy as np
import pytest

from tests.test_gpu_parity import _model

pytestmark = pytest.mark.gpu

FIELDS = {"psv": ("vx", "vz", "sxx", "szz", "sxz"), "sh": ("vy", "sxy", "szy"), "spin": ("vx", "vz", "vyc", "syy")}


def _sim(sw, nx, nz, nt, physics, pdl, two):
    spin = physics == "spin"
    # the spin case on the micropolar model and scale of the spin parity tests
    dt, dx, f0, t0 = (1e-4, 1.0, 50.0, 0.024) if spin else (1.2e-3, 10.0, 20.0, 0.05)
    flags = dict(sh=physics == "sh", psv=physics in ("psv", "spin"), spin=spin, abs_left=True,
                 abs_bottom=True, abs_width=10)
    sim = sw.Sim(nx, nz, nt, dx, dx, dt, **flags)
    sim.set_option("cluster", 0)
    sim.set_option("pdl", pdl)
    for k, v in _model(nx, nz, 3, spin=spin).items():
        sim.upload_model(k, v)
    sim.prepare()
    stf = np.stack([sw.ricker(nt, dt, f0, t0, 30.0, 1.0e10)], axis=1)
    sim.set_sources([nx // 2], [nz // 3], stf)
    sim.set_receivers(list(range(2, nx - 2, 7)), [nz // 2] * len(range(2, nx - 2, 7)))
    if physics != "spin":
        sim.set_option("two_step", 1 if two else 0)
    return sim


@pytest.mark.parametrize("physics,two", [("psv", True), ("psv", False), ("sh", True), ("sh", False),
                                         ("spin", False)])
def test_forward_is_the_same_with_and_without_pdl(physics, two):
    import seiswg_gb300 as sw

    out = []
    for pdl in (1, 0):
        with _sim(sw, 150, 260, 120, physics, pdl, two) as sim:
            sim.forward(0)
            out.append((sim.traces(), [sim.state(f) for f in FIELDS[physics]]))
    assert np.array_equal(out[0][0], out[1][0])
    for a, b in zip(out[0][1], out[1][1]):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("physics", ["psv", "sh"])
def test_gradient_is_the_same_with_and_without_pdl(physics):
    import seiswg_gb300 as sw

    comps = [0, 2] if physics == "psv" else [1]
    grads = []
    for pdl in (1, 0):
        with _sim(sw, 140, 200, 150, physics, pdl, True) as sim:
            sim.gradient_clear()
            sim.forward_op(0, 0)
            obs = 0.9 * sim.traces()[comps]
            _, adj = sw.l2_misfit(sim.traces()[comps], obs, 1.2e-3)
            sim.backward_op(adj)
            grads.append([sim.gradient(p) for p in ("lambda", "mu", "buoyancy")])
    for a, b in zip(grads[0], grads[1]):
        assert np.abs(a).max() > 0 or physics == "sh"
        assert np.array_equal(a, b)


def test_batch_is_the_same_with_and_without_pdl():
    import seiswg_gb300 as sw
    from tests.test_gpu_batch import _problems

    probs = _problems()[:3]
    sims = [w.make_sim() for (w, _, _) in probs]
    batch = sw.Batch(sims, [obs for (_, obs, _) in probs])
    try:
        ref = None
        for mode, pdl in ((2, 1), (2, 0), (0, 1), (0, 0)):
            batch.set_option("concurrent", mode)
            batch.set_option("pdl", pdl)
            batch.run()
            g = [batch.gradient(i, p) for i in range(len(probs)) for p in ("mu", "buoyancy")]
            if ref is None:
                ref = g
                continue
            for a, b in zip(g, ref):
                assert np.array_equal(a, b), (mode, pdl)
    finally:
        batch.close()
        for s in sims:
            s.close()
