"""Kernels whose rows are fetched by producer warps (fd_producer.cuh) against
the kernels whose marches issue their own copies: the marches are the same
code on the same rows, so the results are bitwise equal.  The two-step PSV
kernel (the Sim option "two_step_producer"): traces, snapshots and the final
state on the cases of the two-step tests (grids narrower than one strip,
strip and chunk boundaries, odd nt, snapshot steps that split a pair,
receivers and sources on the edges, every taper edge, chunks shorter than the
two-step reach) and a grid of many strips and chunks, and the exact gradient,
whose recording launches also store the state between their two steps.  The
PSV reverse step ("reverse_producer" of a Sim and of a Batch): the gradient.
Both: an expired row wait is reported as a timeout and the handle stays
usable."""
import numpy as np
import pytest

from tests.test_gpu_parity import _model
from tests.test_gpu_two_step import CASES, FIELDS, SNAP

pytestmark = pytest.mark.gpu


def _sim(sw, nx, nz, nt, src, rec, pc, rows=0, **flags):
    dt = 1.2e-3
    stf = np.stack([sw.ricker(nt, dt, s[2], s[3], s[4], 1.0e10) for s in src], axis=1)
    sim = sw.Sim(nx, nz, nt, 10.0, 10.0, dt, psv=True, **flags)
    for k, v in _model(nx, nz, 0).items():
        sim.upload_model(k, v)
    sim.prepare()
    sim.set_sources([s[0] for s in src], [s[1] for s in src], stf)
    sim.set_receivers([r[0] for r in rec], [r[1] for r in rec])
    sim.set_option("two_step", 1)
    sim.set_option("two_step_producer", pc)
    if rows:
        sim.set_option("two_step_rows", rows)
    return sim


@pytest.mark.parametrize("case", range(len(CASES)))
def test_forward_is_bitwise_the_self_issuing_kernel(case):
    import seiswg_gb300 as sw

    nx, nz, nt, src, rec, rows, snap, flags = CASES[case]
    out = []
    for pc in (0, 1):
        with _sim(sw, nx, nz, nt, src, rec, pc, rows, **flags) as sim:
            snaps = sim.forward(-1, snap, SNAP["psv"] if snap else [])
            out.append((sim.traces(), snaps, [sim.state(f) for f in FIELDS["psv"]]))
    (t0, s0, f0), (t1, s1, f1) = out
    assert np.abs(t0).max() > 0
    assert np.array_equal(t0, t1)
    assert (s0 is None and s1 is None) or np.array_equal(s0, s1)
    for a, b in zip(f0, f1):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("rows", [0, 6, 40])
def test_large_grid_forward_is_bitwise_the_self_issuing_kernel(rows):
    """A grid of many strips and chunks (the model chunk rows, chunks shorter
    than the reach, long chunks), a source in the interior."""
    import seiswg_gb300 as sw

    nx, nz, nt = 700, 900, 60
    src = [(350, 450, 20.0, 0.03, 0.0), (120, 800, 25.0, 0.03, 30.0)]
    rec = [(i, 300) for i in range(3, 700, 17)] + [(350, j) for j in range(0, 900, 23)]
    flags = dict(abs_left=True, abs_right=True, abs_bottom=True, abs_width=20)
    out = []
    for pc in (0, 1):
        with _sim(sw, nx, nz, nt, src, rec, pc, rows, **flags) as sim:
            sim.forward(-1)
            out.append((sim.traces(), [sim.state(f) for f in FIELDS["psv"]]))
    assert np.array_equal(out[0][0], out[1][0])
    for a, b in zip(out[0][1], out[1][1]):
        assert np.abs(a).max() > 0
        assert np.array_equal(a, b)


def test_gradient_is_bitwise_the_self_issuing_kernel():
    """The exact gradient: every state kept, the recording launches storing
    the state between their two steps (the producer kernel's MID
    instantiation)."""
    import seiswg_gb300 as sw

    nx, nz, nt = 140, 200, 150
    src = [(70, 60, 20.0, 0.05, 30.0)]
    rec = [(i, 100) for i in range(2, nx - 2, 7)]
    grads = []
    for pc in (0, 1):
        with _sim(sw, nx, nz, nt, src, rec, pc, abs_left=True, abs_bottom=True, abs_width=10) as sim:
            sim.gradient_clear()
            sim.forward_op(0, 0)
            syn = sim.traces()[[0, 2]]
            _, adj = sw.l2_misfit(syn, 0.9 * syn, 1.2e-3)
            sim.backward_op(adj)
            grads.append([sim.gradient(p) for p in ("lambda", "mu", "buoyancy")])
    for a, b in zip(grads[0], grads[1]):
        assert np.abs(a).max() > 0
        assert np.array_equal(a, b)


def test_expired_wait_reports_timeout_and_the_handle_recovers():
    """Row 0 of every march armed for 16 bytes more than its copies: each
    march gives up at its first row, its producer at the stage it can no
    longer refill (after counting the extra bytes and waiting for its copies),
    the run reports a timeout, and the same handle then runs normally."""
    import seiswg_gb300 as sw

    nx, nz, nt, src, rec, _, _, flags = CASES[1]
    with _sim(sw, nx, nz, nt, src, rec, 0, **flags) as clean:
        clean.forward(-1)
        want = clean.traces()
    with _sim(sw, nx, nz, nt, src, rec, 1, **flags) as sim:
        sim.set_option("wait_polls", 4096)
        sim.set_option("test_arm_extra", 16)
        with pytest.raises(sw.SeiswgError) as e:
            sim.forward(-1)
        assert e.value.code == sw.ETIMEOUT and "bounded wait" in str(e.value)
        sim.set_option("test_arm_extra", 0)
        sim.set_option("wait_polls", 0)
        sim.forward(-1)
        assert np.array_equal(sim.traces(), want)


@pytest.mark.parametrize("nt", [150, 151])
def test_reverse_step_gradient_is_bitwise_the_self_issuing_kernel(nt):
    """The PSV reverse step with producer warps: the same gradient bits,
    every state kept or every second one (recomputation between)."""
    import seiswg_gb300 as sw

    nx, nz = 140, 230
    src = [(70, 60, 20.0, 0.05, 30.0)]
    rec = [(i, 100) for i in range(2, nx - 2, 7)]
    for k in (0, 2):
        grads = []
        for rp in (0, 1):
            with _sim(sw, nx, nz, nt, src, rec, 1, abs_left=True, abs_bottom=True, abs_width=10) as sim:
                sim.set_option("reverse_producer", rp)
                sim.gradient_clear()
                sim.forward_op(0, k)
                syn = sim.traces()[[0, 2]]
                _, adj = sw.l2_misfit(syn, 0.9 * syn, 1.2e-3)
                sim.backward_op(adj)
                grads.append([sim.gradient(p) for p in ("lambda", "mu", "buoyancy")])
        for a, b in zip(grads[0], grads[1]):
            assert np.abs(a).max() > 0
            assert np.array_equal(a, b), k


def test_reverse_step_expired_wait_reports_timeout_and_the_handle_recovers():
    """Row 0 of every reverse march armed for 16 bytes more than its copies:
    the reverse sweep reports a timeout (read with the gradient), and the same
    handle then gives the gradient of a clean run."""
    import seiswg_gb300 as sw

    nx, nz, nt = 96, 140, 40
    src = [(48, 40, 25.0, 0.04, 30.0)]
    rec = [(i, 70) for i in range(5, nx - 5, 9)]
    with _sim(sw, nx, nz, nt, src, rec, 1, abs_left=True, abs_bottom=True, abs_width=10) as sim:
        sim.set_option("reverse_producer", 1)
        sim.gradient_clear()
        sim.forward_op(0, 0)
        syn = sim.traces()[[0, 2]]
        _, adj = sw.l2_misfit(syn, 0.5 * syn, 1.2e-3)
        sim.backward_op(adj)
        want = sim.gradient("mu")
        assert np.abs(want).max() > 0
        sim.gradient_clear()
        sim.forward_op(0, 0)
        sim.traces()
        sim.set_option("wait_polls", 4096)
        sim.set_option("test_arm_extra", 16)
        sim.backward_op(adj)
        with pytest.raises(sw.SeiswgError) as e:
            sim.gradient("mu")
        assert e.value.code == sw.ETIMEOUT
        sim.set_option("test_arm_extra", 0)
        sim.set_option("wait_polls", 0)
        sim.gradient_clear()
        sim.forward_op(0, 0)
        sim.traces()
        sim.backward_op(adj)
        assert np.array_equal(sim.gradient("mu"), want)


def test_batch_reverse_launches_are_bitwise_the_self_issuing_kernel():
    """The batch's grouped PSV reverse launches with producer warps (the
    Batch option "reverse_producer"; each producer warp finds its march's job
    and op as the march does): the same gradients and misfits, in every
    grouped launch order."""
    import seiswg_gb300 as sw
    from tests.test_gpu_batch import _problems

    probs = _problems()
    sims = [w.make_sim() for (w, _, _) in probs]
    batch = sw.Batch(sims, [obs for (_, obs, _) in probs])
    try:
        ref = None
        for mode, rp in ((2, 0), (2, 1), (0, 1), (1, 1)):
            batch.set_option("concurrent", mode)
            batch.set_option("reverse_producer", rp)
            batch.run()
            g = [batch.gradient(i, p) for i in range(len(probs)) for p in ("lambda", "mu", "buoyancy")]
            J = [batch.misfit(i) for i in range(len(probs))]
            if ref is None:
                ref = (g, J)
                assert any(np.abs(a).max() > 0 for a in g)
                continue
            assert J == ref[1], (mode, rp)
            for a, b in zip(g, ref[0]):
                assert np.array_equal(a, b), (mode, rp)
    finally:
        batch.close()
        for s in sims:
            s.close()
