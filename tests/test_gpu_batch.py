"""Batched gradients of uneven problems (grouped launches by default, one per
schedule slot and kind of work, or one persistent launch over a device work
queue; one CUDA graph per run, misfit on the device) against the plain
per-shot path, problem by problem.  The
tolerance is the gradient accuracy the batched configuration asks for,
relative L2 1e-4; the two paths share their marches, so they agree far
closer."""
import numpy as np
import pytest

from tests.examples import rel_l2

pytestmark = pytest.mark.gpu

# (nx, nz, nt, physics, shots)
PROBLEMS = [(130, 160, 300, "psv", 2), (200, 140, 250, "sh", 1), (96, 300, 220, "psv", 3), (150, 150, 280, "sh", 2)]


def _problems():
    import seiswg_gb300 as sw
    from seiswg_gb300.configs import Workload

    out = []
    rng = np.random.default_rng(7)
    for (nx, nz, nt, phys, shots) in PROBLEMS:
        vp = (3000 * (1 + 0.04 * np.tanh(rng.standard_normal((nx, nz))))).astype(np.float32)
        vs = (vp / np.sqrt(3)).astype(np.float32)
        rho = np.full((nx, nz), 2500.0, np.float32)
        flags = dict(sh=phys == "sh", psv=phys == "psv", abs_left=True, abs_right=True, abs_bottom=True,
                     abs_width=10)
        src = [(int(i), 12, 25.0, 0.04, 20.0 * s, 1.0e10)
               for s, i in enumerate(np.linspace(15, nx - 16, shots).astype(int))]
        rec_i = np.arange(5, nx - 5, 9, dtype=np.int32)
        w = Workload("t", nx, nz, nt, 10.0, 10.0, 1.5e-3, flags, dict(vp=vp, vs=vs, rho=rho), src, rec_i,
                     np.full(rec_i.size, 20, np.int32))
        true = dict(vp=vp * 1.03, vs=vs * 0.97, rho=rho)
        st = w.make_sim(model=true)
        comps = [0, 2] if phys == "psv" else [1]
        obs = []
        for s in range(shots):
            st.forward(s)
            obs.append(st.traces()[comps])
        st.close()
        out.append((w, np.array(obs), comps))
    return out


def _plain(w, obs, comps):
    import seiswg_gb300 as sw

    sim = w.make_sim()
    sim.gradient_clear()
    J = 0.0
    for s in range(len(w.sources)):
        sim.forward_op(s, 0)
        j, adj = sw.l2_misfit(sim.traces()[comps], obs[s], w.dt)
        J += j
        sim.backward_op(adj)
    g = {p: sim.gradient(p) for p in ("lambda", "mu", "buoyancy")}
    sim.close()
    return J, g


def test_batch_matches_plain_path_and_replays():
    import seiswg_gb300 as sw

    probs = _problems()
    plain = [_plain(w, obs, comps) for (w, obs, comps) in probs]
    sims = [w.make_sim() for (w, _, _) in probs]
    batch = sw.Batch(sims, [obs for (_, obs, _) in probs])
    info = batch.info()
    assert info["jobs"] == sum(p[4] for p in PROBLEMS)
    results = []
    for _ in range(2):   # first run captures the graph, second replays it
        batch.run()
        results.append([{p: batch.gradient(i, p) for p in ("lambda", "mu", "buoyancy")} for i in range(len(probs))])
        for i, (J, _) in enumerate(plain):
            assert abs(batch.misfit(i) - J) <= 1e-6 * J
    for i, (J, g) in enumerate(plain):
        params = ("lambda", "mu", "buoyancy") if probs[i][0].flags["psv"] else ("mu", "buoyancy")
        for p in params:
            assert np.abs(g[p]).max() > 0
            assert rel_l2(results[0][i][p], g[p]) <= 1e-4, (i, p)
            assert np.array_equal(results[0][i][p], results[1][i][p])
    batch.close()
    for s in sims:
        s.close()


def test_chunk_rows_and_autotune_leave_gradients_unchanged():
    """The chunk rows only re-partition the same cell updates among warps:
    gradients are bitwise equal for every setting, including after autotune."""
    import seiswg_gb300 as sw

    probs = _problems()[:3]
    sims = [w.make_sim() for (w, _, _) in probs]
    batch = sw.Batch(sims, [obs for (_, obs, _) in probs])
    try:
        batch.run()
        ref = [batch.gradient(i, "mu") for i in range(len(probs))]
        for lx in (16, 128, 0):
            batch.set_option("chunk_rows", lx)
            assert batch.info()["chunk_rows"] == lx
            batch.run()
            for i in range(len(probs)):
                assert np.array_equal(batch.gradient(i, "mu"), ref[i]), (lx, i)
        # two-step recording (the default) or not: the same gradient to rounding
        batch.set_option("two_step", 0)
        assert not batch.info()["two_step"]
        batch.run()
        one = [batch.gradient(i, "mu") for i in range(len(probs))]
        for i in range(len(probs)):
            assert rel_l2(one[i], ref[i]) <= 1e-5, ("one-step recording", i)
        batch.set_option("autotune", 8)
        info = batch.info()
        assert info["chunk_rows"] in (0, 16, 32, 48, 64, 96, 128)
        batch.run()
        for i in range(len(probs)):
            assert np.array_equal(batch.gradient(i, "mu"), ref[i] if info["two_step"] else one[i]), ("autotune", i)
        with pytest.raises(sw.SeiswgError):
            batch.set_option("chunk_rows", 2)
    finally:
        batch.close()
        for s in sims:
            s.close()


def test_two_step_recomputation_keeps_the_gradient_to_rounding():
    """Recomputing the intervals' states two steps per grouped launch (the
    default with two-step recording; each launch stores both states) runs the
    same steps in fewer schedule slots (every job's list is shorter; the
    launch count depends on how the jobs' kinds line up in each slot); the
    gradients agree with
    one-step recomputation to FP32 rounding (the two-step kernel contracts
    multiply-adds), bitwise from run to run, and with the plain path."""
    import seiswg_gb300 as sw

    probs = _problems()[:3]
    plain = [_plain(w, obs, comps) for (w, obs, comps) in probs]
    sims = [w.make_sim() for (w, _, _) in probs]
    batch = sw.Batch(sims, [obs for (_, obs, _) in probs])
    try:
        out = {}
        for pair in (1, 0, 1):
            batch.set_option("two_step_recompute", pair)
            info = batch.info()
            batch.run()
            g = [{p: batch.gradient(i, p) for p in ("lambda", "mu", "buoyancy")} for i in range(len(probs))]
            if pair in out:
                for i in range(len(probs)):
                    for p in g[i]:
                        assert np.array_equal(g[i][p], out[pair][1][i][p]), (i, p)
            out[pair] = (info, g)
        assert out[1][0]["slots"] < out[0][0]["slots"]
        assert batch.checkpoint_plan()["recomputed_steps"] > 0
        for i, (_, gp) in enumerate(plain):
            params = ("lambda", "mu", "buoyancy") if probs[i][0].flags["psv"] else ("mu", "buoyancy")
            for p in params:
                assert rel_l2(out[1][1][i][p], out[0][1][i][p]) <= 1e-5, (i, p)
                assert rel_l2(out[1][1][i][p], gp[p]) <= 1e-4, (i, p)
    finally:
        batch.close()
        for s in sims:
            s.close()


def test_launch_orders_give_the_same_gradients():
    """The grouped launch orders -- serial launches, a slot's kinds on forked
    streams, and one stream per kind (and job group) with cross-kind waits
    only where a job changes kind, rows by tensor copies or by bulk copies --
    make the same cell updates in an order the dependencies allow, so their
    gradients are bitwise equal (a missing dependency would show as a
    difference).  The device queue (order 3) gives the same bits
    with tensor or bulk copies, run after run, and agrees with the grouped
    launches to rounding: it builds its one-step recomputation with
    multiply-add contraction."""
    import seiswg_gb300 as sw

    probs = _problems()
    sims = [w.make_sim() for (w, _, _) in probs]
    batch = sw.Batch(sims, [obs for (_, obs, _) in probs])
    try:
        assert batch.info()["concurrent"] == 2   # the default
        batch.set_option("concurrent", 3)        # one persistent launch over the device queue
        info = batch.info()
        assert info["concurrent"] == 3 and info["queue_band"] == 0
        assert info["queue_units"] > 0 and info["queue_blocks"] > 0
        queue = None
        for tma in (1, 0, 1):
            batch.set_option("tma", tma)
            batch.run()
            g = [{p: batch.gradient(i, p) for p in ("lambda", "mu", "buoyancy")} for i in range(len(probs))]
            J = [batch.misfit(i) for i in range(len(probs))]
            if queue is None:
                queue = (g, J)
                continue
            assert J == queue[1], tma
            for i in range(len(probs)):
                for p in g[i]:
                    assert np.array_equal(g[i][p], queue[0][i][p]), ("queue", tma, i, p)
        batch.set_option("queue_band", 4)        # diagonal bands of 4 slots: the same bits
        assert batch.info()["queue_band"] == 4
        batch.run()
        for i in range(len(probs)):
            assert batch.misfit(i) == queue[1][i]
            for p in queue[0][i]:
                assert np.array_equal(batch.gradient(i, p), queue[0][i][p]), ("band", i, p)
        ref = None
        for mode, groups, tma in ((0, 1, 1), (1, 1, 1), (2, 1, 1), (2, 1, 1), (2, 2, 1), (2, 4, 1), (1, 3, 1),
                                  (2, 1, 0)):
            batch.set_option("concurrent", mode)
            batch.set_option("stream_groups", groups)   # jobs split into stream groups
            batch.set_option("tma", tma)                 # rows by tensor copies or bulk copies
            assert batch.info()["concurrent"] == mode
            assert batch.info()["tma_jobs"] == (batch.info()["jobs"] if tma else 0)
            batch.run()                          # (2, 1) twice: the second run replays the graph
            g = [{p: batch.gradient(i, p) for p in ("lambda", "mu", "buoyancy")} for i in range(len(probs))]
            J = [batch.misfit(i) for i in range(len(probs))]
            assert batch.info()["queue_units"] == 0
            if ref is None:
                ref = (g, J)
                continue
            assert J == ref[1], mode
            for i in range(len(probs)):
                for p in g[i]:
                    assert np.array_equal(g[i][p], ref[0][i][p]), (mode, i, p)
        for i in range(len(probs)):
            assert abs(queue[1][i] - ref[1][i]) <= 1e-6 * ref[1][i]
            params = ("lambda", "mu", "buoyancy") if probs[i][0].flags["psv"] else ("mu", "buoyancy")
            for p in params:
                assert rel_l2(queue[0][i][p], ref[0][i][p]) <= 1e-5, ("queue vs grouped", i, p)
        for key, bad in (("concurrent", 4), ("concurrent", -1), ("stream_groups", 0), ("stream_groups", 5),
                         ("queue_wait_us", 0), ("test_queue_need_extra", -1)):
            with pytest.raises(sw.SeiswgError):
                batch.set_option(key, bad)
    finally:
        batch.close()
        for s in sims:
            s.close()


def test_batch_binomial_checkpointing_gives_the_same_gradients():
    """Every job under binomial checkpointing (S state slots, the revolve
    schedule of job_ops_revolve) against the uniform checkpoints of the
    default batch: with one-step recording every stored or recomputed state
    is the same bits, so the gradients are equal bit for bit; the pools
    shrink to S + 2 states per job and the recomputed steps are those the
    schedule states."""
    import seiswg_gb300 as sw

    probs = _problems()
    sims = [w.make_sim() for (w, _, _) in probs]
    batch = sw.Batch(sims, [obs for (_, obs, _) in probs])
    batch.set_option("two_step", 0)
    batch.run()
    ref = [{p: batch.gradient(i, p) for p in ("lambda", "mu", "buoyancy")} for i in range(len(probs))]
    bytes_uniform = batch.info()["device_bytes"]
    for S in (2, 5):
        batch.set_option("checkpoint_slots", S)
        info = batch.info()
        assert info["checkpoint_slots"] == S and info["device_bytes"] < bytes_uniform
        assert info["recomputed_steps"] > 0
        batch.run()
        for i in range(len(probs)):
            for p in ("lambda", "mu", "buoyancy"):
                assert np.array_equal(batch.gradient(i, p), ref[i][p]), (S, i, p)
    batch.set_option("two_step", 1)
    batch.run()
    for i in range(len(probs)):
        for p in ("mu", "buoyancy"):
            assert rel_l2(batch.gradient(i, p), ref[i][p]) <= 1e-5
    # the same through the device queue: binomial against uniform, bit for bit
    batch.set_option("two_step", 0)
    batch.set_option("concurrent", 3)
    batch.run()
    qref = [{p: batch.gradient(i, p) for p in ("mu", "buoyancy")} for i in range(len(probs))]
    batch.set_option("checkpoint_slots", 0)
    batch.run()
    for i in range(len(probs)):
        for p in ("mu", "buoyancy"):
            assert np.array_equal(batch.gradient(i, p), qref[i][p]), ("queue", i, p)
            assert rel_l2(qref[i][p], ref[i][p]) <= 1e-5
    batch.close()
    for s in sims:
        s.close()


def test_queue_wait_expiry_reports_a_timeout_and_the_batch_recovers():
    """The queue kernel's dependency waits are bounded.  With the test hook
    adding one to every dependency after a job's first operation, no such
    wait can be met: each runs out after queue_wait_us, the run fails with
    SEISWG_ETIMEOUT, and no GPU fault or hang results.  With the hook off the
    same batch runs again and gives the gradients of a run before."""
    import seiswg_gb300 as sw

    probs = _problems()[:2]
    sims = [w.make_sim() for (w, _, _) in probs]
    batch = sw.Batch(sims, [obs for (_, obs, _) in probs])
    try:
        batch.set_option("concurrent", 3)
        batch.run()
        ref = [batch.gradient(i, "mu") for i in range(len(probs))]
        batch.set_option("queue_wait_us", 2000)
        batch.set_option("test_queue_need_extra", 1)
        with pytest.raises(sw.SeiswgError) as e:
            batch.run()
        assert e.value.code == sw.ETIMEOUT
        batch.set_option("test_queue_need_extra", 0)
        batch.set_option("queue_wait_us", 2000000)
        batch.run()
        for i in range(len(probs)):
            assert np.array_equal(batch.gradient(i, "mu"), ref[i]), i
    finally:
        batch.close()
        for s in sims:
            s.close()


def test_queue_autotune_windows_and_chunk_rows():
    """The device queue's autotuner runs windows of slots in the middle of the
    schedule, each job's counters set as if the slots before had run: every
    window must finish (a dependency wait that ran out would make the autotune
    call fail with SEISWG_ETIMEOUT) and leave a batch whose next runs give the
    queue's own gradients, for every chunk-row setting."""
    import time

    import seiswg_gb300 as sw

    probs = _problems()[:3]
    sims = [w.make_sim() for (w, _, _) in probs]
    batch = sw.Batch(sims, [obs for (_, obs, _) in probs])
    try:
        batch.set_option("concurrent", 3)
        batch.set_option("queue_wait_us", 200000)   # a stuck window fails the test in 0.2 s
        batch.run()
        ref = [batch.gradient(i, "mu") for i in range(len(probs))]
        t0 = time.perf_counter()
        batch.set_option("autotune", 4)
        assert time.perf_counter() - t0 < 60
        info = batch.info()
        assert info["concurrent"] == 3 and info["chunk_rows"] in (0, 32, 48, 64, 96, 128)
        batch.run()
        for i in range(len(probs)):                  # one- or two-step recording: the same to rounding
            assert rel_l2(batch.gradient(i, "mu"), ref[i]) <= 1e-5
        for lx in (32, 0):
            batch.set_option("chunk_rows", lx)
            batch.set_option("two_step", 1)
            batch.run()
            for i in range(len(probs)):
                assert np.array_equal(batch.gradient(i, "mu"), ref[i]), (lx, i)
    finally:
        batch.close()
        for s in sims:
            s.close()
