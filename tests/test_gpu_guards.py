"""Guards around a run, through the C ABI on the GPU: the stability check of
seiswg_sim_prepare, the NaN / infinity watchdog on traces and gradients, and
the bounded waits of the row pipelines (a wait made to run out reports
SEISWG_ETIMEOUT and leaves the handle usable).  The reference has none of
these; its only guards are errors of its host code (solver.rs:1312-1314).

The expired waits are made on purpose without any fault: the test hook arms
the first stage of every warp's row ring for 16 bytes more than its copies
bring, so every copy still lands and only the count stays short; the kernel
gives up after `wait_polls` polls, takes the 16 bytes back, waits for its
copies and leaves."""
import math

import numpy as np
import pytest

from tests.examples import rel_l2

pytestmark = pytest.mark.gpu


def _sim(nx, nz, nt, dx, dt, model, options=(), prepare=True, dz=None, **flags):
    import seiswg_gb300 as sw

    sim = sw.Sim(nx, nz, nt, dx, dx if dz is None else dz, dt, **flags)
    for k, v in options:
        sim.set_option(k, v)
    for k, v in model.items():
        sim.upload_model(k, v)
    if prepare:
        sim.prepare()
    return sim


def _elastic(nx, nz, vp=3000.0, seed=0):
    rng = np.random.default_rng(seed)
    p = (1.0 + 0.05 * np.tanh(rng.standard_normal((nx, nz)))).astype(np.float32)
    v = (vp * p).astype(np.float32)
    return dict(vp=v, vs=(v / np.float32(math.sqrt(3.0))).astype(np.float32),
                rho=np.full((nx, nz), 2500.0, np.float32))


def _limit(c, dx, dz=None):
    dz = dx if dz is None else dz
    return 1.0 / (c * (7.0 / 6.0) * math.sqrt(1.0 / dx ** 2 + 1.0 / dz ** 2))


def test_stability_numbers_and_rejection():
    import seiswg_gb300 as sw

    nx, nz, dx = 64, 72, 10.0
    m = _elastic(nx, nz)
    cmax = float(np.max(m["vp"].astype(np.float64)))
    dt_max = _limit(cmax, dx)
    sim = _sim(nx, nz, 10, dx, 0.9 * dt_max, m, psv=True)
    wave, spin = sim.stability()
    assert abs(wave - 0.9) < 1e-5 and spin == 0.0
    sim.close()
    with pytest.raises(sw.SeiswgError) as e:
        _sim(nx, nz, 10, dx, 1.05 * dt_max, m, psv=True)
    assert e.value.code == sw.EINVAL and "unstable" in str(e.value)
    # SH alone is limited by the S speed: the same dt passes there.
    cs = float(np.max(m["vs"].astype(np.float64)))
    sim = _sim(nx, nz, 10, dx, 1.05 * dt_max, m, sh=True, psv=False)
    assert abs(sim.stability()[0] - 1.05 * dt_max / _limit(cs, dx)) < 1e-5
    sim.close()
    # rectangular cells
    sim = _sim(nx, nz, 10, dx, 0.5 * _limit(cmax, dx, 2 * dx), m, dz=2 * dx, psv=True)
    assert abs(sim.stability()[0] - 0.5) < 1e-5
    sim.close()


def test_stability_rejects_bad_models():
    import seiswg_gb300 as sw

    nx, nz = 40, 50
    m = _elastic(nx, nz)
    m["rho"][3, 4] = 0.0  # buoyancy 1/0 = inf
    with pytest.raises(sw.SeiswgError) as e:
        _sim(nx, nz, 10, 10.0, 1e-3, m, psv=True)
    assert e.value.code == sw.EINVAL and "non-finite" in str(e.value)


def test_spin_rotation_rate_is_checked():
    import seiswg_gb300 as sw

    nx = nz = 48
    dx, rho, lam = 1.0, 2700.0, 8.1e9
    shape = (nx, nz)
    full = lambda v: np.full(shape, v, np.float32)  # noqa: E731
    model = {"rho": full(rho), "lambda": full(lam), "mu": full(lam), "nu": full(0.1 * lam), "j": full(1.0),
             "lambda_c": full(1e3), "mu_c": full(1e3), "nu_c": full(1e3)}
    # w0 = sqrt(4 nu / J) = 5.7e4 1/s; the P limit alone would allow dt ~ 2.0e-4 here.
    w0 = math.sqrt(4 * 0.1 * lam / 1.0)
    dt = 3.0 / w0
    with pytest.raises(sw.SeiswgError) as e:
        _sim(nx, nz, 10, dx, dt, model, psv=True, spin=True)
    assert e.value.code == sw.EINVAL and "spin" in str(e.value)
    sim = _sim(nx, nz, 10, dx, 1.0 / w0, model, psv=True, spin=True)
    assert 0.45 < sim.stability()[1] < 0.55
    sim.close()


def test_unstable_run_is_caught_by_the_watchdog():
    """With the check off, an unstable dt overflows; the call that finishes
    the run or reads its traces (and the gradients) fails with
    SEISWG_ENUMERIC."""
    import seiswg_gb300 as sw

    nx, nz, nt, dx = 80, 90, 300, 10.0
    m = _elastic(nx, nz)
    dt = 1.6 * _limit(float(np.max(m["vp"])), dx)
    sim = _sim(nx, nz, nt, dx, dt, m, options=[("stability_check", 0)], psv=True)
    assert sim.stability()[0] > 1.5
    stf = sw.ricker(nt, dt, 20.0, 0.05, 30.0, 1.0e10)[:, None, :]
    sim.set_sources([40], [45], stf)
    sim.set_receivers([10, 60], [20, 70])
    with pytest.raises(sw.SeiswgError) as e:
        sim.forward(-1)  # synchronous: waits for the run and reads the error word
    assert e.value.code == sw.ENUMERIC and "NaN" in str(e.value)
    sim.gradient_clear()
    sim.forward_op(-1, 0)
    with pytest.raises(sw.SeiswgError) as e:
        sim.traces()
    assert e.value.code == sw.ENUMERIC
    adj = np.ones((2, 2, nt), np.float32)
    sim.backward_op(adj)
    with pytest.raises(sw.SeiswgError) as e:
        sim.gradient("mu")
    assert e.value.code == sw.ENUMERIC
    sim.close()


CASES = {
    # physics flags, options: the two-step PSV kernel with tensor copies (the
    # default), the one-step PSV kernel with bulk copies, the SH two-step
    # kernel, the spin kernel
    "psv_two_step_tma": (dict(psv=True), []),
    "psv_one_step_bulk": (dict(psv=True), [("two_step", 0)]),
    "sh_two_step": (dict(sh=True, psv=False), [("cluster", 0)]),
    "spin": (dict(psv=True, spin=True), []),
}


def _forward_case(name):
    import seiswg_gb300 as sw

    flags, opts = CASES[name]
    nx, nz, nt, dx = 96, 140, 24, 10.0
    if flags.get("spin"):
        dx, dt = 1.0, 1e-4
        shape = (nx, nz)
        full = lambda v: np.full(shape, v, np.float32)  # noqa: E731
        model = {"rho": full(2700.0), "lambda": full(8.1e9), "mu": full(8.1e9), "nu": full(1e9), "j": full(2700.0),
                 "lambda_c": full(1e8), "mu_c": full(1e8), "nu_c": full(1e8)}
    else:
        dt = 1e-3
        model = _elastic(nx, nz)
    sim = _sim(nx, nz, nt, dx, dt, model, options=opts, **flags)
    stf = sw.ricker(nt, dt, 25.0, 0.01, 30.0, 1.0e10)[:, None, :]
    sim.set_sources([48], [70], stf)
    sim.set_receivers([10, 48, 90], [5, 60, 130])
    return sim


@pytest.mark.parametrize("name", list(CASES))
def test_expired_wait_reports_timeout_and_the_handle_recovers(name):
    import seiswg_gb300 as sw

    clean = _forward_case(name)
    clean.forward(-1)
    want = clean.traces()
    clean.close()

    sim = _forward_case(name)
    sim.set_option("wait_polls", 4096)
    sim.set_option("test_arm_extra", 16)
    with pytest.raises(sw.SeiswgError) as e:
        sim.forward(-1)  # synchronous: waits for the run and reads the error word
    assert e.value.code == sw.ETIMEOUT and "bounded wait" in str(e.value)
    # the error is reported once; the same handle runs normally afterwards
    sim.set_option("test_arm_extra", 0)
    sim.set_option("wait_polls", 0)
    sim.forward(-1)
    got = sim.traces()
    sim.close()
    assert np.array_equal(got, want)


def test_expired_wait_in_the_reverse_step():
    import seiswg_gb300 as sw

    sim = _forward_case("psv_two_step_tma")
    nt = 24
    sim.gradient_clear()
    sim.forward_op(-1, 0)
    syn = sim.traces()[[0, 2]]
    J, adj = sw.l2_misfit(syn, np.zeros_like(syn), 1e-3)
    sim.backward_op(adj)
    want = sim.gradient("mu")
    assert np.any(want)
    sim.gradient_clear()
    sim.forward_op(-1, 0)
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
    sim.forward_op(-1, 0)
    sim.traces()
    sim.backward_op(adj)
    got = sim.gradient("mu")
    sim.close()
    assert nt == 24 and rel_l2(got, want) == 0.0
