"""The oracle's exact discrete adjoint against central finite differences of
J = sum (taper (d - obs))^2, in FP64.  The reference has no PSV adjoint (its
PSV branch zero-fills, solver.rs:1427-1432) and only an imaging-condition SH
kernel, so finite differences are the pin for this part of the oracle."""
import numpy as np
import pytest

from oracle import oracle as O

NX, NZ, NT, DX, DT = 36, 44, 160, 10.0, 1.5e-3


def _setup(phys):
    flags = dict(sh=phys == "sh", psv=phys == "psv", abs_left=True, abs_bottom=True, abs_width=8)
    s = O.Setup(NX, NZ, NT, DX, DX, DT, **flags)
    rng = np.random.default_rng(0)
    vp = 3000 * (1 + 0.05 * rng.standard_normal((NX, NZ)))
    vs = vp / np.sqrt(3)
    rho = 2500 * (1 + 0.03 * rng.standard_normal((NX, NZ)))
    src = [12 * NZ + 15]
    stf = O.stf_table([(0, 0, 25.0, 0.04, 30.0, 1e10)], NT, DT, 64)
    rk = np.array([5 * NZ + 30, 20 * NZ + 30, 30 * NZ + 5, 18 * NZ + 40, 18 * NZ + 41], np.int32)
    comps = ("X", "Z") if phys == "psv" else ("Y",)

    def run(vp, vs, rho):
        o = O.FD2DOracle(s, src, stf, rk, 64)
        o.set_field("LAM", vp)
        o.set_field("MU", vs)
        o.set_field("RHO", rho)
        o.init_model()
        o.run_forward(0)
        return o, np.stack([o.obs(c) for c in comps])

    _, obs = run(vp * 1.02, vs * 0.98, rho)
    return run, obs, vp, vs, rho


@pytest.mark.parametrize("phys", ["psv", "sh"])
def test_oracle_adjoint_matches_finite_differences(phys):
    run, obs, vp, vs, rho = _setup(phys)
    o, syn = run(vp, vs, rho)
    _, adj = O.l2_misfit(syn, obs, DT)
    gl, gm, gb = o.exact_gradient(adj, 0)
    g = dict(zip(("vp", "vs", "rho"), O.lame_to_velocity_gradients(gl, gm, gb, vp, vs, rho)))
    rng = np.random.default_rng(1)
    names = ("vp", "vs", "rho") if phys == "psv" else ("vs", "rho")
    for _ in range(4):
        i, j = int(rng.integers(3, NX - 3)), int(rng.integers(3, NZ - 3))
        for name in names:
            base = dict(vp=vp, vs=vs, rho=rho)
            h = 1e-5 * base[name][i, j]
            plus, minus = dict(base), dict(base)
            plus[name] = base[name].copy()
            plus[name][i, j] += h
            minus[name] = base[name].copy()
            minus[name][i, j] -= h
            jp = O.l2_misfit(run(**plus)[1], obs, DT)[0]
            jm = O.l2_misfit(run(**minus)[1], obs, DT)[0]
            fd = (jp - jm) / (2 * h)
            assert abs(g[name][i, j] - fd) <= 1e-6 * abs(fd) + 1e-12 * np.abs(g[name]).max(), (name, i, j)
