"""The CPU oracle against every WGSL-produced fixture of the reference
(tests/integration.rs:202-282 and examples/adjoint/obs_traces).  These pins
are what make the oracle a valid checker for the GPU path."""
import os

import numpy as np
import pytest

from tests.examples import golden, max_rel, oracle_example, rel_l2

REL_TOL = 1e-4   # the reference's own tolerance (tests/integration.rs:40)
L2_TOL = 1e-5


def test_forward_fixture():
    g = golden("forward")
    o, s, sk, rk = oracle_example("forward", 32)
    snaps = o.run_forward(-1, 100, ["VY"])
    assert snaps.shape == (11, 1, 200, 200)
    vy100 = snaps[0, 0].ravel()
    assert max_rel(vy100, g["fix_proc000100_vy"]) <= REL_TOL
    assert rel_l2(vy100, g["fix_proc000100_vy"]) <= L2_TOL
    uy = o.obs("Y")
    assert uy.shape == (13, 1200)
    assert max_rel(uy, g["fix_uy_000000"]) <= REL_TOL
    assert rel_l2(uy, g["fix_uy_000000"]) <= L2_TOL


def test_forward_fp64_close_to_fp32():
    o32, *_ = oracle_example("forward", 32)
    o64, *_ = oracle_example("forward", 64)
    o32.run_forward(-1)
    o64.run_forward(-1)
    assert rel_l2(o32.obs("Y"), o64.obs("Y")) <= 1e-5


def test_spin_fixture():
    g = golden("spin")
    o, s, sk, rk = oracle_example("spin", 32)
    assert (s.nx, s.nz, s.dx) == (200, 200, 1.0)
    snaps = o.run_forward(-1, 200, ["VX"])
    vx200 = snaps[0, 0].ravel()
    assert max_rel(vx200, g["fix_proc000200_vx"]) <= REL_TOL
    assert rel_l2(vx200, g["fix_proc000200_vx"]) <= L2_TOL
    ry = o.obs("Y")
    assert max_rel(ry, g["fix_ry_000000"]) <= REL_TOL
    assert rel_l2(ry, g["fix_ry_000000"]) <= L2_TOL


@pytest.fixture(scope="module")
def true_obs():
    """Oracle forward on model_true, every shot (the config_true.ini run)."""
    o, s, sk, rk = oracle_example("adjoint", 32, model="true")
    obs = []
    for i in range(len(sk)):
        o.run_forward(i)
        obs.append(o.obs("Y").astype(np.float32))
    return np.array(obs)


def test_obs_traces_fixture(true_obs):
    g = golden("adjoint")
    assert true_obs.shape == (12, 144, 4800)
    for q, shot in enumerate(g["obs_shots"]):
        got = true_obs[shot][g["obs_recs"]]
        assert rel_l2(got, g["obs_uy"][q]) <= L2_TOL
        assert max_rel(got, g["obs_uy"][q]) <= REL_TOL


def test_adjoint_kmu_fixture(true_obs):
    g = golden("adjoint")
    o, s, sk, rk = oracle_example("adjoint", 32)
    mis = o.run_adjoint(np.arange(12), true_obs, 10, 5.0)
    assert np.all(mis > 0)
    kmu = o.field("K_MU").ravel()
    assert max_rel(kmu, g["fix_proc000000_kmu"]) <= REL_TOL
    assert rel_l2(kmu, g["fix_proc000000_kmu"]) <= L2_TOL


# A checkout of the reference (seiswg), named by SEISWG_REFERENCE, where present.
REFERENCE = os.environ.get("SEISWG_REFERENCE", "")
OBS_DIR = os.path.join(REFERENCE, "examples", "adjoint", "obs_traces")


@pytest.mark.skipif(not (REFERENCE and os.path.isdir(OBS_DIR)),
                    reason="SEISWG_REFERENCE does not name a reference checkout")
def test_adjoint_kmu_with_reference_obs_traces():
    """Same pin with all of the reference's own WGSL obs traces (where a
    checkout is named; the committed fixture test above runs everywhere)."""
    g = golden("adjoint")
    obs = np.stack([np.load(os.path.join(OBS_DIR, f"uy_{i:06d}.npy")) for i in range(12)])
    o, *_ = oracle_example("adjoint", 32)
    o.run_adjoint(np.arange(12), obs, 10, 5.0)
    assert rel_l2(o.field("K_MU"), g["fix_proc000000_kmu"]) <= L2_TOL


def test_smoothing_normalises_constant_field():
    """Full-range Gaussian smoothing normalised by GSUM leaves a constant kernel
    constant (fd2d.wgsl:515-609)."""
    from oracle import oracle as O

    s = O.Setup(30, 41, 1, 1.0, 1.0, 1e-3, sh=True, psv=False)
    o = O.FD2DOracle(s, [], np.zeros((3, 0, 1)), [], 64)
    o.set_field("K_MU", np.full(30 * 41, 2.5))
    o.smooth(4.0)
    np.testing.assert_allclose(o.field("K_MU"), 2.5, rtol=1e-12)
