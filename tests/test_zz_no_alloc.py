"""seiswg_smooth_noalloc, the smoothing entry point for callers that cannot
allocate device memory (their device memory belongs to their own pool
allocator, or they run where an allocating call is not allowed).  It must
give the same result as the allocating path, seiswg_sim_kernel_smooth, call
after call, although every call reuses the same fixed scratch.  This file is
collected last so that a stop at its first failure has run every other test."""
import numpy as np
import pytest

from tests.examples import rel_l2

pytestmark = pytest.mark.gpu


def _unsmoothed_and_smoothed_kernel(sigma, nx, nz):
    """kmu of a two-shot reference adjoint before and after
    seiswg_sim_kernel_smooth (the allocating path)."""
    import seiswg_gb300 as sw

    nt, dx, dt, adj = 200, 10.0, 1.5e-3, 10
    src_i, src_j = np.array([20, 44], np.int32), np.array([20, 20], np.int32)
    rec_i, rec_j = np.arange(5, 60, 6, dtype=np.int32), np.full(10, 30, np.int32)
    stf = np.stack([sw.ricker(nt, dt, 20.0, 0.05, 0.0, 1.0e10)] * 2, axis=1)
    rng = np.random.default_rng(11)
    with sw.Sim(nx, nz, nt, dx, dx, dt, sh=True, psv=False, abs_left=True, abs_right=True, abs_bottom=True,
                abs_width=12) as sim:
        sim.upload_model("vp", np.full((nx, nz), 3000.0))
        sim.upload_model("vs", np.full((nx, nz), 1732.0))
        sim.upload_model("rho", np.full((nx, nz), 2500.0))
        sim.prepare()
        sim.set_sources(src_i, src_j, stf)
        sim.set_receivers(rec_i, rec_j)
        sim.kernel_clear()
        for s in range(2):
            sim.adjoint_forward(s, adj)
            syn = sim.traces()[1]
            obs = syn * (1.0 + 0.05 * rng.standard_normal(syn.shape)).astype(np.float32)
            _, adstf = sw.waveform_misfit(syn, obs, dt)
            sim.adjoint_backward(adstf, adj)
        k0 = sim.kernel()
        sim.kernel_smooth(sigma)
        k1 = sim.kernel()
    return k0, k1


# (nx, nz, sigma): a tall grid with radius 8 sigma = 40 inside both axes;
# nx > nz with the radius clamped to max(nx, nz) - 1 = 89 (8 sigma = 160) and
# normaliser tables of different lengths
CASES = [(64, 150, 5.0), (90, 40, 20.0)]


@pytest.mark.parametrize("nx,nz,sigma", CASES)
def test_smooth_noalloc_matches_allocating_path_twice(nx, nz, sigma):
    torch = pytest.importorskip("torch")
    import seiswg_gb300 as sw

    k0, k1 = _unsmoothed_and_smoothed_kernel(sigma, nx, nz)
    assert np.abs(k0).max() > 0 and not np.allclose(k0, k1)
    assert k0.shape == (nx, nz)
    x = torch.from_numpy(np.ascontiguousarray(k0)).cuda()
    y = torch.empty_like(x)
    stream = torch.cuda.current_stream()
    outs = []
    for _ in range(2):  # two calls in a row share the fixed scratch
        y.fill_(float("nan"))
        sw.smooth_noalloc(x.data_ptr(), y.data_ptr(), nx, nz, sigma, stream.cuda_stream)
        stream.synchronize()
        got = y.cpu().numpy()
        assert np.isfinite(got).all()
        assert rel_l2(got, k1) <= 1e-5
        outs.append(got)
    assert np.array_equal(outs[0], outs[1])


def test_smooth_noalloc_rejects_sizes_beyond_its_scratch():
    import seiswg_gb300 as sw

    with pytest.raises(sw.SeiswgError) as e:
        sw.smooth_noalloc(1, 2, 4096, 4096, 5.0)     # 16.8 M cells > 4,194,304
    assert e.value.code == sw.EINVAL and "too large" in str(e.value)
    with pytest.raises(sw.SeiswgError):
        sw.smooth_noalloc(1, 2, 7000, 10, 5.0)      # > 6144 per axis
    with pytest.raises(sw.SeiswgError):
        sw.smooth_noalloc(1, 2, 100, 100, 0.0)
