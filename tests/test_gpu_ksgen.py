"""GPU Kuramoto-Sivashinsky generator (kevd_ks_generate) against the host
generator, which follows the reference's ks_datagen.py scheme:

* short horizon: from the same initial coefficients the first 200 states
  (50 time units, a few Lyapunov times) agree to 1e-4 of the state's range
  (FP64 in a different operation order, FP32 output);
* long horizon: after 1000 time units of warm-up the trajectories have
  decorrelated, but the attractor statistics (mean, variance, spatial
  autocorrelation) of 20,000 states agree;
* FP32 stepping: close to FP64 over 10 time units, same statistics after;
* several trajectories in one launch equal the same trajectories run alone;
* every grid size the workloads use (M = 32, 64, 128) and bad arguments.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("M,L", [(64, 22.0), (32, 16.0), (128, 36.0)])
def test_short_horizon_matches_host_generator(ctx, M, L):
    from kernel_evd_gb300 import datagen
    u0 = 0.1 * np.random.default_rng(5).standard_normal(M)
    v0 = np.fft.rfft(u0)
    host = datagen.run(L, M, 0.25, v0, 400, 200)          # past the initial transient
    vw = np.fft.rfft(datagen.run(L, M, 0.25, v0, 400, 1, dtype=np.float64)[0])
    gpu = datagen.run_gpu([(L, vw, 200)], M, ctx=ctx)[0].cpu().numpy()
    scale = np.abs(host).max()
    assert np.abs(gpu[:40] - host[:40]).max() < 1e-5 * scale
    assert np.abs(gpu - host).max() < 1e-4 * scale


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_long_horizon_statistics(ctx, precision):
    from kernel_evd_gb300 import datagen
    host = datagen.seeded_states(20000, L=22.0, M=64, seed=0, warm_time=1000.0).astype(np.float64)
    gpu = datagen.seeded_states_gpu(20000, L=22.0, M=64, seed=0, warm_time=1000.0, ctx=ctx,
                                    precision=precision).cpu().numpy()
    gpu = gpu.astype(np.float64)
    assert np.isfinite(gpu).all()
    assert abs(gpu.std() - host.std()) < 0.03 * host.std()
    assert abs(gpu.mean() - host.mean()) < 0.05 * host.std()
    ac_h = np.mean(host * np.roll(host, 4, axis=1)) / host.var()
    ac_g = np.mean(gpu * np.roll(gpu, 4, axis=1)) / gpu.var()
    assert abs(ac_h - ac_g) < 0.05


def test_fp32_short_horizon(ctx):
    """FP32 stepping stays within 1e-3 of the FP64 trajectory over 10 time units."""
    from kernel_evd_gb300 import datagen
    u0 = 0.1 * np.random.default_rng(5).standard_normal(64)
    vw = np.fft.rfft(datagen.run(22.0, 64, 0.25, np.fft.rfft(u0), 400, 1, dtype=np.float64)[0])
    host = datagen.run(22.0, 64, 0.25, vw, 0, 40)
    gpu = datagen.run_gpu([(22.0, vw, 40)], 64, ctx=ctx, precision="fp32")[0].cpu().numpy()
    assert np.abs(gpu - host).max() < 1e-3 * np.abs(host).max()


def test_batch_equals_single(ctx):
    from kernel_evd_gb300 import datagen
    rng = np.random.default_rng(3)
    specs = [(L, np.fft.rfft(0.1 * rng.standard_normal(64)), n) for L, n in ((22.0, 300), (16.0, 50), (36.0, 120))]
    together = datagen.run_gpu(specs, 64, n_warm=40, ctx=ctx)
    for sp, got in zip(specs, together):
        alone = datagen.run_gpu([sp], 64, n_warm=40, ctx=ctx)[0]
        assert got.shape == (sp[2], 64)
        assert np.array_equal(got.cpu().numpy(), alone.cpu().numpy())


def test_bad_arguments(ctx):
    from kernel_evd_gb300 import api, datagen
    with pytest.raises(api.KevdError):
        datagen.run_gpu([(22.0, np.zeros(5 // 2 + 1), 10)], 5, ctx=ctx)
    with pytest.raises(api.KevdError):
        datagen.run_gpu([(22.0, np.zeros(256 // 2 + 1), 10)], 256, ctx=ctx)
