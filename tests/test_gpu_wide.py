"""Wide samples (d > 128): the reference's own delay windows are Nq = 512
long.  Every kernel that stages rows does so a fixed feature chunk at a time;
results must match the FP64 oracle as for small d (same summation order)."""
import numpy as np
import pytest
import torch

from oracle import calibrate, kernel, ks, rpchol

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def hankel300():
    # delay windows of a KS time series: 4 gridpoints x 700 samples, Nq = 300
    S = ks.seeded_mode(700, M=64, seed=2, warm_time=50.0)          # 700 times x 64 gridpoints
    u = np.ascontiguousarray(S[:, :4].T).ravel().astype(np.float32)  # 4 gridpoints, time fastest
    return kernel.hankel_rows(u, 700, 4, 300).astype(np.float32)   # (401 * 4) x 300


@pytest.mark.parametrize("d", [200, 512])
def test_calibrate_and_median_wide(ctx, d):
    from kernel_evd_gb300 import api
    rng = np.random.default_rng(d)
    X = rng.standard_normal((300, d)).astype(np.float32)
    Xt = torch.from_numpy(X).cuda()
    eps = calibrate.log_sweep(2.0 * d, 41)
    ref = calibrate.pair_sums(X.astype(np.float64), 1.0 / eps)
    mask = ref > 1e-30
    np.testing.assert_allclose(api.calibrate(ctx, Xt, 1.0 / eps)[mask], ref[mask], rtol=1e-4)
    np.testing.assert_allclose(api.calibrate(ctx, Xt, 1.0 / eps, precision="fp64"), ref, rtol=1e-12, atol=1e-300)
    b = api.calibrate_batched(ctx, [Xt, Xt[:77].contiguous()], [1.0 / eps, 1.0 / eps])
    np.testing.assert_allclose(b[0][mask], ref[mask], rtol=1e-4)
    D = kernel.sqdist_block(X.astype(np.float64), X.astype(np.float64))
    lower = np.sort(D[np.tril_indices(300, -1)])
    med = api.pair_median(ctx, Xt)
    assert abs(med - lower[(lower.size - 1) // 2]) <= 1e-5 * lower.max()


def test_kernel_block_wide(ctx, hankel300):
    from kernel_evd_gb300 import api
    X = hankel300
    rng = np.random.default_rng(3)
    cols = rng.integers(0, X.shape[0], 40)
    sc = 1.0 / (300 * 0.5)
    K = api.kernel_block(ctx, torch.from_numpy(X).cuda(), sc, torch.from_numpy(cols).cuda(), row0=0, nrows=200,
                         precision="fp64").cpu().numpy()
    np.testing.assert_allclose(K, kernel.kblock(X.astype(np.float64), np.arange(200), cols, sc), rtol=0, atol=1e-14)


def test_rpchol_fp64_pivots_bit_exact_wide(ctx, hankel300):
    from kernel_evd_gb300 import api
    X = hankel300
    sc = 1.0 / (300 * 0.5)
    ref = rpchol.rpcholesky(X.astype(np.float64), sc, 64, 16, seed=5)
    g = api.rpcholesky(ctx, torch.from_numpy(X).cuda(), sc, k_max=64, block=16, seed=5, precision="fp64")
    np.testing.assert_array_equal(g.piv, ref["piv"])
    np.testing.assert_allclose(g.factor.cpu().numpy(), ref["F"][:, : g.rank], rtol=0, atol=1e-10)


def test_rpchol_mixed_and_nystrom_wide(ctx):
    from kernel_evd_gb300 import api
    rng = np.random.default_rng(4)
    # a smooth 3-dimensional manifold embedded in 256 dimensions
    t = rng.uniform(0, 2 * np.pi, (3000, 3))
    basis = rng.standard_normal((6, 256)) / 4.0
    X = np.concatenate([np.sin(t), np.cos(t)], axis=1) @ basis
    X = X.astype(np.float32)
    Xt = torch.from_numpy(X).cuda()
    D = kernel.sqdist_block(X[:300].astype(np.float64), X[300:600].astype(np.float64))
    sc = 1.0 / float(np.median(D))
    m = api.rpcholesky(ctx, Xt, sc, k_max=128, block=32, seed=6, precision="mixed")
    f = api.rpcholesky(ctx, Xt, sc, k_max=128, block=32, seed=6, precision="fp64")
    assert m.rank == f.rank == 128
    assert abs(m.trace_error - f.trace_error) <= 0.05 * f.trace_error
    model = api.NystromModel(ctx, Xt, f, k_out=4)
    ev = api.bistochastic_evd(ctx, f.factor, k_out=4)
    idx = np.arange(0, 3000, 11)
    Uy = model(Xt[torch.from_numpy(idx).cuda()].contiguous()).cpu().numpy()
    U = ev.U.cpu().numpy()[idx]
    s = np.sign(np.sum(Uy * U, axis=0))
    np.testing.assert_allclose(Uy * s, U, rtol=0, atol=1e-5 * np.abs(U).max())
