"""GPU parity: sample views, kernel blocks, calibration sums and the median."""
import numpy as np
import pytest
import torch

from oracle import calibrate, kernel, ks

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def states():
    return ks.seeded_mode(3000, warm_time=100.0).astype(np.float32)


def test_hankel_rows_bit_exact(ctx):
    from kernel_evd_gb300 import api
    rng = np.random.default_rng(0)
    Ndata, M, Nq = 300, 5, 17
    u = rng.standard_normal(Ndata * M).astype(np.float32)
    X = api.hankel_rows(ctx, torch.from_numpy(u).cuda(), Ndata, M, Nq).cpu().numpy()
    np.testing.assert_array_equal(X, kernel.hankel_rows(u, Ndata, M, Nq))


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-14), ("mixed", 2e-5)])
def test_kernel_block(ctx, states, prec, tol):
    from kernel_evd_gb300 import api
    X = torch.from_numpy(states).cuda()
    rng = np.random.default_rng(1)
    cols = rng.integers(0, states.shape[0], 45)
    rows = rng.integers(0, states.shape[0], 70)
    sc = 1.0 / 40.0
    K = api.kernel_block(ctx, X, sc, torch.from_numpy(cols).cuda(), rows=torch.from_numpy(rows).cuda(),
                         precision=prec).cpu().numpy()
    ref = kernel.kblock(states.astype(np.float64), rows, cols, sc)
    np.testing.assert_allclose(K, ref, rtol=0, atol=tol)
    K2 = api.kernel_block(ctx, X, sc, torch.from_numpy(cols).cuda(), row0=100, nrows=33,
                          precision=prec).cpu().numpy()
    np.testing.assert_allclose(K2, kernel.kblock(states.astype(np.float64), np.arange(100, 133), cols, sc),
                               rtol=0, atol=tol)


def test_kernel_block_mixed_scale_unbiased(ctx, states):
    """The FP32 kernel block carries no systematic error from rounding the scale to
    FP32. The scale sits 0.45 ulp from its FP32 value (relative 3.4e-8). Every entry
    with K > 1e-3 gives a relative error rel ~ -arg * delta (arg = scale * d^2), and
    the least-squares delta stays below 1e-8; with fl32(scale) alone it is -3.0e-8
    (a NumPy emulation of the FP32 arithmetic gives -3.0e-8 and 5e-10)."""
    from kernel_evd_gb300 import api
    rng = np.random.default_rng(5)
    cols = rng.choice(states.shape[0], 600, replace=False)
    s0 = np.float32(0.025)
    sc = float(s0) + 0.45 * float(np.spacing(s0))
    K = api.kernel_block(ctx, torch.from_numpy(states).cuda(), sc, torch.from_numpy(cols).cuda(),
                         precision="mixed").cpu().numpy().astype(np.float64)
    ref = kernel.kblock(states.astype(np.float64), np.arange(states.shape[0]), cols, sc)
    m = ref > 1e-3
    arg = -np.log(ref[m])
    rel = (K[m] - ref[m]) / ref[m]
    delta = -(rel * arg).sum() / (arg * arg).sum()
    assert m.sum() > 100_000
    assert abs(delta) < 1e-8, delta


@pytest.mark.parametrize("N", [1, 2, 127, 128, 129, 1000])
def test_calibrate_matches_oracle(ctx, states, N):
    from kernel_evd_gb300 import api
    Xn = states[:N]
    med = 100.0
    eps = calibrate.log_sweep(med, 41)
    T = api.calibrate(ctx, torch.from_numpy(np.ascontiguousarray(Xn)).cuda(), 1.0 / eps)
    ref = calibrate.pair_sums(Xn.astype(np.float64), 1.0 / eps)
    if N == 1:
        assert np.all(T == 0)
        return
    # FP32 distances and exp2.approx: relative 1e-4 on every sum that is not negligible
    mask = ref > 1e-30 * N * N
    np.testing.assert_allclose(T[mask], ref[mask], rtol=1e-4)
    np.testing.assert_array_less(T[~mask], 1e-25 * N * N + 1e-300)


@pytest.mark.parametrize("N", [2, 129, 1000])
def test_calibrate_fp64_matches_oracle(ctx, states, N):
    from kernel_evd_gb300 import api
    Xn = np.ascontiguousarray(states[:N])
    eps = calibrate.log_sweep(100.0, 64)
    T = api.calibrate(ctx, torch.from_numpy(Xn).cuda(), 1.0 / eps, precision="fp64")
    ref = calibrate.pair_sums(Xn.astype(np.float64), 1.0 / eps)
    # FP64 distances from the same FP32 states, FP64 exp: summation order only
    np.testing.assert_allclose(T, ref, rtol=1e-12, atol=1e-300)


def test_calibrate_reference_sweep_hankel(ctx):
    from kernel_evd_gb300 import api
    rng = np.random.default_rng(3)
    Ndata, M, Nq = 140, 6, 16
    # reference-mode states on 64 gridpoints; keep the first M gridpoints
    full = ks.reference_mode(Ndata, M=64, n_warm=200)          # (time, gridpoint)
    u = np.ascontiguousarray(full[:, :M].T).reshape(-1).astype(np.float32)
    assert np.all(np.isfinite(u))
    X = api.hankel_rows(ctx, torch.from_numpy(u).cuda(), Ndata, M, Nq)
    bw = calibrate.reference_sweep().astype(np.float64)
    T = api.calibrate(ctx, X, 1.0 / (Nq * bw))
    Xo = kernel.hankel_rows(u, Ndata, M, Nq).astype(np.float64)
    ref = calibrate.pair_sums(Xo, 1.0 / (Nq * bw))
    np.testing.assert_allclose(T, ref, rtol=1e-4, atol=1e-30)
    NM = X.shape[0]
    sel = api.select_bandwidth(bw, T, NM)
    logS, slope, idmax, eopt, mdim = calibrate.select(bw, ref, NM)
    assert sel["idmax"] == idmax and sel["eopt"] == eopt
    np.testing.assert_allclose(sel["mdim"], mdim, rtol=1e-4)


def test_calibrate_selects_same_eps_as_oracle(ctx, states):
    from kernel_evd_gb300 import api
    Xn = states[:1500].astype(np.float64)
    med = calibrate.median_sqdist_exact(Xn)
    eps = calibrate.log_sweep(med, 41)
    T = api.calibrate(ctx, torch.from_numpy(states[:1500].copy()).cuda(), 1.0 / eps)
    ref = calibrate.pair_sums(Xn, 1.0 / eps)
    s1 = api.select_bandwidth(eps, T, 1500)
    _, _, idmax, eopt, _ = calibrate.select(eps, ref, 1500)
    assert s1["idmax"] == idmax


def test_pair_median_exact_and_sampled(ctx, states):
    from kernel_evd_gb300 import api
    Xn = states[:1200]
    X = torch.from_numpy(np.ascontiguousarray(Xn)).cuda()
    m = api.pair_median(ctx, X)
    ref = calibrate.median_sqdist_exact(Xn.astype(np.float64))
    assert abs(m - ref) <= 2e-6 * ref
    pi, pl = calibrate.sample_pairs(1200, 50001, seed=4)
    ms = api.pair_median(ctx, X, pairs=(torch.from_numpy(pi).cuda(), torch.from_numpy(pl).cuda()))
    D = ((Xn[pi].astype(np.float64) - Xn[pl].astype(np.float64)) ** 2).sum(1)
    refs = np.sort(D)[(D.size - 1) // 2]
    assert abs(ms - refs) <= 2e-6 * refs


def test_calibrate_batched_matches_single(ctx):
    """Uneven datasets (N, d) in one persistent launch: each job's sums equal the
    single-dataset pass up to FP64 summation order, for any work-item size."""
    from kernel_evd_gb300 import api
    shapes = [(1, 64), (2, 32), (129, 128), (700, 64), (3000, 32), (1500, 128)]
    Xs, scs = [], []
    for q, (n, m) in enumerate(shapes):
        Xn = ks.seeded_mode(max(n, 2), M=m, seed=q, warm_time=50.0)[:n].astype(np.float32)
        Xs.append(torch.from_numpy(np.ascontiguousarray(Xn)).cuda())
        scs.append(1.0 / calibrate.log_sweep(10.0 * m, 41 if q % 2 else 64))
    single = [api.calibrate(ctx, X, sc) for X, sc in zip(Xs, scs)]
    for tpi in (0, 1, 7):
        batched = api.calibrate_batched(ctx, Xs, scs, tiles_per_item=tpi)
        for q in range(len(shapes)):
            np.testing.assert_allclose(batched[q], single[q], rtol=1e-12, atol=1e-300, err_msg=f"job {q} tpi {tpi}")
    ref = calibrate.pair_sums(Xs[4].cpu().numpy().astype(np.float64), scs[4])
    mask = ref > 1e-30
    np.testing.assert_allclose(batched[4][mask], ref[mask], rtol=1e-4)
