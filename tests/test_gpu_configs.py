"""The named workloads at (or near) their own sizes, through the C ABI.

* The plain FP64 pipeline at N = 20,000 KS states (L = 22, d = 64, seed 0),
  eps by the 41-value calibration procedure, unblocked RPCholesky (b = 1) to
  rank 500, bistochastic EVD, top 32: pivots, per-round trace error, the top-32
  eigenvalues and the eigenvectors against the FP64 oracle run of the same
  low-rank pipeline (same Philox draws).
* The mixed form (FP32 factor, tensor-core residual update and Grams) against
  the FP64 factor and EVD of its own pivots: top-32 eigenvalues within 1e-8.
* A low-rank batched dataset (L = 16, N = 13,475, d = 64: the kernel's
  numerical rank is below the requested k = 607) in the mixed form: the
  factorisation must stop at the FP32 floor instead of accepting pivots on
  rounding noise, its pivots must form a nonsingular FP64 pivot block, and the
  mixed EVD must succeed."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _eps_exact_median(ctx, Xd):
    from kernel_evd_gb300 import api
    med = api.pair_median(ctx, Xd)
    eps = api.log_sweep(med, 41)
    return api.select_bandwidth(eps, api.calibrate(ctx, Xd, 1.0 / eps), Xd.shape[0])["eopt"]


def _eps_sampled_median(ctx, Xd, n_pairs=1_000_000):
    from kernel_evd_gb300 import api
    N = Xd.shape[0]
    rng = np.random.default_rng(0)
    i = rng.integers(0, N, n_pairs, dtype=np.int64)
    l = rng.integers(0, N - 1, n_pairs, dtype=np.int64)
    l = l + (l >= i)
    med = api.pair_median(ctx, Xd, pairs=(torch.from_numpy(i).cuda(), torch.from_numpy(l).cuda()))
    eps = api.log_sweep(med, 41)
    return api.select_bandwidth(eps, api.calibrate(ctx, Xd, 1.0 / eps), N)["eopt"]


@pytest.fixture(scope="module")
def c1_states():
    from kernel_evd_gb300 import datagen
    return datagen.seeded_states(20_000, L=22.0, M=64, seed=0, warm_time=1000.0, dt=0.25)


def test_c1_plain_fp64_pipeline_against_oracle(ctx, c1_states):
    from kernel_evd_gb300 import api
    from oracle import evd, rpchol
    X = c1_states
    Xd = torch.from_numpy(X).cuda()
    eps = _eps_exact_median(ctx, Xd)
    scale = 1.0 / eps
    k, b, top = 500, 1, 32
    g = api.rpcholesky(ctx, Xd, scale, k_max=k, block=b, seed=1234, precision="fp64")
    ref = rpchol.rpcholesky(X.astype(np.float64), scale, k, b, seed=1234)
    assert g.rank == k == ref["F"].shape[1]
    np.testing.assert_array_equal(g.piv, ref["piv"])
    np.testing.assert_allclose(g.err, ref["err"], rtol=1e-10, atol=1e-14)
    assert abs(g.trace_error - ref["err"][-1]) <= 1e-10 * ref["err"][-1]
    e = api.bistochastic_evd(ctx, g.factor, k_out=top)
    eo = evd.evd_from_factor(ref["F"], top)
    np.testing.assert_allclose(e.lam[-top:], eo["lam"][-top:], rtol=1e-10, atol=0)
    U = e.U.cpu().numpy().astype(np.float64)
    Uo = eo["U"]
    # U is written in FP32: eigenvectors up to sign, to FP32 resolution
    np.testing.assert_allclose(evd.align_signs(U, Uo), Uo, rtol=0, atol=2e-6 * np.abs(Uo).max())


def test_mixed_factorisation_and_evd_against_fp64_on_same_pivots(ctx):
    from kernel_evd_gb300 import api, datagen
    from oracle import evd
    X = datagen.seeded_states(200_000, L=22.0, M=64, seed=0, warm_time=1000.0, dt=0.25)
    Xd = torch.from_numpy(X).cuda()
    eps = _eps_exact_median(ctx, Xd[:20_000].contiguous())
    scale = 1.0 / eps
    k, top = 1000, 32
    m = api.rpcholesky(ctx, Xd, scale, k_max=k, block=64, seed=1234, precision="mixed")
    assert m.rank == k
    em = api.bistochastic_evd(ctx, m.factor, k_out=top)
    F64 = api.factor_from_pivots(ctx, Xd, scale, m.piv, precision="fp64")
    e64 = api.bistochastic_evd(ctx, F64, k_out=top)
    err = np.abs(em.lam[-top:] - e64.lam[-top:])
    assert err.max() <= 1e-8, f"top-{top} eigenvalue error {err.max():.3e} (leading {err[::-1][:4]})"
    # more eigenvectors than the refinement covers (the reference's k_out = 256 is of
    # this kind): the leading 32 pairs are refined all the same
    em64 = api.bistochastic_evd(ctx, m.factor, k_out=64)
    err64 = np.abs(em64.lam[-top:] - e64.lam[-top:])
    assert err64.max() <= 1e-8, f"k_out = 64: top-{top} eigenvalue error {err64.max():.3e}"
    assert abs(em64.lam[-1] - 1.0) <= 1e-8
    U32, U64 = em.U.cpu().numpy().astype(np.float64), em64.U.cpu().numpy().astype(np.float64)
    # the refined leading eigenvector (lambda = 1, well separated; the pairs below it
    # may be nearly degenerate) agrees with the k_out = 32 run's up to sign
    ang = evd.eigvec_angles(U64[:, -1:], U32[:, -1:])
    assert ang[0] < 1e-4, ang
    # trace error of the mixed run against the FP64 factor of the same pivots
    t64 = float((X.shape[0] - torch.sum(F64 * F64).item()) / X.shape[0])
    assert abs(m.trace_error - t64) <= 1e-6 + 1e-3 * t64


def test_mixed_low_rank_dataset_stops_at_the_fp32_floor(ctx):
    from kernel_evd_gb300 import api, datagen
    # the batched workload's dataset 21: L = 16, d = 64, N = 13,475, k = 607, b = 32
    X = datagen.seeded_states(13_475, L=16.0, M=64, seed=21, warm_time=1000.0, dt=0.25)
    Xd = torch.from_numpy(X).cuda()
    eps = _eps_sampled_median(ctx, Xd)
    scale = 1.0 / eps
    m = api.rpcholesky(ctx, Xd, scale, k_max=607, block=32, seed=21, precision="mixed")
    f64 = api.rpcholesky(ctx, Xd, scale, k_max=607, block=32, seed=21, precision="fp64")
    # mixed stops at or above the floor (16 x 2^-24) instead of reporting 0
    assert m.trace_error > 0.0
    assert m.trace_error >= min(f64.trace_error, 1e-6)
    # its pivot block is nonsingular in FP64 and both EVDs succeed
    F64 = api.factor_from_pivots(ctx, Xd, scale, m.piv, precision="fp64")
    e64 = api.bistochastic_evd(ctx, F64, k_out=16)
    em = api.bistochastic_evd(ctx, m.factor, k_out=16)
    # a nearly exact low-rank factor makes A = F^T Dtil^-2 F ill-conditioned, so
    # the tensor-core Gram's error weighs more here than at the large workload
    assert abs(em.lam[-1] - 1.0) < 1e-6
    assert np.abs(em.lam[-16:] - e64.lam[-16:]).max() < 1e-6


@pytest.mark.parametrize("k", [115, 116])
def test_mixed_evd_of_a_nearly_diagonal_kernel(ctx, k):
    """A batched-workload dataset whose calibrated eps is tiny against its
    pair distances (L = 22, d = 32, N = 51,194, eps = 2.806; its own k is 115):
    the kernel is nearly the identity, rows far from every pivot keep a tiny
    factor row, and the EVD's row weights 1/dtil^2 span about 1e17.  The Grams
    must take the split that keeps such weights (tf32), the factorisation the
    FP32 residual update also when the factor layout would allow the
    tensor-core one (k = 116), and the mixed EVD must match the FP64 EVD of the
    same pivots."""
    from kernel_evd_gb300 import api, datagen
    i, eps = 16, 2.805720090866089
    rng = np.random.default_rng(1000 + i)
    L = float(rng.choice([16.0, 22.0, 36.0]))
    m = int(rng.choice([32, 64, 128]))
    n = int(np.exp(rng.uniform(np.log(1e4), np.log(4e5))))
    k_own = min(int(rng.integers(100, 1001)), n // 2)
    assert (L, m, n, k_own) == (22.0, 32, 51194, 115)
    X = datagen.seeded_states(n, L=L, M=m, seed=i, warm_time=1000.0, dt=0.25).astype(np.float32)
    Xd = torch.from_numpy(X).cuda()
    fac = api.rpcholesky(ctx, Xd, 1.0 / eps, k_max=k, block=32, seed=i, precision="mixed")
    ev = api.bistochastic_evd(ctx, fac.factor.contiguous(), k_out=16)
    F64 = api.factor_from_pivots(ctx, Xd, fac.scale, fac.piv, precision="fp64")
    ev64 = api.bistochastic_evd(ctx, F64, k_out=16)
    assert abs(ev.lam[-1] - 1.0) < 1e-8
    np.testing.assert_allclose(ev.lam[-16:], ev64.lam[-16:], rtol=0, atol=1e-6)
    if k == 116:   # the update form in use: the SIMT update writes no tensor-core profile entry
        api.profile_enable(ctx, True)
        api.rpcholesky(ctx, Xd, 1.0 / eps, k_max=k, block=32, seed=i, precision="mixed")
        prof = api.profile_read(ctx)
        api.profile_enable(ctx, False)
        assert "rp_update" in prof and "rp_update_kcols" not in prof
