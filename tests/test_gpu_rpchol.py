"""GPU parity of block RPCholesky against the FP64 oracle.

The plain FP64 form must reproduce the oracle's pivot sequence bit-exactly for
the same uniform draws (Philox stream or an injected array) and match its
factor and per-round trace error to 1e-10 relative.  The mixed form (FP32
factor) is checked against the FP64 oracle by trace error."""
import numpy as np
import pytest
import torch

from oracle import ks, philox, rpchol

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def states():
    return ks.seeded_mode(5000, warm_time=100.0).astype(np.float32)


SCALE = 1.0 / 30.0


def _gpu(ctx, X, **kw):
    from kernel_evd_gb300 import api
    return api.rpcholesky(ctx, torch.from_numpy(np.ascontiguousarray(X)).cuda(), SCALE, **kw)


@pytest.mark.parametrize("N,k,b", [(5000, 200, 1), (5000, 300, 16), (4999, 400, 64), (777, 150, 32),
                                   (5000, 600, 128), (5000, 800, 256), (5000, 900, 512)])
def test_fp64_pivots_bit_exact(ctx, states, N, k, b):
    X = states[:N]
    seed = 1000 + b
    ref = rpchol.rpcholesky(X.astype(np.float64), SCALE, k, b, seed=seed)
    g = _gpu(ctx, X, k_max=k, block=b, seed=seed, precision="fp64")
    assert g.rank == ref["F"].shape[1]
    np.testing.assert_array_equal(g.piv, ref["piv"])
    np.testing.assert_array_equal(g.accepted, ref["hm"])
    np.testing.assert_allclose(g.err, ref["err"], rtol=1e-10, atol=1e-14)
    F = g.factor.cpu().numpy()
    np.testing.assert_allclose(F, ref["F"], rtol=0, atol=1e-10)


def test_fp64_injected_uniforms(ctx, states):
    X = states[:3000]
    b, k, rounds = 8, 96, 40
    rng = np.random.default_rng(11)
    U = 1.0 - rng.random((rounds, 2, b))          # (0, 1]

    def draw(rnd, stream, n):
        return U[rnd, stream, :n]
    ref = rpchol.rpcholesky(X.astype(np.float64), SCALE, k, b, n_rounds=rounds, draw=draw)
    g = _gpu(ctx, X, k_max=k, block=b, max_rounds=rounds, uniforms=U, precision="fp64")
    np.testing.assert_array_equal(g.piv, ref["piv"])
    np.testing.assert_allclose(g.err, ref["err"], rtol=1e-10)


def test_fp64_round_limit_and_err_target(ctx, states):
    X = states[:2000]
    g = _gpu(ctx, X, k_max=500, block=16, max_rounds=5, seed=3, precision="fp64")
    assert g.rounds == 5 and g.err.size == 5
    ref = rpchol.rpcholesky(X.astype(np.float64), SCALE, 500, 16, seed=3, n_rounds=5)
    np.testing.assert_array_equal(g.piv, ref["piv"])
    g2 = _gpu(ctx, X, k_max=500, block=16, seed=3, err_target=0.2, precision="fp64")
    ref2 = rpchol.rpcholesky(X.astype(np.float64), SCALE, 500, 16, seed=3, err_target=0.2)
    assert g2.rounds == len(ref2["err"]) and g2.err[-1] <= 0.2
    np.testing.assert_array_equal(g2.piv, ref2["piv"])


def test_mixed_trace_error_close_to_fp64(ctx, states):
    X = states[:5000]
    ref = rpchol.rpcholesky(X.astype(np.float64), SCALE, 400, 32, seed=9)
    g = _gpu(ctx, X, k_max=400, block=32, seed=9, precision="mixed")
    assert g.rank == 400
    # same draws: the pivot sequences agree at least at the start
    n_same = int(np.argmax(g.piv != ref["piv"])) if np.any(g.piv != ref["piv"]) else g.rank
    assert n_same >= 64
    assert abs(g.trace_error - ref["err"][-1]) <= 0.05 * ref["err"][-1]
    # the stored FP32 factor is consistent with the residual diagonal it reports
    F = g.factor.double().cpu().numpy()
    direct = (X.shape[0] - (F ** 2).sum()) / X.shape[0]
    assert abs(direct - g.trace_error) <= 1e-5 * max(1.0, g.trace_error)


@pytest.mark.parametrize("N,b", [(5000, 64), (3001, 17), (640, 1), (5000, 128), (4000, 256)])
def test_mixed_factor_columns_match_oracle(ctx, states, N, b):
    """With the same draws, the FP32 factor (tensor-core residual update) agrees
    with the FP64 oracle column by column while the pivot sequences agree."""
    X = states[:N]
    k = 3 * b if b > 1 else 40
    ref = rpchol.rpcholesky(X.astype(np.float64), SCALE, k, b, seed=77)
    g = _gpu(ctx, X, k_max=k, block=b, seed=77, precision="mixed")
    same = int(np.argmax(g.piv != ref["piv"])) if np.any(g.piv != ref["piv"]) else min(g.rank, ref["piv"].size)
    # a larger block accepts more proposals per round after many Schur updates,
    # whose residuals lie nearer the acceptance threshold (FP32 rounding of H
    # can flip a decision sooner) and nearer the FP32 floor (a column divides
    # by sqrt(H_ii) >= 1e-3, so its error can reach 1e-7 / 1e-3)
    assert same >= min(k, 2 * b if b <= 64 else b)
    F = g.factor.double().cpu().numpy()[:, :same]
    np.testing.assert_allclose(F, ref["F"][:, :same], rtol=0, atol=2e-5 if b <= 64 else 2e-4)


def test_linv_matches_oracle(ctx, states):
    from kernel_evd_gb300 import api
    X = states[:2000]
    g = _gpu(ctx, X, k_max=120, block=16, seed=2, precision="fp64")
    Li = api.linv(ctx, g)
    ref = rpchol.rpcholesky(X.astype(np.float64), SCALE, 120, 16, seed=2)
    Lref = rpchol.linv_from_F(ref["F"], ref["piv"])
    np.testing.assert_allclose(Li, Lref, rtol=1e-8, atol=1e-8 * np.abs(Lref).max())


def test_bad_arguments(ctx, states):
    from kernel_evd_gb300 import KevdError, api
    X = torch.from_numpy(states[:100].copy()).cuda()
    with pytest.raises(KevdError) as e:
        api.rpcholesky(ctx, X, SCALE, k_max=10, block=513, precision="fp64")
    assert e.value.name == "KEVD_ERR_ARG"
    with pytest.raises(KevdError):
        api.rpcholesky(ctx, X, SCALE, k_max=10, block=4, precision="fp64",
                       F=torch.empty((100, 5), dtype=torch.float64, device="cuda"))


@pytest.mark.parametrize("use_graph", [True, False])
def test_batched_factorisations_match_single(ctx, use_graph):
    """Uneven jobs (N, d, k, b) in one call, with and without the captured
    graph: each job equals the single-job factorisation (same pivots, same
    trace error, same factor columns)."""
    from kernel_evd_gb300 import api
    shapes = [(3000, 64, 256, 32), (1200, 32, 100, 16), (5000, 128, 320, 64), (800, 64, 64, 32), (4000, 64, 400, 128)]
    Xs, scales = [], []
    for q, (n, m, k, b) in enumerate(shapes):
        Xn = ks.seeded_mode(n, M=m, seed=10 + q, warm_time=60.0).astype(np.float32)
        Xs.append(torch.from_numpy(Xn).cuda())
        scales.append(1.0 / (0.5 * m))
    ks_ = [s[2] for s in shapes]
    bs = [s[3] for s in shapes]
    got = api.rpcholesky_batched(ctx, Xs, scales, ks_, bs, seeds=[7, 8, 9, 10, 11], use_graph=use_graph)
    for q in range(len(shapes)):
        ref = api.rpcholesky(ctx, Xs[q], scales[q], k_max=ks_[q], block=bs[q], seed=7 + q, precision="mixed")
        assert got[q].rank == ref.rank
        np.testing.assert_array_equal(got[q].piv, ref.piv)
        assert got[q].trace_error == ref.trace_error
        np.testing.assert_array_equal(got[q].factor.cpu().numpy(), ref.factor.cpu().numpy())


def test_autotuner_picks_a_candidate_and_caches(ctx, tmp_path, monkeypatch):
    from kernel_evd_gb300 import autotune
    monkeypatch.setenv("KEVD_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    monkeypatch.setattr(autotune, "_loaded", False)
    monkeypatch.setattr(autotune, "_cache", {})
    X = torch.from_numpy(ks.seeded_mode(6000, warm_time=60.0).astype(np.float32)).cuda()
    r1 = autotune.tune_block(ctx, X, 1.0 / 30.0, 300, candidates=(16, 32, 64), probe_rows=6000, probe_k=192)
    assert r1["block"] in (16, 32, 64) and not r1["cached"] and len(r1["ms_per_column"]) == 3
    r2 = autotune.tune_block(ctx, X, 1.0 / 30.0, 300, candidates=(16, 32, 64))
    assert r2["cached"] and r2["block"] == r1["block"]
    assert (tmp_path / "tune.json").exists()
    c = autotune.tune_calibration_items(ctx, [X[:3000], X[3000:4500]], [1.0 / np.geomspace(1, 300, 41)] * 2,
                                        candidates=(0, 4, 64))
    assert c["tiles_per_item"] in (0, 4, 64)
