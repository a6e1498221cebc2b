"""GPU parity of the bistochastic EVD against the FP64 oracle, at every dump
point of the reference (c1, dtil, cq, qtil, A, B, W, Z, lam, U)."""
import numpy as np
import pytest
import torch

from oracle import evd, ks, rpchol

pytestmark = pytest.mark.gpu

SCALE = 1.0 / 30.0


@pytest.fixture(scope="module")
def fac():
    X = ks.seeded_mode(4000, warm_time=100.0).astype(np.float32)
    r = rpchol.rpcholesky(X.astype(np.float64), SCALE, 300, 32, seed=21)
    return X, r


def test_fp64_evd_every_intermediate(ctx, fac):
    from kernel_evd_gb300 import api
    X, r = fac
    F = torch.from_numpy(r["F"]).cuda()
    g = api.bistochastic_evd(ctx, F, k_out=16, dump=True)
    e = evd.evd_from_factor(r["F"], 16)
    for name in ("c1", "dtil", "cq", "qtil"):
        np.testing.assert_allclose(g.dump[name], e[name], rtol=1e-12, err_msg=name)
    for name in ("A", "B", "W"):
        np.testing.assert_allclose(g.dump[name], e[name], rtol=0, atol=1e-11 * np.abs(e[name]).max(),
                                   err_msg=name)
    assert abs(g.trace_A - e["trA"]) <= 1e-12 * e["trA"] and g.shift == pytest.approx(e["shift"], rel=1e-12)
    np.testing.assert_allclose(g.lam, e["lam"], rtol=0, atol=1e-10)
    top = e["lam"][-16:]
    np.testing.assert_allclose(g.lam[-16:], top, rtol=1e-10)
    U = g.U.cpu().numpy().astype(np.float64)
    Ua = evd.align_signs(U, e["U"])
    # U is written in FP32
    np.testing.assert_allclose(Ua, e["U"], rtol=0, atol=2e-6 * np.abs(e["U"]).max())
    assert np.all(evd.eigvec_angles(U[:, -8:], e["U"][:, -8:]) < 1e-5)


@pytest.mark.parametrize("k_out", [100, 256])
def test_fp64_evd_many_eigenvectors(ctx, fac, k_out):
    """The reference computes k_out = 256 eigenvectors (ks_kevd.cu:481): U is
    formed in 64-column chunks."""
    from kernel_evd_gb300 import api
    X, r = fac
    g = api.bistochastic_evd(ctx, torch.from_numpy(r["F"]).cuda(), k_out=k_out, dump=True)
    e = evd.evd_from_factor(r["F"], k_out)
    np.testing.assert_allclose(g.lam, e["lam"], rtol=0, atol=1e-10)
    # the leading eigenvectors are well separated; deep in the spectrum the
    # eigenvalues cluster near zero and only the subspace is determined
    lead = 32
    Z, Ze = g.dump["Z"][:, -lead:], e["Z"][:, -lead:]
    np.testing.assert_allclose(evd.align_signs(Z, Ze), Ze, rtol=0, atol=1e-8 * np.abs(Ze).max())
    U = g.U.cpu().numpy().astype(np.float64)
    Ue = e["U"][:, -lead:]
    np.testing.assert_allclose(evd.align_signs(U[:, -lead:], Ue), Ue, rtol=0, atol=2e-6 * np.abs(Ue).max())
    # every 64-column chunk of U was written (the last chunk is ragged at k_out = 100)
    assert np.all(np.isfinite(U)) and np.all(np.abs(U).max(axis=0) > 0)


def test_mixed_evd_close_to_fp64(ctx, fac):
    from kernel_evd_gb300 import api
    X, r = fac
    F = torch.from_numpy(r["F"].astype(np.float32)).cuda()
    g = api.bistochastic_evd(ctx, F, k_out=16)
    e = evd.evd_from_factor(r["F"].astype(np.float32).astype(np.float64), 16)
    # the leading eigenpairs of the FP32 factor are Rayleigh-Ritz refined in FP64:
    # eigenvalue error <= 1e-8 against the FP64 EVD of the same factor
    assert abs(g.lam[-1] - 1.0) < 1e-8
    np.testing.assert_allclose(g.lam[-16:], e["lam"][-16:], rtol=0, atol=1e-8)
    ang = evd.eigvec_angles(g.U.cpu().numpy()[:, -4:], e["U"][:, -4:])
    assert np.all(ang < 1e-4)
    # the rest of the spectrum comes from the tensor-core Grams and the FP32 eigensolve of W
    np.testing.assert_allclose(g.lam[:-16], e["lam"][:-16], rtol=0, atol=1e-4)


def test_factor_from_linv_roundtrip(ctx, fac):
    from kernel_evd_gb300 import api
    X, r = fac
    Li = rpchol.linv_from_F(r["F"], r["piv"])
    Xt = torch.from_numpy(X).cuda()
    F = api.factor_from_linv(ctx, Xt, SCALE, r["piv"], Li, precision="fp64").cpu().numpy()
    np.testing.assert_allclose(F, r["F"], rtol=0, atol=1e-8)
    # L^{-1} is lower triangular: whatever its upper part holds is not read
    Lg = Li + np.triu(np.random.default_rng(0).standard_normal(Li.shape), 1)
    Fg = api.factor_from_linv(ctx, Xt, SCALE, r["piv"], Lg, precision="fp64").cpu().numpy()
    assert Fg.tobytes() == F.tobytes()
    e_lm = evd.evd_from_linv(X.astype(np.float64), SCALE, Li, r["piv"], 8)
    g = api.bistochastic_evd(ctx, torch.from_numpy(F).cuda(), k_out=8)
    np.testing.assert_allclose(g.lam[-8:], e_lm["lam"][-8:], rtol=1e-9)


def test_nonpositive_degree_is_reported(ctx, fac):
    from kernel_evd_gb300 import KevdError, api
    X, r = fac
    F = r["F"].copy()
    F[17, :] = 0.0          # an isolated row: dtil = 0 (the reference aborts with code 2)
    with pytest.raises(KevdError) as e:
        api.bistochastic_evd(ctx, torch.from_numpy(F).cuda(), k_out=4)
    assert e.value.name == "KEVD_ERR_NONPOS_DTIL"
    # the context stays usable
    g = api.bistochastic_evd(ctx, torch.from_numpy(r["F"]).cuda(), k_out=4)
    assert abs(g.lam[-1] - 1.0) < 1e-10


def test_indefinite_gram_is_reported(ctx, fac):
    from kernel_evd_gb300 import KevdError, api
    X, r = fac
    F = r["F"].copy()
    F[:, 5] = F[:, 4]       # rank-deficient factor: A is singular up to its rounding,
    F[:, 6] = F[:, 4]       # which the eps*tr(A) shift may or may not cover
    try:
        g = api.bistochastic_evd(ctx, torch.from_numpy(F).cuda(), k_out=4)
    except KevdError as e:
        # an indefinite shifted Gram is reported as the reference's potrf abort
        assert e.name == "KEVD_ERR_POTRF"
    else:
        # a shifted Gram that factors gives a usable decomposition: the
        # repeated columns add nothing to Khat = F F^T beyond the original ones
        assert np.all(np.isfinite(g.lam)) and abs(g.lam[-1] - 1.0) < 1e-8
        assert torch.isfinite(g.U).all()


def test_nystrom_reproduces_training_rows(ctx, fac):
    from kernel_evd_gb300 import api
    X, r = fac
    Xt = torch.from_numpy(X).cuda()
    g = api.rpcholesky(ctx, Xt, SCALE, k_max=200, block=32, seed=5, precision="fp64")
    e = api.bistochastic_evd(ctx, g.factor.contiguous(), k_out=8)
    model = api.NystromModel(ctx, Xt, g, k_out=8)
    idx = np.arange(0, 4000, 7)
    Uy = model(Xt[torch.from_numpy(idx).cuda()].contiguous()).cpu().numpy()
    U = e.U.cpu().numpy()[idx]
    np.testing.assert_allclose(Uy, U, rtol=0, atol=1e-5 * np.abs(U).max())


def test_factor_from_pivots_matches_oracle(ctx, fac):
    from kernel_evd_gb300 import api
    X, r = fac
    F = api.factor_from_pivots(ctx, torch.from_numpy(X).cuda(), SCALE, r["piv"][:200]).cpu().numpy()
    np.testing.assert_allclose(F, r["F"][:, :200], rtol=0, atol=1e-9)
