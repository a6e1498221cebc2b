"""Serving loop and out-of-sample eigenfunctions on the GPU.

* the fused Nystrom kernel against the FP64 oracle extension (oracle/nystrom.py);
* batch invariance: a state's eigenfunction values are bit-identical whatever
  batch it is evaluated in;
* the server: a query answered alone and the same query answered in a mix of
  other queries, with factorizations running beside it, are identical; a
  factorization repeated in the mix gives the same model (eigenfunction values
  within 1e-6 of their maximum, FP32 output); admission by HBM footprint.
"""
import numpy as np
import pytest
import torch

from oracle import evd, ks, nystrom

pytestmark = pytest.mark.gpu

SCALE = 1.0 / 30.0


@pytest.fixture(scope="module")
def states():
    S = ks.seeded_mode(9000, warm_time=100.0).astype(np.float32)
    return S[:6000], S[6000:]          # training states, fresh states


@pytest.fixture(scope="module")
def model64(ctx, states):
    from kernel_evd_gb300 import api
    X, _ = states
    Xt = torch.from_numpy(X).cuda()
    fac = api.rpcholesky(ctx, Xt, SCALE, k_max=256, block=32, seed=3, precision="fp64")
    m = api.NystromModel(ctx, Xt, fac, k_out=8)
    yield fac, m
    m.close()


def _align(U, Uref):
    s = np.sign(np.sum(U * Uref, axis=0))
    s[s == 0] = 1.0
    return U * s[None, :]


def test_nystrom_matches_fp64_oracle(ctx, states, model64):
    X, Y = states
    fac, m = model64
    Uy = m(torch.from_numpy(Y).cuda()).cpu().numpy().astype(np.float64)
    F = fac.factor.cpu().numpy()
    om = nystrom.nystrom_model(X, SCALE, fac.piv, F, 8)
    ref = nystrom.nystrom_eval(om, Y)
    # FP32 output of an FP64 evaluation
    np.testing.assert_allclose(_align(Uy, ref), ref, rtol=0, atol=2e-6 * np.abs(ref).max())
    # training rows reproduce the EVD's U
    e = evd.evd_from_factor(F, 8)
    idx = np.arange(0, X.shape[0], 13)
    Ux = m(torch.from_numpy(X[idx]).cuda()).cpu().numpy().astype(np.float64)
    np.testing.assert_allclose(_align(Ux, e["U"][idx]), e["U"][idx], rtol=0, atol=2e-6 * np.abs(e["U"]).max())


def test_nystrom_batch_invariance(ctx, states, model64):
    _, Y = states
    _, m = model64
    Yt = torch.from_numpy(Y).cuda()
    whole = m(Yt).cpu().numpy()
    rng = np.random.default_rng(0)
    cuts = np.sort(rng.choice(np.arange(1, Y.shape[0]), size=40, replace=False))
    parts = [m(Yt[a:b].contiguous()).cpu().numpy() for a, b in zip(np.r_[0, cuts], np.r_[cuts, Y.shape[0]])]
    assert np.array_equal(np.concatenate(parts), whole)
    for i in rng.choice(Y.shape[0], size=10, replace=False):
        assert np.array_equal(m(Yt[i:i + 1].contiguous()).cpu().numpy()[0], whole[i])
    perm = rng.permutation(Y.shape[0])
    shuffled = m(Yt[torch.from_numpy(perm).cuda()].contiguous()).cpu().numpy()
    assert np.array_equal(shuffled, whole[perm])


def test_server_same_alone_and_in_the_mix(states):
    from kernel_evd_gb300 import api
    X, Y = states
    Xb = ks.seeded_mode(20000, warm_time=50.0).astype(np.float32)
    q = Y[:300]
    with api.Server(factor_workers=2, max_query_batch=4096, batch_window_us=200.0) as srv:
        # alone
        r1 = srv.wait(srv.submit_factorization(X, SCALE, k=256, block=32, k_out=8, seed=3))
        assert r1.rank == 256 and r1.trace_error > 0
        rid, out_alone = srv.submit_query(r1.model_id, q, 8)
        ra = srv.wait(rid)
        assert ra.batch_rows == q.shape[0]
        # the mix: the same factorization and a larger one run while queries of
        # many sizes, the same query among them, pile up against the first model
        f_again = srv.submit_factorization(X, SCALE, k=256, block=32, k_out=8, seed=3)
        f_big = srv.submit_factorization(Xb, SCALE, k=512, block=64, k_out=8, seed=4)
        rng = np.random.default_rng(1)
        pending = []
        for i in range(60):
            n = int(rng.integers(1, 400))
            a = int(rng.integers(0, Y.shape[0] - n))
            pending.append(srv.submit_query(r1.model_id, Y[a:a + n], 8) + (a, n))
            if i == 30:
                pending.append(srv.submit_query(r1.model_id, q, 8) + (0, q.shape[0]))
        mixed = [(srv.wait(rid), out, a, n) for rid, out, a, n in pending]
        assert max(r.batch_rows - n for r, _, _, n in mixed) > 0, "no query was batched with another"
        for r, out, a, n in mixed:
            if a == 0 and n == q.shape[0]:
                assert np.array_equal(out, out_alone)
        # each query equals its rows evaluated alone
        r_solo, out_solo = srv.submit_query(r1.model_id, Y[:400], 8)
        srv.wait(r_solo)
        for r, out, a, n in mixed[:10]:
            if a + n <= 400:
                assert np.array_equal(out, out_solo[a:a + n])
        rf = srv.wait(f_again)
        rb = srv.wait(f_big)
        assert rb.rank == 512
        assert rf.rank == r1.rank and rf.trace_error == pytest.approx(r1.trace_error, rel=1e-12)
        rid2, out_again = srv.submit_query(rf.model_id, q, 8)
        srv.wait(rid2)
        np.testing.assert_allclose(_align(out_again, out_alone), out_alone, rtol=0,
                                   atol=1e-6 * np.abs(out_alone).max())
        st = srv.stats("query")
        assert st["count"] >= 62 and 0 < st["p50_s"] <= st["p99_s"]
        assert srv.stats("factorization")["count"] == 3


def test_server_admission_by_footprint(states):
    from kernel_evd_gb300 import api
    X, _ = states
    fp = api.factorization_footprint(X.shape[0], X.shape[1], 192, 8, "mixed")
    assert fp > 4 * X.shape[0] * 192
    mb = api.model_bytes(192, X.shape[1], 8)
    # room for one running factorization (plus the models it leaves behind)
    with api.Server(factor_workers=2, hbm_budget_bytes=fp + 4 * mb) as srv:
        ids = [srv.submit_factorization(X, SCALE, k=192, block=32, k_out=8, seed=s) for s in range(3)]
        res = [srv.wait(i) for i in ids]
        mem = srv.memory()
        assert mem["peak_active"] == 1 and mem["models"] == 3 and mem["active"] == 0
        # charged: the resident models plus the workspaces the workers keep
        models = sum(api.model_bytes(r.rank, X.shape[1], 8) for r in res)
        assert mem["used_bytes"] >= models
        with pytest.raises(api.KevdError) as ei:
            srv.submit_factorization(np.zeros((200000, 64), np.float32), SCALE, k=2000, k_out=8)
        assert ei.value.name == "KEVD_ERR_NOMEM"
        before = srv.memory()["used_bytes"]
        srv.release_model(res[0].model_id)
        after = srv.memory()
        assert after["models"] == 2
        assert before - after["used_bytes"] == api.model_bytes(res[0].rank, X.shape[1], 8)
        with pytest.raises(api.KevdError):
            srv.submit_query(res[0].model_id, X[:4], 8)
    # room for two: both workers run at once
    with api.Server(factor_workers=2, hbm_budget_bytes=4 * fp) as srv:
        ids = [srv.submit_factorization(X, SCALE, k=192, block=32, k_out=8, seed=s) for s in range(3)]
        for i in ids:
            srv.wait(i)
        assert srv.memory()["peak_active"] == 2
