"""CPU checks of the oracle against the reference's own outputs (golden fixtures)
and published known-answer vectors."""
import numpy as np
import pytest

from oracle import calibrate, dense, evd, kernel, ks, philox, rpchol


def test_philox_known_answers():
    # Random123 known-answer vectors for philox4x32-10
    z = np.uint64(0)
    assert [int(v) for v in philox.philox4x32(z, z, z, z, z, z)] == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    m = np.uint64(0xFFFFFFFF)
    assert [int(v) for v in philox.philox4x32(m, m, m, m, m, m)] == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    c = [np.uint64(v) for v in (0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344, 0xA4093822, 0x299F31D0)]
    assert [int(v) for v in philox.philox4x32(*c)] == [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def test_uniforms_range():
    u = philox.uniforms(7, 3, 1, 10000)
    assert u.min() > 0.0 and u.max() <= 1.0
    assert abs(u.mean() - 0.5) < 0.02


def test_ks_generator_matches_reference(golden):
    u = ks.reference_mode(95, n_warm=40)
    np.testing.assert_array_equal(u, golden["datagen_u"])


def test_hankel_order_matches_reference_preproc(golden):
    u = golden["datagen_u"]                      # (time, gridpoint)
    X = kernel.hankel_rows(u.T.reshape(-1), 95, 64, 64)
    N, M = 32, 64
    Xt = X.reshape(M, N, 64).transpose(1, 0, 2).reshape(N * M, 64)  # time-major like ks_preproc.py
    np.testing.assert_array_equal(Xt, golden["udelay"])


def test_dense_evd_matches_reference(golden):
    w, V = dense.dense_evd(golden["udelay"], 1.0 / (64 * 0.8))
    np.testing.assert_allclose(w, golden["ref_eigvals"], rtol=0, atol=1e-13)
    V16 = evd.align_signs(V[:, :16], golden["ref_eigvecs_top16"])
    np.testing.assert_allclose(V16, golden["ref_eigvecs_top16"], rtol=0, atol=1e-11)


def test_full_rank_factor_reproduces_reference_dense_evd(golden):
    X = golden["udelay"]
    r = rpchol.rpcholesky(X, 1.0 / (64 * 0.8), 2048, 32, tol=1e-10, n_rounds=200, err_target=1e-13)
    e = evd.evd_from_factor(r["F"], 16)
    lam = e["lam"][::-1]
    np.testing.assert_allclose(lam[:16], golden["ref_eigvals"][:16], rtol=0, atol=1e-12)
    U = evd.align_signs(e["U"][:, ::-1], golden["ref_eigvecs_top16"])
    np.testing.assert_allclose(U, golden["ref_eigvecs_top16"], rtol=0, atol=1e-10)


@pytest.mark.parametrize("b", [1, 16])
def test_lm_form_matches_factor_form(golden, b):
    X = golden["udelay"]
    sc = 1.0 / (64 * 0.8)
    r = rpchol.rpcholesky(X, sc, 300, b, tol=1e-10)
    e1 = evd.evd_from_factor(r["F"], 16)
    Li = rpchol.linv_from_F(r["F"], r["piv"])
    e2 = evd.evd_from_linv(X, sc, Li, r["piv"], 16)
    np.testing.assert_allclose(e2["lam"], e1["lam"], rtol=0, atol=1e-13)
    np.testing.assert_allclose(np.abs(e2["U"]), np.abs(e1["U"]), rtol=0, atol=1e-11)


@pytest.mark.parametrize("b", [1, 16, 64])
def test_reference_round_algebra_matches_stored_factor(b):
    """The reference's low-memory rounds (L^{-1} and d only, K(R, S) regenerated per row
    block) and the stored-factor rounds make the same decisions on the same draws: the
    same pivots and accept counts, trace errors to 1e-13, and L^{-1} equal to the one
    recovered from F (measured: 3e-15 and 5e-14)."""
    X = ks.seeded_mode(1500, warm_time=50.0)
    sc = 1.0 / 30.0
    f = rpchol.rpcholesky(X, sc, 160, b, seed=11)
    g = rpchol.rpcholesky_linv(X, sc, 160, b, seed=11, rblk=512)
    np.testing.assert_array_equal(g["piv"], f["piv"])
    np.testing.assert_array_equal(g["hm"], f["hm"])
    np.testing.assert_allclose(g["err"], f["err"], rtol=1e-13, atol=0)
    np.testing.assert_allclose(g["d"], f["d"], rtol=0, atol=1e-13)
    Li = rpchol.linv_from_F(f["F"], f["piv"])
    np.testing.assert_allclose(g["Linv"], Li, rtol=0, atol=1e-12 * np.abs(Li).max())


def test_rpchol_trace_error_matches_factor():
    X = ks.seeded_mode(600, warm_time=50.0)
    sc = 1.0 / 30.0
    r = rpchol.rpcholesky(X, sc, 120, 8, seed=5)
    assert r["F"].shape[1] == 120
    direct = (X.shape[0] - (r["F"] ** 2).sum()) / X.shape[0]
    assert abs(r["err"][-1] - direct) < 1e-12
    assert np.all(np.diff(r["err"]) <= 1e-15)
    # residual diagonal of the factor equals d
    np.testing.assert_allclose(1.0 - (r["F"] ** 2).sum(1), r["d"], atol=1e-12)


def test_duplicate_proposals_are_rejected():
    X = ks.seeded_mode(200, warm_time=20.0)
    draws = {}

    def draw(rnd, stream, n):
        if stream == 0:
            return np.full(n, 0.37)           # every proposal the same row
        return np.full(n, 0.5)
    r = rpchol.rpcholesky(X, 1 / 30.0, 10, 4, n_rounds=1, draw=draw)
    assert r["hm"][0] == 1


def test_calibration_selection_reference_sweep():
    bw = calibrate.reference_sweep()
    assert bw.size == 36 and bw.dtype == np.float32
    assert np.isclose(bw[0], 1e-3) and np.isclose(bw[-1], 9.0)
    X = ks.seeded_mode(300, warm_time=20.0)
    T = calibrate.pair_sums(X, 1.0 / (64 * bw.astype(np.float64)))
    logS, slope, idmax, eopt, mdim = calibrate.select(bw, T, X.shape[0])
    assert 0 <= idmax < bw.size - 2
    assert eopt == float(bw[idmax + 1])
    assert np.isclose(mdim, 2 * slope[idmax])
    txt = calibrate.bw0_text(bw, logS, slope, eopt, mdim)
    assert len(txt.strip().split("\n")) == (bw.size - 2) + 3


@pytest.mark.parametrize("N", [2, 3, 7, 64, 1001])
def test_flat_triangle_index_is_a_bijection(N):
    """tri_ind maps 0 .. N(N-1)/2 - 1 onto the strict lower triangle, column by column."""
    total = N * (N - 1) // 2
    row, col = calibrate.tri_ind(np.arange(total), N)
    want_col, want_row = np.nonzero(np.tril(np.ones((N, N), dtype=bool), -1).T)
    np.testing.assert_array_equal(col, want_col)
    np.testing.assert_array_equal(row, want_row)


def test_flat_triangle_index_at_column_boundaries_of_large_matrices():
    """Where the square root rounds the wrong way: the first and last index of columns
    of the reference's calibration size (NM = 524,288) and of N = 4,194,304 agree with
    exact integer arithmetic."""
    rng = np.random.default_rng(3)
    for N in (524_288, 4_194_304):
        k = np.concatenate([np.arange(0, 64), N - 2 - np.arange(64), rng.integers(0, N - 1, 4000)])
        first = calibrate.tri_count(k, N)
        last = calibrate.tri_count(k + 1, N) - 1
        for p, want_col, want_row in ((first, k, k + 1), (last, k, np.full_like(k, N - 1))):
            row, col = calibrate.tri_ind(p, N)
            np.testing.assert_array_equal(col, want_col)
            np.testing.assert_array_equal(row, want_row)


def test_pair_sums_in_flat_order_match_blocked():
    X = ks.seeded_mode(700, warm_time=20.0)
    scales = 1.0 / np.array([0.5, 5.0, 50.0])
    np.testing.assert_allclose(calibrate.pair_sums_flat(X, scales, batch=10_000), calibrate.pair_sums(X, scales),
                               rtol=1e-12)


def test_pair_sums_bruteforce():
    rng = np.random.default_rng(0)
    X = rng.standard_normal((37, 5))
    sc = np.array([0.1, 1.0])
    T = calibrate.pair_sums(X, sc, block=8)
    brute = np.zeros(2)
    for i in range(37):
        for l in range(i):
            D = ((X[i] - X[l]) ** 2).sum()
            brute += np.exp(-sc * D)
    np.testing.assert_allclose(T, brute, rtol=1e-13)


def test_median_exact_vs_bruteforce():
    rng = np.random.default_rng(1)
    X = rng.standard_normal((41, 3))
    D = [((X[i] - X[l]) ** 2).sum() for i in range(41) for l in range(i)]
    assert calibrate.median_sqdist_exact(X, block=7) == sorted(D)[(len(D) - 1) // 2]
