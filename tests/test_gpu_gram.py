"""Weighted Gram G = F^T diag(s)^2 F: the FP32 factor on the tcgen05 tensor cores
(two-term f16 split scaled to max |F| and max s^2, FP64 across row chunks) and
the FP64 factor on the FP64 path, against NumPy FP64 on the same inputs."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


# Relative error bound of a Gram entry against sqrt(G_ii G_jj): the tensor-core
# FP32 accumulator rounds each MMA update with a one-sided bias, and a TMEM
# partial takes 1920 rows before its FP64 flush.
GRAM_RTOL = 6e-5


def _ref(F, s):
    Y = F.astype(np.float64) * s[:, None]
    return Y.T @ Y


@pytest.mark.parametrize("N,k,ld", [(5000, 300, 300), (4097, 128, 128), (100, 2, 2), (9000, 257, 257),
                                    (7000, 250, 256), (33, 129, 132), (20000, 130, 130)])
def test_gram_tc_fp32_factor(ctx, N, k, ld):
    from kernel_evd_gb300 import api
    rng = np.random.default_rng(N + k)
    Fb = rng.standard_normal((N, ld)).astype(np.float32)
    Fb[:, : k // 3] = np.abs(Fb[:, : k // 3]) + 0.5     # some columns with a large mean, like a kernel factor
    s = rng.uniform(0.5, 2.0, N)
    G = api.weighted_gram(ctx, torch.from_numpy(Fb).cuda()[:, :k] if ld != k else torch.from_numpy(Fb).cuda(),
                          torch.from_numpy(s).cuda(), k=k).cpu().numpy()
    R = _ref(Fb[:, :k], s)
    scale = np.sqrt(np.outer(np.diag(R), np.diag(R)))
    err = np.abs(G - R) / scale
    # two-term f16 products (22-bit hi/lo pieces); the tensor-core FP32
    # accumulator over 1920-row partials limits the relative error (FP64 across
    # partials)
    assert err.max() < GRAM_RTOL, err.max()
    np.testing.assert_allclose(G, G.T, rtol=0, atol=0)


@pytest.mark.parametrize("N,k,ld", [(5000, 300, 300), (4097, 128, 128), (100, 2, 2), (33, 129, 132),
                                    (70000, 260, 260)])
def test_gram2_tc_one_pass(ctx, N, k, ld):
    """Both Grams in one pass over F: the same values as two single-Gram calls,
    bit for bit (same split, MMA order and FP64 flushes per output tile)."""
    from kernel_evd_gb300 import api
    rng = np.random.default_rng(7 * N + k)
    Fb = rng.standard_normal((N, ld)).astype(np.float32)
    Fb[:, : k // 3] = np.abs(Fb[:, : k // 3]) + 0.5
    s = rng.uniform(0.5, 2.0, N)
    s2 = rng.uniform(0.1, 3.0, N)
    Ft = torch.from_numpy(Fb).cuda()
    Ft = Ft[:, :k] if ld != k else Ft
    st, s2t = torch.from_numpy(s).cuda(), torch.from_numpy(s2).cuda()
    G, G2 = api.weighted_gram2(ctx, Ft, st, s2t, k=k)
    assert torch.equal(G, api.weighted_gram(ctx, Ft, st, k=k))
    assert torch.equal(G2, api.weighted_gram(ctx, Ft, s2t, k=k))
    R2 = _ref(Fb[:, :k], s2)
    scale = np.sqrt(np.outer(np.diag(R2), np.diag(R2)))
    assert (np.abs(G2.cpu().numpy() - R2) / scale).max() < GRAM_RTOL


def test_gram2_tc_full_flush_length(ctx):
    """Row splits long enough for full 1920-row TMEM partials before each FP64
    flush (N = 300,000, k = 512: about 2,500 rows per split)."""
    from kernel_evd_gb300 import api
    N, k = 300_000, 512
    rng = np.random.default_rng(11)
    Fb = rng.standard_normal((N, k)).astype(np.float32)
    Fb[:, : k // 3] = np.abs(Fb[:, : k // 3]) + 0.5
    s = rng.uniform(0.5, 2.0, N)
    s2 = rng.uniform(0.1, 3.0, N)
    G, G2 = api.weighted_gram2(ctx, torch.from_numpy(Fb).cuda(), torch.from_numpy(s).cuda(),
                               torch.from_numpy(s2).cuda())
    for Gt, w in ((G, s), (G2, s2)):
        R = _ref(Fb, w)
        scale = np.sqrt(np.outer(np.diag(R), np.diag(R)))
        err = (np.abs(Gt.cpu().numpy() - R) / scale).max()
        assert err < GRAM_RTOL, err


def test_gram_fp64_factor(ctx):
    from kernel_evd_gb300 import api
    rng = np.random.default_rng(3)
    F = rng.standard_normal((3000, 170))
    s = rng.uniform(0.5, 2.0, 3000)
    G = api.weighted_gram(ctx, torch.from_numpy(F).cuda(), torch.from_numpy(s).cuda()).cpu().numpy()
    np.testing.assert_allclose(G, _ref(F, s), rtol=1e-12, atol=1e-10)


@pytest.mark.parametrize("spread", [1e2, 1e9])
def test_gram2_tc_weight_range(ctx, spread):
    """Row weights spanning a factor `spread` (s^2 spans its square): up to
    2^16 in s^2 the Grams take the f16 split, beyond it the tf32 split (the
    bistochastic weights of a nearly diagonal kernel span 1e17); both stay
    within the tolerance of FP64 sums."""
    from kernel_evd_gb300 import api
    N, k = 40000, 200
    rng = np.random.default_rng(5)
    Fb = rng.standard_normal((N, k)).astype(np.float32)
    Fb[:, : k // 3] = np.abs(Fb[:, : k // 3]) + 0.5
    s = np.exp(rng.uniform(-0.5, 0.5, N) * np.log(spread))
    s2 = np.exp(rng.uniform(-0.5, 0.5, N) * np.log(spread))
    G, G2 = api.weighted_gram2(ctx, torch.from_numpy(Fb).cuda(), torch.from_numpy(s).cuda(),
                               torch.from_numpy(s2).cuda())
    for Gt, w in ((G, s), (G2, s2)):
        R = _ref(Fb, w)
        scale = np.sqrt(np.outer(np.diag(R), np.diag(R)))
        err = (np.abs(Gt.cpu().numpy() - R) / scale).max()
        assert err < GRAM_RTOL, err
