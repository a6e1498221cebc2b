"""The allocation-free calibration entry point (for callers that cannot call
cudaMalloc: graph captures, foreign memory pools, allocation freezes) against
the regular entry point, through the C ABI.

Collected last on purpose: it is the only test that uses the library's fixed
device scratch array, and it must also pass in a fresh process on its own."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _states(n, seed):
    from oracle import ks
    return ks.seeded_mode(n, warm_time=50.0, seed=seed).astype(np.float32)


def test_noalloc_matches_calibrate_twice_in_a_row(ctx):
    from kernel_evd_gb300 import api
    # two calls in a row with different inputs and sizes: the second must not
    # see anything left by the first
    for n, nsc, seed in ((1500, 41, 3), (333, 17, 4)):
        X = torch.from_numpy(_states(n, seed)).cuda()
        scales = 1.0 / (100.0 * 2.0 ** np.linspace(-10, 10, nsc))
        ref = api.calibrate(ctx, X, scales)
        got = api.calibrate_noalloc(X, scales)
        # same kernels, a different split of the tile range over CTAs: FP64 partial
        # sums in another order
        np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-300)


def test_noalloc_rejects_too_many_scales():
    from kernel_evd_gb300 import KevdError, api
    X = torch.from_numpy(_states(64, 5)).cuda()
    with pytest.raises(KevdError) as e:
        api.calibrate_noalloc(X, np.full(65, 0.01))
    assert e.value.name == "KEVD_ERR_ARG"
