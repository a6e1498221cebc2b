"""The allocation-free calibration entry point against the regular one, through
the C ABI.

kevd_calibrate_noalloc serves callers that cannot call cudaMalloc: a process
whose device memory belongs to a pool it does not own (another framework's
caching allocator, or a host that gives a plugin a fixed budget), or a service
that forbids allocation once it has started.  Its scratch is a fixed device
array shared by every call, so these tests check that consecutive calls do not
see each other's leftovers, that a fresh process (first call on the device)
gets the same answer, and that sizes beyond the array are refused.

Collected last on purpose: a failure here leaves every other test already run."""
import os
import subprocess
import sys

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _states(n, seed):
    from oracle import ks
    return ks.seeded_mode(n, warm_time=50.0, seed=seed).astype(np.float32)


def _scales(nsc, med=100.0):
    return 1.0 / (med * 2.0 ** np.linspace(-10, 10, nsc))


def test_noalloc_matches_calibrate_twice_in_a_row(ctx):
    from kernel_evd_gb300 import api
    # two calls in a row with different inputs and sizes: the second must not
    # see anything left by the first
    for n, nsc, seed in ((1500, 41, 3), (333, 17, 4)):
        X = torch.from_numpy(_states(n, seed)).cuda()
        scales = _scales(nsc)
        ref = api.calibrate(ctx, X, scales)
        got = api.calibrate_noalloc(X, scales)
        # same kernels, a different split of the tile range over CTAs: FP64 partial
        # sums in another order
        np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-300)


def test_noalloc_single_state_has_no_pairs():
    from kernel_evd_gb300 import api
    # after a call that filled the scratch, N = 1 (no pair at all) must give zeros
    X = torch.from_numpy(_states(700, 6)).cuda()
    assert np.all(api.calibrate_noalloc(X, _scales(20)) > 0)
    got = api.calibrate_noalloc(X[:1].contiguous(), _scales(20))
    assert np.array_equal(got, np.zeros(20))


def test_noalloc_wide_states_on_a_side_stream(ctx):
    from kernel_evd_gb300 import api
    # d = 300 stages the features in several chunks; the call runs on a stream
    # other than the default one, ordered after the copy that fills X there
    Xh = np.random.default_rng(7).standard_normal((900, 300)).astype(np.float32)
    side = torch.cuda.Stream()
    with torch.cuda.stream(side):
        X = torch.from_numpy(Xh).cuda(non_blocking=False)
        scales = _scales(33, med=600.0)
        got = api.calibrate_noalloc(X, scales)
        ref = api.calibrate(ctx, X, scales)
    torch.cuda.synchronize()
    np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-300)


def test_noalloc_first_call_in_a_fresh_process(ctx, tmp_path):
    from kernel_evd_gb300 import api
    # the first call in a process resolves the scratch address on the device;
    # a child process makes that call twice and writes its sums
    X = _states(1200, 8)
    scales = _scales(41)
    np.save(tmp_path / "x.npy", X)
    np.save(tmp_path / "s.npy", scales)
    code = (
        "import sys, numpy as np, torch\n"
        f"sys.path.insert(0, {ROOT!r})\n"
        "from kernel_evd_gb300 import api\n"
        f"X = torch.from_numpy(np.load({str(tmp_path / 'x.npy')!r})).cuda()\n"
        f"s = np.load({str(tmp_path / 's.npy')!r})\n"
        "a = api.calibrate_noalloc(X, s)\n"
        "b = api.calibrate_noalloc(X, s)\n"
        f"np.save({str(tmp_path / 'out.npy')!r}, np.stack([a, b]))\n")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    out = np.load(tmp_path / "out.npy")
    ref = api.calibrate(ctx, torch.from_numpy(X).cuda(), scales)
    np.testing.assert_allclose(out[0], ref, rtol=1e-12, atol=1e-300)
    assert np.array_equal(out[0], out[1])


def test_noalloc_rejects_too_many_scales():
    from kernel_evd_gb300 import KevdError, api
    X = torch.from_numpy(_states(64, 5)).cuda()
    with pytest.raises(KevdError) as e:
        api.calibrate_noalloc(X, np.full(65, 0.01))
    assert e.value.name == "KEVD_ERR_ARG"
