"""The host KS generator (libksgen.so) against the oracle's NumPy ETDRK4 and the
reference generator's output."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def datagen():
    from kernel_evd_gb300 import build, datagen
    import os
    if not os.path.exists(datagen.LIB_PATH):
        build.build()
    return datagen


def test_short_horizon_matches_oracle(datagen):
    from oracle import ks
    a = datagen.seeded_states(400, warm_time=10.0, dtype=np.float64)
    b = ks.seeded_mode(400, warm_time=10.0)
    np.testing.assert_allclose(a, b, rtol=0, atol=1e-9)


def test_reference_settings_match_reference_generator(datagen, golden):
    a = datagen.reference_states(95, n_warm=40, dtype=np.float64)
    np.testing.assert_allclose(a, golden["datagen_u"], rtol=0, atol=1e-11)


def test_statistics_of_long_run(datagen):
    X = datagen.seeded_states(20000)
    assert X.dtype == np.float32 and X.shape == (20000, 64)
    assert np.all(np.isfinite(X))
    assert 1.0 < X.std() < 1.4          # KS L=22 attractor
    assert abs(X.mean()) < 0.05
