"""The C-ABI library loads and exports every entry point include/kevd.h declares
(no compute calls: these run without a GPU)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = open(os.path.join(ROOT, "include", "kevd.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(kevd_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    from kernel_evd_gb300 import _lib, build
    if not os.path.exists(_lib.LIB_PATH):
        build.build()
    return ctypes.CDLL(_lib.LIB_PATH)


def test_every_declared_symbol_is_exported(lib):
    names = _declared()
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header():
    from kernel_evd_gb300 import _lib
    assert set(_declared()) == set(_lib.SIGNATURES)


def test_status_names_and_version(lib):
    lib.kevd_status_name.restype = ctypes.c_char_p
    assert lib.kevd_status_name(0) == b"KEVD_OK"
    assert lib.kevd_status_name(3) == b"KEVD_ERR_NONPOS_DTIL"
    assert lib.kevd_abi_version() == 1


def test_select_is_host_only_and_matches_oracle(lib):
    import numpy as np
    from kernel_evd_gb300 import api
    from oracle import calibrate
    bw = calibrate.reference_sweep().astype(np.float64)
    T = np.exp(np.linspace(0.0, 12.0, bw.size)) * np.linspace(1.0, 3.0, bw.size)
    sel = api.select_bandwidth(bw, T, 5000)
    logS, slope, idmax, eopt, mdim = calibrate.select(bw, T, 5000)
    np.testing.assert_allclose(sel["logS"], logS, rtol=1e-15)
    np.testing.assert_allclose(sel["slope"], slope, rtol=1e-13)
    assert sel["idmax"] == idmax and sel["eopt"] == eopt
    assert api.bw0_text(bw, sel) == calibrate.bw0_text(bw, logS, slope, eopt, mdim)


def test_null_context_is_an_argument_error(lib):
    lib.kevd_calibrate.restype = ctypes.c_int
    assert lib.kevd_calibrate(None, None, 0, 0, None, 0, None, None) == 1


def test_server_arguments_and_footprint_without_gpu(lib):
    from kernel_evd_gb300 import _lib
    L = _lib.load()
    cfg = _lib.ServerConfig(0, 0, 4096, 1 << 30, 0.0)            # no factor worker
    h = ctypes.c_void_p()
    assert L.kevd_server_create(ctypes.byref(cfg), ctypes.byref(h)) == 1
    assert L.kevd_server_create(None, ctypes.byref(h)) == 1
    cfg = _lib.ServerConfig(0, 2, 0, 1 << 30, 0.0)               # empty query batch
    assert L.kevd_server_create(ctypes.byref(cfg), ctypes.byref(h)) == 1
    # footprint: F and its transposed copy dominate; FP64 factors cost more
    N, d, k = 2_000_000, 64, 2000
    fm = L.kevd_factorization_footprint(N, d, k, 32, 1)
    f64 = L.kevd_factorization_footprint(N, d, k, 32, 0)
    assert 2 * 4 * N * k < fm < 3 * 4 * N * k and f64 > fm + 2 * 4 * N * k
    assert L.kevd_factorization_footprint(0, d, k, 32, 1) == -1
    assert L.kevd_factorization_footprint(N, d, k, 32, 7) == -1
