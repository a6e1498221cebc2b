"""The three stage drivers (cuband, cuarpclm, cukevd) run as the reference's
programs do: no arguments, compile-time configuration, HDF5 files under ./data
with the reference's names and datasets (/u, /linv, /spiv, /lam, /U), bw0.out
and the round table on stdout.  The built drivers (kernel_evd_gb300/bin) carry
the reference's own constants; these tests compile test-sized copies of the
same sources with -D overrides, as a user of the reference edits its constants,
and check their outputs against the FP64 oracle."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from kernel_evd_gb300 import h5
from oracle import calibrate, evd, kernel, ks, rpchol

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "kernel_evd_gb300", "csrc", "drivers")
LIBDIR = os.path.join(ROOT, "kernel_evd_gb300", "lib")
M, NQ, LFACT, BLK, NROUNDS, BW = 8, 32, 22, 32, 8, 0.8
DEFS = {"cuband": dict(LFACT=LFACT, MGRID=M, NDATA=600, NQ=NQ),
        "cuarpclm": dict(LFACT=LFACT, MGRID=M, NDATA=2000, NQ=NQ, BLK=BLK, NROUNDS=NROUNDS, BW=BW,
                         PRECISION="KEVD_FP64"),
        "cukevd": dict(LFACT=LFACT, MGRID=M, NDATA=2000, NQ=NQ, BLK=BLK, NROUNDS=NROUNDS, BW=BW, KOUT=16,
                       PRECISION="KEVD_FP64", DUMP_H5=1)}
# Relative (to the largest magnitude) agreement of the dump points with the
# reference's own algebra on the same L^{-1} and pivots: R and G carry the
# conditioning of chol(A + sI), p1 / pq and Z that of L^{-1}.
DUMP_TOL = dict(c1=1e-11, dtil=1e-11, cq=1e-11, qtil=1e-11, A=1e-10, Atil=1e-10, Btil=1e-10, W=1e-10,
                lam=1e-10, p1=1e-8, pq=1e-8, R=1e-7, G=1e-6)


@pytest.fixture(scope="module")
def bindir(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(os.path.join(LIBDIR, "libkevd.so")) or not os.path.exists(nvcc):
        pytest.skip("libkevd.so or nvcc missing")
    if not os.path.exists(os.path.join(LIBDIR, "libkevdh5.so")):
        from kernel_evd_gb300 import build
        build.build_h5()
    out = tmp_path_factory.mktemp("drivers")
    for prog, defs in DEFS.items():
        cmd = [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17",
               "-I", os.path.join(ROOT, "include"), *[f"-D{k}={v}" for k, v in defs.items()],
               os.path.join(SRC, prog + ".cpp"), "-o", str(out / prog), "-L", LIBDIR, "-lkevd", "-lkevdh5",
               "-Xlinker", "-rpath", "-Xlinker", LIBDIR]
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stdout + r.stderr
    return str(out)


def _write_u(d, ndata):
    S = ks.seeded_mode(ndata, M=64, seed=3, warm_time=60.0)       # ndata times x 64 gridpoints
    u = np.ascontiguousarray(S[:, :M].T).astype(np.float32)         # M gridpoints, time fastest
    h5.write(os.path.join(d, "data", f"ks_true_{ndata}_{M}_{LFACT}_u32.h5"), {"u": u.ravel()})
    return u.ravel()


def _run(bindir, d, prog):
    exe = os.path.join(bindir, prog)
    r = subprocess.run([exe], cwd=d, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


def test_cuband_selects_the_oracle_bandwidth(bindir, tmp_path):
    d = str(tmp_path)
    os.makedirs(os.path.join(d, "data"))
    u = _write_u(d, 600)
    out = _run(bindir, d, "cuband")
    assert "Total time:" in out
    lines = open(os.path.join(d, "bw0.out")).read().split("\n")
    eopt = float(lines[-3])
    X = kernel.hankel_rows(u, 600, M, NQ).astype(np.float64)
    bw = calibrate.reference_sweep().astype(np.float64)
    T = calibrate.pair_sums(X, 1.0 / (NQ * bw))
    logS, slope, idmax, eopt_ref, mdim = calibrate.select(bw, T, X.shape[0])
    assert eopt == pytest.approx(eopt_ref, rel=1e-5)
    got = np.array([[float(v) for v in l.split()] for l in lines[:len(bw) - 2]])
    np.testing.assert_allclose(got[:, 1], logS[1:-1], rtol=1e-4, atol=1e-6)


def test_run_time_flags_match_the_compiled_constants(bindir, tmp_path):
    """The in-tree cuband (the reference's constants) given the test constants as
    flags writes the same bw0.out, byte for byte, as the copy compiled with them."""
    exe = os.path.join(ROOT, "kernel_evd_gb300", "bin", "cuband")
    if not os.path.exists(exe):
        pytest.skip("in-tree drivers not built")
    runs = []
    for how in ("compiled", "flags"):
        d = str(tmp_path / how)
        os.makedirs(os.path.join(d, "data"))
        _write_u(d, 600)
        if how == "compiled":
            _run(bindir, d, "cuband")
        else:
            flags = [f"--{k.lower()}={v}" for k, v in DEFS["cuband"].items()]
            r = subprocess.run([exe, *flags], cwd=d, capture_output=True, text=True, timeout=600)
            assert r.returncode == 0, r.stdout + r.stderr
        runs.append(open(os.path.join(d, "bw0.out")).read())
    assert runs[0] == runs[1]


def test_cuarpclm_then_cukevd_match_the_oracle(bindir, tmp_path):
    d = str(tmp_path)
    os.makedirs(os.path.join(d, "data"))
    ndata = 2000
    u = _write_u(d, ndata)
    out = _run(bindir, d, "cuarpclm")
    assert "# round accepted cumrank relerr" in out
    N = ndata - NQ + 1
    spiv = h5.read(os.path.join(d, "data", f"spiv_{N}_{M}_b{BLK}_r{NROUNDS}_{LFACT}.h5"), "/spiv")
    linv = h5.read(os.path.join(d, "data", f"linv_{N}_{M}_b{BLK}_r{NROUNDS}_{LFACT}.h5"), "/linv")
    assert spiv.dtype == np.uint64 and linv.dtype == np.float64
    X = kernel.hankel_rows(u, ndata, M, NQ).astype(np.float64)
    scale = 1.0 / (NQ * BW)
    ref = rpchol.rpcholesky(X, scale, BLK * NROUNDS, BLK, seed=1234, n_rounds=NROUNDS)
    np.testing.assert_array_equal(spiv.astype(np.int64), ref["piv"])
    r = spiv.size
    Li = rpchol.linv_from_F(ref["F"], ref["piv"])
    np.testing.assert_allclose(linv.reshape(r, r, order="F"), Li, rtol=0, atol=1e-8 * np.abs(Li).max())
    run = subprocess.run([os.path.join(bindir, "cukevd"), "--memcheck=1"], cwd=d, capture_output=True, text=True,
                         timeout=600)
    assert run.returncode == 0, run.stdout + run.stderr
    mem = [l for l in run.stdout.split("\n") if l.startswith("MEM[")]
    assert [l[4:14].strip() for l in mem] == ["post-init", "pre-pass1", "post-pass4"]
    out_file = os.path.join(d, "data", f"evd_{N}_{M}_{NQ}_16_{LFACT}.h5")
    assert h5.names(out_file) == ["U", "lam"]
    lam = h5.read(out_file, "/lam")
    U = h5.read(out_file, "/U")
    assert lam.dtype == np.float64 and U.dtype == np.float32
    e = evd.evd_from_factor(ref["F"], 16)
    np.testing.assert_allclose(lam[-16:], e["lam"][-16:], rtol=0, atol=1e-9)
    assert U.size == X.shape[0] * 16
    # the optional dump file (ks_kevd.cu:533-542) against the reference's pass algebra
    dump = os.path.join(d, "data", f"kevd_dump_{N}_{M}_{LFACT}.h5")
    assert h5.names(dump) == sorted(list(DUMP_TOL) + ["Z", "U"])
    g = evd.evd_from_linv(X, scale, linv.reshape(r, r, order="F"), spiv.astype(np.int64), 16)
    for k, tol in DUMP_TOL.items():
        got, want = h5.read(dump, k), g[k].ravel(order="F")
        assert got.dtype == np.float64 and got.size == want.size, k
        assert np.max(np.abs(got - want)) <= tol * np.max(np.abs(want)), k
    Z = evd.align_signs(h5.read(dump, "Z").reshape(r, 16, order="F"), g["Z"])
    assert np.max(np.abs(Z - g["Z"])) <= 1e-8 * np.max(np.abs(g["Z"]))
    np.testing.assert_array_equal(h5.read(dump, "U"), U)
    Ug = evd.align_signs(U.reshape(-1, 16).astype(np.float64), g["U"])
    assert np.max(np.abs(Ug - g["U"])) <= 1e-5 * np.max(np.abs(g["U"]))
