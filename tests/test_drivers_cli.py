"""Run-time configuration of the stage drivers (kernel_evd_gb300/bin): with no
arguments they carry the reference's constants; flags and a JSON file override
them; a bad setting ends the program with status 2 before it opens a file or a
GPU.  ``--print-config`` resolves the settings and the file names without
touching either, so these tests run without a GPU."""
import json
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BIN = os.path.join(ROOT, "kernel_evd_gb300", "bin")


@pytest.fixture(scope="module")
def bindir():
    if not all(os.path.exists(os.path.join(BIN, p)) for p in ("cuband", "cuarpclm", "cukevd")):
        if not (shutil.which("nvcc") or os.path.exists("/usr/local/cuda/bin/nvcc")):
            pytest.skip("drivers not built and nvcc missing")
        from kernel_evd_gb300 import build
        build.build()
    return BIN


def _run(bindir, prog, *args, cwd=None):
    return subprocess.run([os.path.join(bindir, prog), *args], capture_output=True, text=True, timeout=60,
                          cwd=cwd)


def _settings(out):
    return dict(l.split(" = ", 1) for l in out.strip().split("\n"))


def test_defaults_are_the_reference_constants(bindir):
    r = _run(bindir, "cuband", "--print-config")
    assert r.returncode == 0, r.stderr
    s = _settings(r.stdout)
    # ks_bandwidth.cu:359-365
    assert (s["lfact"], s["mgrid"], s["ndata"], s["nq"]) == ("30", "128", "4607", "512")
    assert s["input"] == "data/ks_true_4607_128_30_u32.h5:/u"
    r = _run(bindir, "cukevd", "--print-config")
    s = _settings(r.stdout)
    # ks_kevd.cu:439-481 (k_out = 256) and ks_arpclm.cu:587-612 (Nq = 64, BLK = 512, bw = 0.8)
    assert (s["ndata"], s["nq"], s["blk"], s["kout"], s["precision"], s["dump"]) == \
        ("32831", "64", "512", "256", "mixed", "0")
    assert float(s["bw"]) == 0.8
    assert s["output"] == "data/evd_32768_128_64_256_30.h5:/lam,/U"


def test_flags_and_json_override(bindir, tmp_path):
    r = _run(bindir, "cuarpclm", "--ndata", "2000", "--mgrid=8", "--nq", "32", "--blk", "32", "--precision", "fp64",
             "--print-config")
    assert r.returncode == 0, r.stderr
    s = _settings(r.stdout)
    assert (s["ndata"], s["mgrid"], s["nq"], s["blk"], s["precision"]) == ("2000", "8", "32", "32", "fp64")
    assert "data/spiv_1969_8_b32_r8_30.h5:/spiv" in r.stdout
    cfg = tmp_path / "c.json"
    cfg.write_text(json.dumps({"ndata": 2000, "mgrid": 8, "nq": 32, "kout": 16, "precision": "fp64", "dump": True,
                               "bw": 0.5}))
    r = _run(bindir, "cukevd", "--config", str(cfg), "--kout", "8", "--print-config")
    assert r.returncode == 0, r.stderr
    s = _settings(r.stdout.replace("output = data/kevd", "dumpfile = data/kevd"))
    assert (s["kout"], s["precision"], s["dump"], float(s["bw"])) == ("8", "fp64", "1", 0.5)   # the flag wins
    assert s["dumpfile"] == "data/kevd_dump_1969_8_30.h5"


@pytest.mark.parametrize("args", [["--nope", "1"], ["--ndata", "12x"], ["--ndata", "-5"], ["--precision", "fp16"],
                                  ["--dump", "2"], ["--ndata"], ["stray"], ["--nq", "0"],
                                  ["--config", "/nonexistent/c.json"]])
def test_bad_settings_end_with_status_2(bindir, args, tmp_path):
    r = _run(bindir, "cukevd", *args, "--print-config", cwd=str(tmp_path))
    assert r.returncode == 2, (r.stdout, r.stderr)
    assert os.listdir(tmp_path) == []


@pytest.mark.parametrize("text", ['{"ndata": 2000,}', '{"ndata" 2000}', '[1, 2]', '{"ndata": 2000} x',
                                  '{"a\\"b": 1}'])
def test_malformed_json_is_rejected(bindir, tmp_path, text):
    cfg = tmp_path / "c.json"
    cfg.write_text(text)
    r = _run(bindir, "cuband", "--config", str(cfg), "--print-config")
    assert r.returncode == 2, (text, r.stdout, r.stderr)


def test_help_lists_every_setting(bindir):
    r = _run(bindir, "cukevd", "--help")
    assert r.returncode == 0
    for key in ("lfact", "mgrid", "ndata", "nq", "blk", "nrounds", "bw", "kout", "precision", "dump", "memcheck"):
        assert f"--{key}" in r.stdout
