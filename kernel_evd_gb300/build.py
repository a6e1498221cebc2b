"""Build the kevd CUDA library in-tree for sm_103a.

``python -m kernel_evd_gb300.build`` compiles every ``csrc/*.cu`` translation
unit in parallel with nvcc (one ``-gencode``, ``-lineinfo``) and links
``kernel_evd_gb300/lib/libkevd.so`` against cuBLAS and cuSOLVER; the host KS generator
(``csrc/host/ksgen.c``) is compiled with gcc into ``lib/libksgen.so`` and the HDF5
dataset layer (``csrc/host/h5file.c``) into ``lib/libkevdh5.so``.  The drivers
(``csrc/drivers/*.cpp``) are linked against both into ``kernel_evd_gb300/bin``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
BINDIR = os.path.join(HERE, "bin")
LIB = os.path.join(LIBDIR, "libkevd.so")
KSGEN = os.path.join(LIBDIR, "libksgen.so")
H5LIB = os.path.join(LIBDIR, "libkevdh5.so")
INCLUDE = os.path.join(HERE, "..", "include")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r.stdout + r.stderr


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def build_h5() -> str:
    """The HDF5 dataset layer alone (host C, no CUDA)."""
    os.makedirs(LIBDIR, exist_ok=True)
    cc = shutil.which("gcc") or shutil.which("cc")
    _run([cc, "-O2", "-std=c11", "-Wall", "-fPIC", "-shared", "-I", INCLUDE, "-o", H5LIB,
          os.path.join(CSRC, "host", "h5file.c"), "-lm"])
    return H5LIB


def build(verbose: bool = False, ptxas_info: bool = False) -> str:
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    flags = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
                    "--expt-relaxed-constexpr", "-I", os.path.join(HERE, "..", "include")]
    if ptxas_info:
        flags += ["-Xptxas", "-v"]
    objs, jobs = [], []
    with cf.ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
        for src in sources():
            obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
            objs.append(obj)
            jobs.append(ex.submit(_run, [nvcc, *flags, "-c", src, "-o", obj]))
        logs = [j.result() for j in jobs]
    _run([nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-lcublas", "-lcusolver", "-lcudart", "-lpthread"])
    cc = shutil.which("gcc") or shutil.which("cc")
    _run([cc, "-O3", "-std=c11", "-fPIC", "-shared", "-o", KSGEN,
          os.path.join(CSRC, "host", "ksgen.c"), "-lm"])
    build_h5()
    drivers = os.path.join(CSRC, "drivers")
    if os.path.isdir(drivers):
        os.makedirs(BINDIR, exist_ok=True)
        for f in sorted(os.listdir(drivers)):
            if f.endswith(".cpp"):
                exe = os.path.join(BINDIR, f[:-4])
                _run([nvcc, *ARCH, "-O2", "-std=c++17", "-I", os.path.join(HERE, "..", "include"),
                      os.path.join(drivers, f), "-o", exe, "-L", LIBDIR, "-lkevd", "-lkevdh5",
                      "-Xlinker", "-rpath", "-Xlinker", "$ORIGIN/../lib"])
    if verbose:
        for l in logs:
            if l.strip():
                print(l)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, ptxas_info="--ptxas" in sys.argv))
