"""Generate golden fixtures by running the reference's own Python programs.

Run in a container where the reference tree is mounted (default
``/root/reference``, override with ``KEVD_REFERENCE``); the outputs are committed
as ``tests/golden/*.npz`` so the tests never need the reference at run time.

The reference programs hard-code their problem sizes and write HDF5 through
h5py (absent here).  This script therefore
  * injects a minimal in-memory ``h5py`` stand-in that records datasets, and
  * shrinks the size constants in the program text before executing it
    (``Nequil``/``Nfinal`` of ks_datagen.py, ``Ntrue`` of ks_preproc.py,
    ``N`` of ks_reference.py); the algorithms run unmodified.

``--check-h5`` runs the same three programs again with this repository's HDF5
layer in place of h5py (``kernel_evd_gb300.h5.h5py_module()``), in a scratch
directory, writing real HDF5 files, and checks that every dataset read back from
them equals the committed fixture bit for bit.
"""
from __future__ import annotations

import os
import re
import sys
import types

import numpy as np

REF = os.environ.get("KEVD_REFERENCE", "/root/reference")
HERE = os.path.dirname(os.path.abspath(__file__))

_store: dict[str, np.ndarray] = {}


class _DS:
    def __init__(self, arr):
        self._a = arr

    def __getitem__(self, key):
        return self._a[key]


class _File:
    def __init__(self, name, mode="r"):
        self.name, self.mode = os.path.basename(name), mode

    def __enter__(self):
        return self

    def __exit__(self, *a):
        return False

    def create_dataset(self, key, shape=None, dtype=None, data=None):
        _store[f"{self.name}:{key}"] = np.array(data, dtype=dtype).reshape(shape)

    def __getitem__(self, key):
        return _DS(_store[f"{self.name}:{key}"])


def _install_h5py():
    m = types.ModuleType("h5py")
    m.File = _File
    sys.modules["h5py"] = m


def _run(fname, subs):
    src = open(os.path.join(REF, fname)).read()
    for pat, rep in subs:
        src, n = re.subn(pat, rep, src)
        assert n == 1, (fname, pat, n)
    ns = {"__name__": f"ref_{fname[:-3]}"}
    exec(compile(src, os.path.join(REF, fname), "exec"), ns)
    ns["main"]()
    return ns


def main():
    _install_h5py()
    out = {}
    # 1. ks_datagen.py with a short warm-up and a short record (chaos makes any
    #    long trajectory incomparable at the last bit).
    _run("ks_datagen.py", [(r"Nequil = 10000", "Nequil = 40"), (r"Nfinal = 512", "Nfinal = 32")])
    Ntrue, M = 32 + 64 - 1, 64
    u = _store[f"ks_true_{Ntrue}_{M}_7.h5:u"]
    out["datagen_u"] = u.reshape((Ntrue, M), order="F")          # (time, gridpoint)
    out["datagen_t"] = _store[f"ks_true_{Ntrue}_{M}_7.h5:t"]
    out["datagen_u32"] = _store[f"ks_true_{Ntrue}_{M}_7_u32.h5:u"]  # flat, time fastest
    # 2. ks_preproc.py on that record: delay embedding, time-major sample order.
    _run("ks_preproc.py", [(r"Ntrue = 575", f"Ntrue = {Ntrue}")])
    N = Ntrue - 64 + 1
    NM = N * M
    ud = _store[f"ks_train_{NM}_64_7_udelay.h5:u"].reshape((NM, 64), order="F")
    out["udelay"] = ud
    # 3. ks_reference.py: dense FP64 bistochastic EVD at eps = 0.8.
    _run("ks_reference.py", [(r"N = 512 ", f"N = {N} ")])
    w = _store[f"evd_ref_{N}_{M}_64_7.h5:eigvals"]
    V = _store[f"evd_ref_{N}_{M}_64_7.h5:eigvecs"].reshape((NM, NM), order="F")
    out["ref_eigvals"] = w
    out["ref_eigvecs_top16"] = V[:, :16].copy()
    out["ref_eps"] = np.array(0.8)
    out["ref_Nq"] = np.array(64)
    np.savez_compressed(os.path.join(HERE, "ks_reference_small.npz"), **out)
    print("wrote ks_reference_small.npz:", {k: v.shape for k, v in out.items()})


def check_h5_layer():
    import tempfile
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    from kernel_evd_gb300 import h5
    sys.modules["h5py"] = h5.h5py_module()
    g = np.load(os.path.join(HERE, "ks_reference_small.npz"))
    cwd = os.getcwd()
    with tempfile.TemporaryDirectory() as d:
        os.chdir(d)
        os.makedirs("data")
        try:
            _run("ks_datagen.py", [(r"Nequil = 10000", "Nequil = 40"), (r"Nfinal = 512", "Nfinal = 32")])
            Ntrue, M = 32 + 64 - 1, 64
            _run("ks_preproc.py", [(r"Ntrue = 575", f"Ntrue = {Ntrue}")])
            N = Ntrue - 64 + 1
            _run("ks_reference.py", [(r"N = 512 ", f"N = {N} ")])
            f = f"data/ks_true_{Ntrue}_{M}_7"
            got = {
                "datagen_u": h5.read(f + ".h5", "/u").reshape((Ntrue, M), order="F"),
                "datagen_t": h5.read(f + ".h5", "/t"),
                "datagen_u32": h5.read(f + "_u32.h5", "/u"),
                "udelay": h5.read(f"data/ks_train_{N * M}_64_7_udelay.h5", "/u").reshape((N * M, 64), order="F"),
                "ref_eigvals": h5.read(f"data/evd_ref_{N}_{M}_64_7.h5", "/eigvals"),
                "ref_eigvecs_top16": h5.read(f"data/evd_ref_{N}_{M}_64_7.h5", "/eigvecs").reshape(
                    (N * M, N * M), order="F")[:, :16],
            }
        finally:
            os.chdir(cwd)
    bad = [k for k, v in got.items() if v.dtype != g[k].dtype or v.tobytes() != g[k].tobytes()]
    print("HDF5 round trip of the reference's programs:", "all equal" if not bad else f"differ: {bad}")
    return not bad


if __name__ == "__main__":
    if "--check-h5" in sys.argv:
        sys.exit(0 if check_h5_layer() else 1)
    main()
