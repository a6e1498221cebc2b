"""ctypes binding of ``libkevdh5.so`` (include/kevd_h5.h): the HDF5 datasets the
reference's programs exchange ("/u", "/linv", "/spiv", "/lam", "/U"), read and
written without libhdf5.

``read`` mirrors the reference's ``h5read_*`` helpers (ks_bandwidth.cu:51-83,
ks_kevd.cu:134-243): the stored elements converted to the requested type.
``write`` mirrors ``h5write_*`` (ks_arpclm.cu:121-172, one file, one-dimensional
datasets), ``create`` + ``append`` the empty-file-then-``h5add_*`` pattern of
ks_kevd.cu:247-290 and :492-503.  The library is built in-tree with the rest
(``python -m kernel_evd_gb300.build``; ``build.build_h5()`` alone needs only gcc);
there is no fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.environ.get("KEVD_H5_LIB") or os.path.join(HERE, "lib", "libkevdh5.so")

F32, F64, I32, U32, I64, U64 = 1, 2, 3, 4, 5, 6
_TYPES = {np.dtype(np.float32): F32, np.dtype(np.float64): F64, np.dtype(np.int32): I32,
          np.dtype(np.uint32): U32, np.dtype(np.int64): I64, np.dtype(np.uint64): U64}
_DTYPES = {v: k for k, v in _TYPES.items()}

STATUS = {0: "KEVD_H5_OK", 1: "KEVD_H5_ERR_ARG", 2: "KEVD_H5_ERR_IO", 3: "KEVD_H5_ERR_FORMAT",
          4: "KEVD_H5_ERR_NOTFOUND", 5: "KEVD_H5_ERR_UNSUPPORTED"}

SIGNATURES = {
    "kevd_h5_last_error": (C.c_char_p, []),
    "kevd_h5_dataset_info": (C.c_int, [C.c_char_p, C.c_char_p, C.POINTER(C.c_int64), C.POINTER(C.c_int32),
                                       C.POINTER(C.c_int32), C.POINTER(C.c_int64)]),
    "kevd_h5_read": (C.c_int, [C.c_char_p, C.c_char_p, C.c_int32, C.c_void_p, C.c_int64]),
    "kevd_h5_list": (C.c_int, [C.c_char_p, C.c_char_p, C.c_int64, C.POINTER(C.c_int32)]),
    "kevd_h5_create": (C.c_int, [C.c_char_p]),
    "kevd_h5_append": (C.c_int, [C.c_char_p, C.c_char_p, C.c_int32, C.c_void_p, C.c_int64]),
    "kevd_h5_write": (C.c_int, [C.c_char_p, C.c_int32, C.POINTER(C.c_char_p), C.POINTER(C.c_int32),
                                C.POINTER(C.c_void_p), C.POINTER(C.c_int64)]),
}


class H5Error(RuntimeError):
    """A non-zero kevd_h5 status.  ``code`` is the enum value, ``name`` its name."""

    def __init__(self, code: int, msg: str):
        self.code = int(code)
        self.name = STATUS.get(self.code, "KEVD_H5_ERR_UNKNOWN")
        super().__init__(f"{self.name}: {msg}")


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise H5Error(2, f"{LIB_PATH} is not built (python -m kernel_evd_gb300.build)")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _check(status: int):
    if status != 0:
        raise H5Error(status, lib().kevd_h5_last_error().decode(errors="replace"))


def _b(s) -> bytes:
    return os.fsencode(s)


def info(path, name: str) -> dict:
    """Element count, stored type (a numpy dtype), rank and shape of a dataset."""
    n, t, r = C.c_int64(), C.c_int32(), C.c_int32()
    dims = (C.c_int64 * 32)()
    _check(lib().kevd_h5_dataset_info(_b(path), name.encode(), C.byref(n), C.byref(t), C.byref(r), dims))
    return {"count": n.value, "dtype": _DTYPES[t.value], "rank": r.value,
            "shape": tuple(dims[i] for i in range(r.value))}


def read(path, name: str, dtype=None, count: int | None = None) -> np.ndarray:
    """All elements of a dataset, flat, as ``dtype`` (default: the stored type).  With
    ``count`` given, a dataset of another size is an error (the reference's assert)."""
    meta = info(path, name)
    dt = np.dtype(dtype) if dtype is not None else meta["dtype"]
    if dt not in _TYPES:
        raise H5Error(1, f"unsupported element type {dt}")
    n = meta["count"] if count is None else int(count)
    out = np.empty(n, dtype=dt)
    _check(lib().kevd_h5_read(_b(path), name.encode(), _TYPES[dt], out.ctypes.data, n))
    return out


def names(path) -> list[str]:
    """Names in the root group."""
    cap = 1 << 16
    while True:
        buf = C.create_string_buffer(cap)
        n = C.c_int32()
        st = lib().kevd_h5_list(_b(path), buf, cap, C.byref(n))
        if st == 1 and cap < (1 << 26):
            cap *= 16
            continue
        _check(st)
        return [s.decode() for s in buf.raw.split(b"\0")[: n.value]]


def _flat(a) -> np.ndarray:
    a = np.ascontiguousarray(a).ravel()
    if a.dtype not in _TYPES:
        raise H5Error(1, f"unsupported element type {a.dtype}")
    return a


def create(path) -> None:
    """An empty HDF5 file (truncates)."""
    _check(lib().kevd_h5_create(_b(path)))


def append(path, name: str, a) -> None:
    """Adds ``a`` (flattened, C order) as the one-dimensional dataset ``name``."""
    a = _flat(a)
    _check(lib().kevd_h5_append(_b(path), name.encode(), _TYPES[a.dtype], a.ctypes.data, a.size))


def write(path, datasets: dict) -> None:
    """A new file holding ``{name: array}`` as one-dimensional datasets."""
    arrs = [(k, _flat(v)) for k, v in datasets.items()]
    n = len(arrs)
    nm = (C.c_char_p * max(n, 1))(*[k.encode() for k, _ in arrs])
    ty = (C.c_int32 * max(n, 1))(*[_TYPES[a.dtype] for _, a in arrs])
    da = (C.c_void_p * max(n, 1))(*[a.ctypes.data for _, a in arrs])
    ct = (C.c_int64 * max(n, 1))(*[a.size for _, a in arrs])
    _check(lib().kevd_h5_write(_b(path), n, nm, ty, da, ct))


# ---- the subset of h5py the reference's Python programs use --------------------
# ks_datagen.py:91-103, ks_preproc.py:17-32 and ks_reference.py:18-47 open files
# with ``h5py.File(path, "r" | "w")`` as a context manager, read ``f["u"][:]`` and
# write ``f.create_dataset(name, shape=(n,), dtype=..., data=...)``.  ``File``
# gives that surface over this library, and ``h5py_module()`` a module object to
# place in ``sys.modules["h5py"]`` so those programs run unmodified without h5py,
# writing files that the stage drivers (and libhdf5) read.

class Dataset:
    """A dataset of an open ``File``: shape, dtype, and indexing (``d[:]``, ``d[...]``)
    that reads the stored elements."""

    def __init__(self, path, name: str):
        self._path, self.name = path, name
        meta = info(path, name)
        self.shape, self.dtype, self.size = meta["shape"], meta["dtype"], meta["count"]

    def __len__(self):
        return self.shape[0] if self.shape else 1

    def __getitem__(self, key):
        return read(self._path, self.name).reshape(self.shape)[key]

    def __array__(self, dtype=None, copy=None):
        a = read(self._path, self.name).reshape(self.shape)
        return a if dtype is None else a.astype(dtype)


class File:
    """``File(path, mode)``: "r" reads, "w" creates (truncating), "a" / "r+" add
    datasets to an existing file ("a" creates it when missing)."""

    def __init__(self, path, mode: str = "r"):
        self.filename, self.mode = os.fspath(path), mode
        if mode == "w" or (mode == "a" and not os.path.exists(self.filename)):
            create(self.filename)
        elif mode in ("r", "r+", "a"):
            names(self.filename)          # fails now if the file is missing or not HDF5
        else:
            raise ValueError(f"unsupported mode {mode!r}")

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
        return False

    def close(self):
        pass                              # every call opens and closes the file itself

    def keys(self):
        return names(self.filename)

    def __contains__(self, name):
        return name.lstrip("/") in names(self.filename)

    def __iter__(self):
        return iter(self.keys())

    def __getitem__(self, name: str) -> Dataset:
        return Dataset(self.filename, name)

    def create_dataset(self, name: str, shape=None, dtype=None, data=None) -> Dataset:
        if self.mode == "r":
            raise H5Error(1, f"{self.filename} is open read-only")
        if data is None:
            if shape is None:
                raise ValueError("create_dataset needs shape or data")
            data = np.zeros(shape, dtype=dtype if dtype is not None else np.float32)
        a = np.asarray(data, dtype=dtype)
        if shape is not None:
            shape = (shape,) if np.isscalar(shape) else tuple(shape)
            a = a.reshape(shape)
        if a.ndim != 1:
            raise H5Error(5, "one-dimensional datasets only (as the reference writes them)")
        append(self.filename, name, a)
        return Dataset(self.filename, name)


def h5py_module():
    """A module with ``File``, for ``sys.modules["h5py"]``."""
    import types
    m = types.ModuleType("h5py")
    m.File = File
    m.Dataset = Dataset
    return m


def _main(argv=None) -> int:
    """``python -m kernel_evd_gb300.h5 FILE [DATASET]``: the root group's datasets
    with their element type and shape (like ``h5ls``), or one dataset's first values."""
    import argparse
    ap = argparse.ArgumentParser(prog="python -m kernel_evd_gb300.h5")
    ap.add_argument("file")
    ap.add_argument("dataset", nargs="?")
    ap.add_argument("-n", type=int, default=8, help="values shown with a dataset name")
    a = ap.parse_args(argv)
    try:
        if a.dataset:
            meta = info(a.file, a.dataset)
            v = read(a.file, a.dataset)
            print(f"{a.dataset}: {meta['dtype']} {meta['shape']}")
            print(" ".join(repr(x.item()) for x in v[: a.n]) + (" ..." if v.size > a.n else ""))
        else:
            for name in names(a.file):
                try:
                    meta = info(a.file, name)
                    print(f"{name:24s} {str(meta['dtype']):8s} {meta['shape']}")
                except H5Error as e:
                    print(f"{name:24s} ({e.name})")
    except H5Error as e:
        print(f"{a.file}: {e}")
        return 1
    return 0


if __name__ == "__main__":
    raise SystemExit(_main())
