"""HDF5 dataset layer (include/kevd_h5.h, libkevdh5.so): host code only, no GPU.

Pinning.  There is no libhdf5 or h5py here, but scipy ships one file that
libhdf5 wrote: a MATLAB 7.3 MAT-file (HDF5 behind a 512-byte user block) holding
the variable ``testdouble``, which scipy also ships saved as a MATLAB 7 MAT-file
that scipy itself reads.  The reader must return the same values bit for bit.
Files the writer makes are read back by that reader and walked here, in Python,
for what libhdf5 checks when it opens one (message counts, full-size B-tree and
symbol nodes inside the file, the local heap's free-list terminator, sorted
names and B-tree keys, the end-of-file address); the datatype messages are
compared byte for byte with the one libhdf5 wrote into the MATLAB file.
"""
import os
import re
import struct
import subprocess
import sys

import numpy as np
import pytest

from kernel_evd_gb300 import h5

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DTYPES = [np.float32, np.float64, np.int32, np.uint32, np.int64, np.uint64]


@pytest.fixture(scope="module", autouse=True)
def built():
    if not os.path.exists(h5.LIB_PATH):
        from kernel_evd_gb300 import build
        build.build_h5()


def _scipy_data():
    try:
        import scipy.io.matlab as m
    except ImportError:
        return None
    d = os.path.join(os.path.dirname(m.__file__), "tests", "data")
    ok = all(os.path.exists(os.path.join(d, f)) for f in ("testhdf5_7.4_GLNX86.mat", "testdouble_7.4_GLNX86.mat"))
    return d if ok else None


def _values(dt, n, seed):
    rng = np.random.default_rng(seed)
    dt = np.dtype(dt)
    if dt.kind == "f":
        return (rng.standard_normal(n) * 10.0 ** rng.integers(-30, 30, n)).astype(dt)
    info = np.iinfo(dt)
    return rng.integers(info.min, info.max, n, dtype=dt, endpoint=True)


def test_every_declared_symbol_is_exported():
    import ctypes
    src = open(os.path.join(ROOT, "include", "kevd_h5.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = sorted(set(re.findall(r"\b(kevd_h5_[a-z0-9_]+)\s*\(", src)))
    assert len(names) == 7
    lib = ctypes.CDLL(h5.LIB_PATH)
    assert [n for n in names if not hasattr(lib, n)] == []
    assert set(names) == set(h5.SIGNATURES)


def test_reads_a_file_written_by_libhdf5():
    d = _scipy_data()
    if d is None:
        pytest.skip("scipy's MAT-file test data are not installed")
    import scipy.io as sio
    path = os.path.join(d, "testhdf5_7.4_GLNX86.mat")
    assert h5.names(path) == ["testdouble"]
    meta = h5.info(path, "/testdouble")
    assert meta["dtype"] == np.float64 and meta["shape"] == (9, 1) and meta["count"] == 9
    want = sio.loadmat(os.path.join(d, "testdouble_7.4_GLNX86.mat"))["testdouble"].ravel()
    got = h5.read(path, "/testdouble")
    assert got.tobytes() == want.tobytes()
    np.testing.assert_array_equal(h5.read(path, "testdouble", np.float32), want.astype(np.float32))


def test_append_to_a_file_written_by_libhdf5(tmp_path):
    """Appending keeps the libhdf5-written dataset where it is (user block, its own
    B-tree K values) and adds the new one beside it."""
    d = _scipy_data()
    if d is None:
        pytest.skip("scipy's MAT-file test data are not installed")
    src = open(os.path.join(d, "testhdf5_7.4_GLNX86.mat"), "rb").read()
    p = tmp_path / "copy.mat"
    p.write_bytes(src)
    before = h5.read(p, "testdouble")
    extra = np.arange(40, dtype=np.uint64) * 3
    h5.append(p, "/extra", extra)
    after = p.read_bytes()
    assert after[:512] == src[:512]                                     # the user block is untouched
    assert h5.names(p) == ["extra", "testdouble"]
    assert h5.read(p, "testdouble").tobytes() == before.tobytes()
    assert h5.read(p, "extra").tobytes() == extra.tobytes()
    assert struct.unpack_from("<Q", after, 512 + 40)[0] == len(after)  # absolute end of file


@pytest.mark.parametrize("dt", DTYPES)
@pytest.mark.parametrize("n", [0, 1, 7, 100003])
def test_round_trip(tmp_path, dt, n):
    a = _values(dt, n, seed=n)
    p = tmp_path / "a.h5"
    h5.write(p, {"/x": a})
    meta = h5.info(p, "x")
    assert meta["dtype"] == np.dtype(dt) and meta["shape"] == (n,) and meta["rank"] == 1
    b = h5.read(p, "/x", count=n)
    assert b.dtype == np.dtype(dt) and b.tobytes() == a.tobytes()


def test_more_links_than_one_symbol_node(tmp_path):
    arrs = {f"ds{i:03d}": _values(DTYPES[i % 6], i, seed=i) for i in range(70, 0, -1)}
    p = tmp_path / "many.h5"
    h5.write(p, arrs)
    assert h5.names(p) == sorted(arrs)
    for k, a in arrs.items():
        assert h5.read(p, k).tobytes() == a.tobytes()
    _walk(p)


def test_append_as_the_reference_dump_file(tmp_path):
    p = tmp_path / "dump.h5"
    h5.create(p)
    assert h5.names(p) == []
    parts = {"c1": np.arange(5.0), "p1": np.linspace(0, 1, 11), "dtil": np.ones(3), "U": np.arange(6, dtype=np.float32),
             "lam": np.array([0.5, 1.0])}
    for k, v in parts.items():
        h5.append(p, "/" + k, v)
        _walk(p)
    assert h5.names(p) == sorted(parts)
    for k, v in parts.items():
        assert h5.read(p, k).tobytes() == v.tobytes()
    with pytest.raises(h5.H5Error) as e:
        h5.append(p, "c1", np.zeros(2))
    assert e.value.name == "KEVD_H5_ERR_ARG"
    with pytest.raises(h5.H5Error) as e:
        h5.read(p, "/nope")
    assert e.value.name == "KEVD_H5_ERR_NOTFOUND"
    with pytest.raises(h5.H5Error) as e:
        h5.read(p, "/c1", count=4)
    assert e.value.name == "KEVD_H5_ERR_ARG"
    with pytest.raises(h5.H5Error) as e:
        h5.info(p, "/")
    assert e.value.name == "KEVD_H5_ERR_ARG"
    for bad in ("", "/", "a/b"):
        with pytest.raises(h5.H5Error):
            h5.append(p, bad, np.zeros(1))
    with pytest.raises(h5.H5Error) as e:
        h5.read(tmp_path / "missing.h5", "x")
    assert e.value.name == "KEVD_H5_ERR_IO"


def test_conversions_follow_native_reads(tmp_path):
    p = tmp_path / "c.h5"
    f = np.array([0.0, -3.7, 3.7, 1e30, -1e30, np.inf, -np.inf, np.nan, 2.0 ** 40, 1.0 / 3.0])
    u = np.array([0, 1, 2 ** 63, 2 ** 64 - 1], dtype=np.uint64)
    i = np.array([-(2 ** 63), -5, 0, 7, 2 ** 62], dtype=np.int64)
    h5.write(p, {"f": f, "u": u, "i": i})
    np.testing.assert_array_equal(h5.read(p, "f", np.float32), f.astype(np.float32))
    np.testing.assert_array_equal(h5.read(p, "f", np.int32),
                                  [0, -3, 3, 2 ** 31 - 1, -(2 ** 31), 2 ** 31 - 1, -(2 ** 31), 0, 2 ** 31 - 1, 0])
    np.testing.assert_array_equal(h5.read(p, "f", np.uint64)[[0, 1, 2, 3, 7, 8]], [0, 0, 3, 2 ** 64 - 1, 0, 2 ** 40])
    np.testing.assert_array_equal(h5.read(p, "u", np.int64), [0, 1, 2 ** 63 - 1, 2 ** 63 - 1])
    np.testing.assert_array_equal(h5.read(p, "u", np.float64), u.astype(np.float64))
    np.testing.assert_array_equal(h5.read(p, "i", np.uint64), [0, 0, 0, 7, 2 ** 62])
    np.testing.assert_array_equal(h5.read(p, "i", np.int32), [-(2 ** 31), -5, 0, 7, 2 ** 31 - 1])
    np.testing.assert_array_equal(h5.read(p, "i", np.float32), i.astype(np.float32))


def test_version2_headers_link_messages_and_continuations(tmp_path):
    """A file in the newer layout (superblock version 2, object header version 2,
    links stored in the root group's header, one continuation block), built here
    from the format specification: the reader's second path."""
    p = tmp_path / "v2.h5"
    a = np.arange(12, dtype=np.float64) * 0.25
    b = np.arange(5, dtype=np.int32) - 2
    p.write_bytes(_v2_file({"alpha": a, "beta": b}))
    assert h5.names(p) == ["alpha", "beta"]
    assert h5.read(p, "/alpha").tobytes() == a.tobytes()
    assert h5.read(p, "beta").tobytes() == b.tobytes()
    with pytest.raises(h5.H5Error) as e:
        h5.append(p, "gamma", a)
    assert e.value.name == "KEVD_H5_ERR_UNSUPPORTED"


def test_h5py_subset_in_the_reference_call_pattern(tmp_path):
    """The calls of ks_datagen.py:91-103 and ks_preproc.py:17-32 (h5py.File as a context
    manager, create_dataset(name, shape, dtype, data), f["u"][:]) on the golden
    fixture's arrays, through ``h5.h5py_module()``: what is read equals what was written."""
    g = np.load(os.path.join(ROOT, "tests", "golden", "ks_reference_small.npz"))
    h5py = h5.h5py_module()
    usave = g["datagen_u"]
    Ntrue, M = usave.shape
    p = tmp_path / "ks_true.h5"
    with h5py.File(p, "w") as f:
        f.create_dataset("u", shape=(Ntrue * M,), dtype=np.float32, data=usave.astype(np.float32).flatten(order="F"))
        f.create_dataset("t", shape=(Ntrue,), dtype=np.float64, data=g["datagen_t"])
    with h5py.File(p, "r") as f:
        assert sorted(f.keys()) == ["t", "u"] and "u" in f and "/t" in f
        utrue = f["u"][:].reshape((Ntrue, M), order="F")
        assert f["u"].shape == (Ntrue * M,) and f["u"].dtype == np.float32 and len(f["t"]) == Ntrue
        assert np.asarray(f["t"]).tobytes() == g["datagen_t"].tobytes()
        with pytest.raises(h5.H5Error):
            f.create_dataset("x", data=np.zeros(3))
    assert utrue.tobytes() == usave.astype(np.float32).tobytes()
    assert h5.read(p, "/u").tobytes() == g["datagen_u32"].tobytes()     # what the drivers read
    with h5py.File(p, "a") as f:
        f.create_dataset("extra", data=np.arange(4))
    assert h5.names(p) == ["extra", "t", "u"]
    with pytest.raises(h5.H5Error):
        h5py.File(p, "w").create_dataset("m", data=np.zeros((2, 2)))
    with pytest.raises(h5.H5Error):
        h5py.File(tmp_path / "none.h5", "r")


def test_listing_tool(tmp_path):
    p = tmp_path / "l.h5"
    h5.write(p, {"lam": np.array([0.25, 0.5, 1.0]), "spiv": np.arange(5, dtype=np.uint64)})
    run = lambda *a: subprocess.run([sys.executable, "-m", "kernel_evd_gb300.h5", *a], cwd=ROOT,
                                    capture_output=True, text=True, timeout=60)
    r = run(str(p))
    assert r.returncode == 0 and r.stdout.split() == ["lam", "float64", "(3,)", "spiv", "uint64", "(5,)"]
    r = run(str(p), "/lam", "-n", "2")
    assert r.returncode == 0 and r.stdout.split("\n")[1] == "0.25 0.5 ..."
    r = run(str(tmp_path / "missing.h5"))
    assert r.returncode == 1 and "KEVD_H5_ERR_IO" in r.stdout


def test_reader_paths_the_writer_does_not_make(tmp_path):
    """Big-endian elements, 1- and 2-byte integers, a scalar and a 2-D dataspace, compact
    storage and a dataset inside a group, in a file built here from the specification."""
    f64 = np.linspace(-2.0, 3.0, 12).reshape(3, 4)
    i16 = np.array([-300, -1, 0, 1, 32767], dtype=np.int16)
    u8 = np.array([0, 7, 255], dtype=np.uint8)
    f32 = np.array([1.5, -2.25, 3.0e-8], dtype=np.float32)
    p = tmp_path / "paths.h5"
    p.write_bytes(_v2_file({"be2d": (f64, {"be": True}),
                            "i16be": (i16, {"be": True}),
                            "u8": u8,
                            "scalar": (np.array([0.75], dtype=np.float32), {"shape": ()}),
                            "compact": (np.arange(5, dtype=np.int32), {"compact": True}),
                            "f32be": (f32, {"be": True})},
                           group=("grp", {"x": np.array([4.0, 5.0])})))
    assert h5.names(p) == ["be2d", "i16be", "u8", "scalar", "compact", "f32be", "grp"]
    meta = h5.info(p, "be2d")
    assert meta["shape"] == (3, 4) and meta["dtype"] == np.float64
    assert h5.read(p, "be2d").tobytes() == f64.ravel().tobytes()
    assert h5.info(p, "i16be")["dtype"] == np.int32
    np.testing.assert_array_equal(h5.read(p, "i16be"), i16.astype(np.int32))
    assert h5.info(p, "u8")["dtype"] == np.uint32
    np.testing.assert_array_equal(h5.read(p, "u8", np.float64), u8.astype(np.float64))
    meta = h5.info(p, "scalar")
    assert meta["rank"] == 0 and meta["count"] == 1 and h5.read(p, "scalar")[0] == np.float32(0.75)
    np.testing.assert_array_equal(h5.read(p, "compact"), np.arange(5, dtype=np.int32))
    np.testing.assert_array_equal(h5.read(p, "/f32be", np.float64), f32.astype(np.float64))
    np.testing.assert_array_equal(h5.read(p, "/grp/x"), [4.0, 5.0])
    with pytest.raises(h5.H5Error) as e:
        h5.read(p, "/grp")
    assert e.value.name == "KEVD_H5_ERR_ARG"
    with pytest.raises(h5.H5Error) as e:
        h5.read(p, "/grp/y")
    assert e.value.name == "KEVD_H5_ERR_NOTFOUND"


def test_corrupt_files_are_errors_not_crashes(tmp_path):
    """Truncated or byte-flipped files end in a status, never in a crash (run in a
    child process so that a crash fails this test instead of the session)."""
    good = tmp_path / "good.h5"
    h5.write(good, {f"d{i}": np.arange(i + 1, dtype=DTYPES[i % 6]) for i in range(12)})
    script = r"""
import os, sys
import numpy as np
from kernel_evd_gb300 import h5
src = open(sys.argv[1], "rb").read()
rng = np.random.default_rng(5)
p = sys.argv[2]
seen = set()
for it in range(600):
    b = bytearray(src)
    if it % 3 == 0:
        b = b[: int(rng.integers(0, len(b)))]
    for _ in range(int(rng.integers(1, 5))):
        if b:
            b[int(rng.integers(0, len(b)))] = int(rng.integers(0, 256))
    open(p, "wb").write(bytes(b))
    for call in (lambda: h5.names(p), lambda: h5.read(p, "d7"), lambda: h5.info(p, "/d11")):
        try:
            call()
            seen.add("ok")
        except h5.H5Error as e:
            seen.add(e.name)
        except (MemoryError, ValueError, OverflowError, KeyError):
            seen.add("python")
print(sorted(seen))
"""
    r = subprocess.run([sys.executable, "-c", script, str(good), str(tmp_path / "bad.h5")], cwd=ROOT,
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "KEVD_H5_ERR_FORMAT" in r.stdout


# ----------------------------------------------------------------- structure walk

def _walk(path):
    """Checks a file this library wrote against what libhdf5 verifies on open."""
    b = open(path, "rb").read()
    assert b[:8] == b"\x89HDF\r\n\x1a\n" and b[8] == 0           # superblock version 0
    assert b[13] == 8 and b[14] == 8                            # offsets and lengths
    leaf_k, node_k = struct.unpack_from("<HH", b, 16)
    assert (leaf_k, node_k) == (4, 16)
    base, free, eof, drv = struct.unpack_from("<QQQQ", b, 24)
    assert base == 0 and free == drv == 2 ** 64 - 1 and eof == len(b)
    _, root, cache, _, bt, heap = struct.unpack_from("<QQIIQQ", b, 56)
    assert cache == 1
    msgs = _v1_messages(b, root)
    stab = [m for m in msgs if m[0] == 0x11]
    assert len(stab) == 1 and struct.unpack_from("<QQ", stab[0][2]) == (bt, heap)
    assert b[heap:heap + 4] == b"HEAP"
    hsize, hfree, hdata = struct.unpack_from("<QQQ", b, heap + 8)
    assert hfree == 1                                            # the free-list terminator
    names = b[hdata:hdata + hsize]
    assert names[:8] == bytes(8)

    def name(off):
        assert off % 8 == 0 and off < hsize
        return names[off:names.index(b"\0", off)]

    assert b[bt:bt + 6] == b"TREE\x00\x00"                        # group node, leaf level
    nent = struct.unpack_from("<H", b, bt + 6)[0]
    assert bt + 24 + (2 * node_k + 1) * 8 + 2 * node_k * 8 <= len(b)
    keys = [struct.unpack_from("<Q", b, bt + 24 + 16 * i)[0] for i in range(nent + 1)]
    kids = [struct.unpack_from("<Q", b, bt + 32 + 16 * i)[0] for i in range(nent)]
    assert keys[0] == 0
    all_names = []
    for i, s in enumerate(kids):
        assert b[s:s + 5] == b"SNOD\x01" and s + 8 + 2 * leaf_k * 40 <= len(b)
        nsym = struct.unpack_from("<H", b, s + 6)[0]
        assert 1 <= nsym <= 2 * leaf_k
        ents = [struct.unpack_from("<QQI", b, s + 8 + 40 * j) for j in range(nsym)]
        nm = [name(e[0]) for e in ents]
        assert nm == sorted(nm) and nm[-1] == name(keys[i + 1])
        assert all(name(keys[i]) < x for x in nm)
        for _, oh, ct in ents:
            assert ct == 0
            _check_dataset(b, oh, eof)
        all_names += nm
    assert all_names == sorted(set(all_names))
    return all_names


def _v1_messages(b, addr):
    ver, _, n, refc, size = struct.unpack_from("<BBHII", b, addr)
    assert ver == 1 and refc == 1 and size % 8 == 0
    out, p, end = [], addr + 16, addr + 16 + size
    while p + 8 <= end:
        t, ln, fl = struct.unpack_from("<HHB", b, p)
        assert ln % 8 == 0 and p + 8 + ln <= end
        out.append((t, fl, b[p + 8:p + 8 + ln]))
        p += 8 + ln
    assert p == end and len(out) == n                            # libhdf5 checks the count
    return out


_LIBHDF5_F64 = None


def _libhdf5_f64_message():
    """The float64 datatype message libhdf5 wrote for ``testdouble``."""
    global _LIBHDF5_F64
    d = _scipy_data()
    if _LIBHDF5_F64 is None and d is not None:
        b = open(os.path.join(d, "testhdf5_7.4_GLNX86.mat"), "rb").read()[512:]
        _, root, *_ = struct.unpack_from("<QQIIQQ", b, 56)
        st = [m for m in _v1_messages(b, root) if m[0] == 0x11][0][2]
        bt, heap = struct.unpack_from("<QQ", st)
        snod = struct.unpack_from("<Q", b, bt + 32)[0]
        oh = struct.unpack_from("<Q", b, snod + 16)[0]
        ver, _, n, _, size = struct.unpack_from("<BBHII", b, oh)
        p = oh + 16
        while p < oh + 16 + size:
            t, ln = struct.unpack_from("<HH", b, p)
            if t == 3:
                _LIBHDF5_F64 = b[p + 8:p + 8 + ln]
            p += 8 + ln
    return _LIBHDF5_F64


def _check_dataset(b, oh, eof):
    msgs = {t: (fl, d) for t, fl, d in _v1_messages(b, oh)}
    assert set(msgs) == {0x01, 0x03, 0x05, 0x08}
    sp = msgs[0x01][1]
    assert sp[0] == 1 and sp[1] == 1 and sp[2] == 1
    n, nmax = struct.unpack_from("<QQ", sp, 8)
    assert n == nmax
    dt = msgs[0x03][1]
    size = struct.unpack_from("<I", dt, 4)[0]
    if dt[0] == 0x11 and size == 8:
        ref = _libhdf5_f64_message()
        if ref is not None:
            assert dt == ref
    fill = msgs[0x05][1]
    assert fill[:4] == bytes([2, 2, 2, 1]) and struct.unpack_from("<I", fill, 4)[0] == 0
    ly = msgs[0x08][1]
    assert ly[0] == 3 and ly[1] == 1
    addr, nbytes = struct.unpack_from("<QQ", ly, 2)
    assert nbytes == n * size
    if n:
        assert addr % 16 == 0 and addr + nbytes <= eof
    else:
        assert addr == 2 ** 64 - 1


# ----------------------------------------------------------------- a version-2 file

def _v2_file(datasets, group=None):
    """Superblock v2, root object header v2 whose link messages sit half in the first
    chunk and half in a continuation block, dataset headers v2 with dataspace v2,
    layout v4.  ``datasets``: name -> array, or name -> (array, options) with options
    ``be`` (big-endian elements), ``shape`` (() for a scalar dataspace) and ``compact``
    (the elements inside the layout message).  ``group``: (name, datasets) of one
    subgroup linked from the root.  Checksums are left zero (the reader does not
    verify them)."""
    out = bytearray(48)                                          # superblock v2: 12 + 4 * 8 + 4

    def ohdr(msgs):
        body = b"".join(struct.pack("<BHB", t, len(d), 0) + d for t, d in msgs)
        return b"OHDR" + bytes([2, 0x02]) + struct.pack("<I", len(body)) + body + bytes(4)

    def link(name, addr):
        nm = name.encode()
        return bytes([1, 0]) + bytes([len(nm)]) + nm + struct.pack("<Q", addr)

    def put_dataset(a, be=False, shape=None, compact=False):
        a = np.asarray(a)
        raw = a.astype(a.dtype.newbyteorder(">" if be else "<")).tobytes()
        shape = a.shape if shape is None else shape
        if shape == ():
            space = bytes([2, 0, 0, 0])
        else:
            space = bytes([2, len(shape), 0, 1]) + b"".join(struct.pack("<Q", n) for n in shape)
        order = 1 if be else 0
        if a.dtype.kind == "f":
            if a.itemsize == 8:
                dt = bytes([0x11, 0x20 | order, 63, 0]) + struct.pack("<IHHBBBBI", 8, 0, 64, 52, 11, 0, 52, 1023)
            else:
                dt = bytes([0x11, 0x20 | order, 31, 0]) + struct.pack("<IHHBBBBI", 4, 0, 32, 23, 8, 0, 23, 127)
        else:
            sign = 0x08 if a.dtype.kind == "i" else 0
            dt = bytes([0x10, sign | order, 0, 0]) + struct.pack("<IHH", a.itemsize, 0, 8 * a.itemsize)
        if compact:
            layout = bytes([4, 0]) + struct.pack("<H", len(raw)) + raw
        else:
            out.extend(bytes((-len(out)) % 16))
            at = len(out)
            out.extend(raw)
            layout = bytes([4, 1]) + struct.pack("<QQ", at, len(raw))
        out.extend(bytes((-len(out)) % 8))
        addr = len(out)
        out.extend(ohdr([(0x01, space), (0x03, dt), (0x08, layout)]))
        return addr

    def put_all(ds):
        addrs = {}
        for k, v in ds.items():
            a, opt = v if isinstance(v, tuple) else (v, {})
            addrs[k] = put_dataset(a, **opt)
        return addrs

    headers = put_all(datasets)
    if group is not None:
        gname, gds = group
        ga = put_all(gds)
        linfo = bytes([0, 0]) + struct.pack("<QQ", 2 ** 64 - 1, 2 ** 64 - 1)
        out.extend(bytes((-len(out)) % 8))
        headers[gname] = len(out)
        out.extend(ohdr([(0x02, linfo)] + [(0x06, link(k, a)) for k, a in ga.items()]))
    keys = list(headers)
    cont_links = [(0x06, link(k, headers[k])) for k in keys[1:]]
    cont_body = b"".join(struct.pack("<BHB", t, len(d), 0) + d for t, d in cont_links)
    out.extend(bytes((-len(out)) % 8))
    cont_at = len(out)
    out.extend(b"OCHK" + cont_body + bytes(4))
    linfo = bytes([0, 0]) + struct.pack("<QQ", 2 ** 64 - 1, 2 ** 64 - 1)
    root_msgs = [(0x02, linfo), (0x06, link(keys[0], headers[keys[0]])),
                 (0x10, struct.pack("<QQ", cont_at, 8 + len(cont_body)))]
    out.extend(bytes((-len(out)) % 8))
    root_at = len(out)
    out.extend(ohdr(root_msgs))
    sb = b"\x89HDF\r\n\x1a\n" + bytes([2, 8, 8, 0]) + struct.pack("<QQQQ", 0, 2 ** 64 - 1, len(out), root_at)
    out[:48] = sb + bytes(4)
    return bytes(out)
