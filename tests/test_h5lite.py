"""The HDF5 subset of the analysis file (host/h5lite.*), on the CPU.

* Reading is pinned on a file written by the HDF5 library itself: scipy's
  MATLAB 7.3 test file (HDF5 behind a 512-byte user block, a version 0
  superblock, a symbol-table root group, a version 2 layout message), whose
  variable `testdouble` scipy's own tests define as pi/4 * [0 .. 8].
* Files made or changed by the writer are read back both through the
  library (`h5lite_tool dump`) and through tests/h5walk.py, an independent
  walk of the format that also checks the structural rules (B-tree keys,
  sorted nodes, heap free lists, cached addresses, end-of-file address).
"""
import os
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

import h5walk
import refio

SCIPY_MAT73 = "io/matlab/tests/data/testhdf5_7.4_GLNX86.mat"


@pytest.fixture(scope="module")
def tool():
    from build import build_h5tool
    return str(build_h5tool())


def run(tool, *args, ok=True):
    r = subprocess.run([tool, *map(str, args)], capture_output=True, text=True, timeout=120)
    if ok:
        assert r.returncode == 0, r.stderr
    return r


def dump(tool, path):
    """{path: (kind+size, dims, values)} from the library's reader."""
    out = {}
    for line in run(tool, "dump", path).stdout.splitlines():
        if line.startswith("skip "):
            continue
        parts = line.split(" ", 3)
        out[parts[0]] = (parts[1], parts[2], parts[3] if len(parts) > 3 else "")
    return out


def mat73():
    scipy = pytest.importorskip("scipy")
    p = Path(scipy.__file__).parent / SCIPY_MAT73
    if not p.exists():
        pytest.skip("scipy's MATLAB 7.3 test file is not installed")
    return p


def test_reads_a_file_written_by_the_hdf5_library(tool):
    path = mat73()
    want = np.pi / 4 * np.arange(9, dtype=float)
    d = dump(tool, path)
    kind, dims, vals = d["/testdouble"]
    assert kind == "float8" and dims == "9,1"
    got = np.array([float(v) for v in vals.split()])
    assert np.array_equal(got, want)
    w = h5walk.read(path)
    assert np.array_equal(w["/testdouble"].ravel(), want)


VALUES = {
    "/a/i8": ("i8", "4", [-128, -1, 0, 127]),
    "/a/u8": ("u8", "3", [0, 1, 255]),
    "/a/i16": ("i16", "2,2", [-32768, 7, 8, 32767]),
    "/a/u16": ("u16", "scalar", [65535]),
    "/a/i32": ("i32", "2,3", [1, -2, 3, -4, 5, -6]),
    "/a/u32": ("u32", "1", [4294967295]),
    "/a/i64": ("i64", "2", [-(1 << 62), (1 << 62)]),
    "/b/c/d/f32": ("f32", "3", [1.5, -0.25, 3.0e38]),
    "/b/c/d/f64": ("f64", "2,1,2", [1e-300, -2.5, 3.141592653589793, 0.0]),
    "/b/s": ("str", "scalar", ["/exchange"]),
    "/top": ("f64", "scalar", [42.0]),
}


def _np(kind, vals):
    dt = {"i8": np.int8, "u8": np.uint8, "i16": np.int16, "u16": np.uint16, "i32": np.int32,
          "u32": np.uint32, "i64": np.int64, "f32": np.float32, "f64": np.float64}[kind]
    return np.array(vals, dtype=dt)


def test_written_datasets_read_back_through_both_readers(tool, tmp_path):
    f = tmp_path / "new.h5"
    run(tool, "create", f)
    for path, (kind, dims, vals) in VALUES.items():
        run(tool, "put", f, path, kind, dims, *vals)
    w = h5walk.read(f)
    d = dump(tool, f)
    assert set(w) == set(VALUES) == set(d)
    for path, (kind, dims, vals) in VALUES.items():
        if kind == "str":
            assert w[path] == vals[0] and d[path][2] == f'"{vals[0]}"'
            continue
        want = _np(kind, vals)
        shape = () if dims == "scalar" else tuple(int(x) for x in dims.split(","))
        assert w[path].shape == shape and w[path].dtype == want.dtype
        assert np.array_equal(w[path].ravel(), want), path
        got = np.array([float(v) for v in d[path][2].split()])
        assert np.array_equal(got, want.astype(np.float64)), path


def test_group_with_hundreds_of_links(tool, tmp_path):
    """More links than one B-tree node of symbol-table nodes holds (2K x 2K'
    = 8 x 32 = 256 by default): a second B-tree level."""
    f = tmp_path / "many.h5"
    run(tool, "create", f)
    names = [f"q{i:03d}" for i in range(300)]
    rng = np.random.default_rng(1)
    for n in rng.permutation(names):  # out of order: the nodes must come out sorted
        run(tool, "put", f, f"/exchange/{n}", "i32", "1", int(n[1:]))
    w = h5walk.read(f)
    assert sorted(w) == [f"/exchange/{n}" for n in names]
    for n in names:
        assert int(w[f"/exchange/{n}"][0]) == int(n[1:])


def test_overwrite_in_place_and_refuse_another_shape(tool, tmp_path):
    f = tmp_path / "ow.h5"
    run(tool, "create", f)
    run(tool, "put", f, "/exchange/norm-0-g2", "f32", "2,2", 1, 2, 3, 4)
    size = f.stat().st_size
    run(tool, "put", f, "/exchange/norm-0-g2", "f32", "2,2", 5, 6, 7, 8)
    assert f.stat().st_size == size  # the same storage, written again
    assert np.array_equal(h5walk.read(f)["/exchange/norm-0-g2"], [[5, 6], [7, 8]])
    r = run(tool, "put", f, "/exchange/norm-0-g2", "f32", "3", 1, 2, 3, ok=False)
    assert r.returncode != 0 and "another type or shape" in r.stderr
    r = run(tool, "put", f, "/exchange/norm-0-g2", "f64", "2,2", 1, 2, 3, 4, ok=False)
    assert r.returncode != 0


def test_writes_into_a_library_file_behind_a_user_block(tool, tmp_path):
    """New group and datasets appended to the library-written file: its user
    block and its own dataset are untouched, and both readers see all three."""
    src = mat73()
    f = tmp_path / "m.h5"
    shutil.copy(src, f)
    head = f.read_bytes()[:512]
    run(tool, "put", f, "/exchange/tau", "f32", "1,3", 1, 2, 4)
    run(tool, "put", f, "/exchange/norm-0-g2", "f64", "2", 0.5, 1.5)
    assert f.read_bytes()[:512] == head
    w = h5walk.read(f)
    assert np.array_equal(w["/testdouble"].ravel(), np.pi / 4 * np.arange(9))
    assert np.array_equal(w["/exchange/tau"], [[1, 2, 4]])
    assert np.array_equal(w["/exchange/norm-0-g2"], [0.5, 1.5])
    d = dump(tool, f)
    assert set(d) == {"/testdouble", "/exchange/tau", "/exchange/norm-0-g2"}


def test_xh5c_container_converts_to_hdf5(tool, tmp_path):
    cfg = {"/xpcs/dqmap": np.arange(12, dtype=np.int32).reshape(3, 4),
           "/xpcs/output_data": "/exchange",
           "/xpcs/lld": np.array([1.25], np.float32),
           "/measurement/instrument/detector/flatfield": np.linspace(0.9, 1.1, 12).reshape(3, 4),
           "/xpcs/stride_frames": np.array([2], np.int64)}
    src, dst = tmp_path / "a.xh5c", tmp_path / "a.h5"
    refio.write_xh5c(src, cfg)
    run(tool, "from-xh5c", src, dst)
    w = h5walk.read(dst)
    assert set(w) == set(cfg)
    for k, v in cfg.items():
        if isinstance(v, str):
            assert w[k] == v
        else:
            assert w[k].dtype == v.dtype and np.array_equal(w[k], v), k


def test_not_hdf5_and_truncated_files_are_errors(tool, tmp_path):
    f = tmp_path / "t.h5"
    run(tool, "create", f)
    run(tool, "put", f, "/x/y", "i32", "4", 1, 2, 3, 4)
    b = f.read_bytes()
    cut = tmp_path / "cut.h5"
    cut.write_bytes(b[: len(b) // 2])
    r = run(tool, "dump", cut, ok=False)
    assert r.returncode != 0 and "HDF5" in r.stderr
    junk = tmp_path / "junk.h5"
    junk.write_bytes(os.urandom(4096))
    assert run(tool, "dump", junk, ok=False).returncode != 0


def _vlstr_file(path, name: str, text: str):
    """A file built byte by byte from the format specification: version 0
    superblock, a root symbol-table group with one link, and a scalar
    variable-length string dataset whose characters live in a global heap
    collection (the way h5py stores Python strings)."""
    import struct

    def pad8(b):
        return b + b"\0" * (-len(b) % 8)

    def v1_header(msgs):
        body = b"".join(struct.pack("<HHB3x", t, len(pad8(d)), 0) + pad8(d) for t, d in msgs)
        return struct.pack("<BBHII4x", 1, 0, len(msgs), 1, len(body)) + body

    U = 0xFFFFFFFFFFFFFFFF
    out = bytearray(96)  # the superblock, filled in last
    def put(b):
        while len(out) % 8:
            out.append(0)
        a = len(out)
        out.extend(b)
        return a
    tb = text.encode()
    gcol = b"GCOL" + bytes([1, 0, 0, 0])
    obj = struct.pack("<HH4xQ", 1, 0, len(tb)) + pad8(tb)
    free = 4096 - 16 - len(obj)
    gcol += struct.pack("<Q", 4096) + obj + struct.pack("<HH4xQ", 0, 0, free - 16) + b"\0" * (free - 16)
    g = put(gcol)
    elem = put(struct.pack("<IQI", len(tb), g, 1))
    char = bytes([0x10, 0, 0, 0]) + struct.pack("<IHH", 1, 0, 8)
    vl = bytes([0x19, 0x01, 0, 0]) + struct.pack("<I", 16) + char
    space = bytes([1, 0, 0, 0, 0, 0, 0, 0])
    layout = bytes([3, 1]) + struct.pack("<QQ", elem, 16)
    ds = put(v1_header([(0x01, space), (0x03, vl), (0x08, layout)]))
    nm = pad8(name.encode() + b"\0")
    seg = b"\0" * 8 + nm + struct.pack("<QQ", 1, 16)
    seg_a = put(seg)
    heap = put(b"HEAP" + b"\0" * 4 + struct.pack("<QQQ", len(seg), 8 + len(nm), seg_a))
    snod = put((b"SNOD" + bytes([1, 0]) + struct.pack("<H", 1)
                + struct.pack("<QQI4x16x", 8, ds, 0)).ljust(8 + 8 * 40, b"\0"))
    tree = put((b"TREE" + bytes([0, 0]) + struct.pack("<HQQ", 1, U, U)
                + struct.pack("<QQQ", 0, snod, 8)).ljust(24 + 33 * 8 + 32 * 8, b"\0"))
    root = put(v1_header([(0x11, struct.pack("<QQ", tree, heap))]))
    sb = (b"\x89HDF\r\n\x1a\n" + bytes([0, 0, 0, 0, 0, 8, 8, 0]) + struct.pack("<HHI", 4, 16, 0)
          + struct.pack("<QQQQ", 0, U, len(out), U)
          + struct.pack("<QQI4xQQ", 0, root, 1, tree, heap))
    out[:96] = sb
    Path(path).write_bytes(bytes(out))


def test_variable_length_string_from_a_global_heap(tool, tmp_path):
    f = tmp_path / "vl.h5"
    _vlstr_file(f, "output_data", "/exchange_run7")
    d = dump(tool, f)
    assert d["/output_data"][0].startswith("str") and d["/output_data"][2] == '"/exchange_run7"'
    # the writer appends next to it and the string survives
    run(tool, "put", f, "/exchange/tau", "f32", "2", 1, 2)
    d = dump(tool, f)
    assert d["/output_data"][2] == '"/exchange_run7"' and d["/exchange/tau"][2] == "1 2"


def test_corrupted_files_end_in_an_error_not_a_crash(tool, tmp_path):
    """Bytes flipped at random across a written file (and the library-written
    one): every dump must finish by itself with status 0 or 1, never a signal
    or a hang, since every read is bounds-checked and every walk bounded."""
    f = tmp_path / "base.h5"
    run(tool, "create", f)
    for path, (kind, dims, vals) in VALUES.items():
        run(tool, "put", f, path, kind, dims, *vals)
    bases = [f.read_bytes()]
    scipy = pytest.importorskip("scipy")
    lib = Path(scipy.__file__).parent / SCIPY_MAT73
    if lib.exists():
        bases.append(lib.read_bytes())
    rng = np.random.default_rng(7)
    bad = tmp_path / "bad.h5"
    for base in bases:
        for trial in range(150):
            b = bytearray(base)
            for _ in range(int(rng.integers(1, 6))):
                i = int(rng.integers(0, len(b)))
                b[i] = int(rng.integers(0, 256))
            if trial % 10 == 0:
                b = b[: int(rng.integers(8, len(b)))]
            bad.write_bytes(bytes(b))
            r = subprocess.run([tool, "dump", str(bad)], capture_output=True, timeout=30)
            assert r.returncode in (0, 1), (trial, r.returncode,
                                            r.stderr[-200:].decode(errors="replace"))
