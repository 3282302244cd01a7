"""ctypes front end of the CPU oracle (oracle/xpcs_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
and by the CPU-baseline leg of ``bench.py`` -- never by the product.

Each wrapper returns numpy arrays in the reference's layouts:
  * G2/IP/IF            float32 [D][P]   (Corr::multiTau2, src/xpcs/corr.cpp:315)
  * g2/stderr           [D][nq]          (Corr::normalizeG2s, src/xpcs/corr.cpp:927)
  * event lists (rows)  CSR by pixel     (SparseData/Row, src/xpcs/data_structure)
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libxpcs_oracle.so"
REF_CORR = HERE / "_ref" / "corr"


def build(force: bool = False) -> Path:
    """Compile the oracle shared library (gcc, OpenMP, no FP contraction)."""
    src = HERE / "xpcs_oracle.c"
    if force or not LIB.exists() or LIB.stat().st_mtime < max(
        src.stat().st_mtime, (HERE / "xpcs_oracle.h").stat().st_mtime
    ):
        LIB.parent.mkdir(parents=True, exist_ok=True)
        subprocess.check_call(
            ["gcc", "-std=c11", "-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
             "-o", str(LIB), str(src), "-lm"]
        )
    return LIB


def reference_root() -> Path:
    """The upstream checkout the reference build reads: $XPCS_REFERENCE_SRC, or
    the default the build recipe (ref_build/Makefile) names."""
    env = os.environ.get("XPCS_REFERENCE_SRC")
    if env:
        return Path(env)
    out = subprocess.run(["make", "-s", "-C", str(HERE / "ref_build"), "print-ref"],
                         capture_output=True, text=True)
    return Path(out.stdout.strip()) if out.returncode == 0 and out.stdout.strip() else Path()


def build_reference(ref_root: str | None = None, jobs: int = 8) -> Path | None:
    """Build the upstream `corr` from its own sources into oracle/_ref, when
    the upstream checkout is present (None otherwise)."""
    root = Path(ref_root) if ref_root else reference_root()
    if not (root / "src" / "xpcs" / "corr.cpp").exists():
        return None
    subprocess.check_call(
        ["make", "-s", "-C", str(HERE / "ref_build"), f"REF={root}", f"-j{jobs}"]
    )
    return REF_CORR


class _QMap(C.Structure):
    _fields_ = [
        ("pixels", C.c_int32), ("total_static", C.c_int32), ("total_dynamic", C.c_int32),
        ("nq", C.c_int32), ("nsb", C.c_int32), ("npix", C.c_int32),
        ("valid", C.POINTER(C.c_int16)), ("sbin_mask", C.POINTER(C.c_int32)),
        ("pixels_per_bin", C.POINTER(C.c_int32)), ("q_ids", C.POINTER(C.c_int32)),
        ("q_sb_ptr", C.POINTER(C.c_int32)), ("sb_ids", C.POINTER(C.c_int32)),
        ("sb_pix_ptr", C.POINTER(C.c_int32)), ("pix", C.POINTER(C.c_int32)),
        ("error", C.c_int32),
    ]


class _FilterParams(C.Structure):
    _fields_ = [
        ("pixels", C.c_int32), ("frames", C.c_int32), ("real_frames", C.c_int32),
        ("stride", C.c_int32), ("average", C.c_int32), ("static_window", C.c_int32),
        ("total_static", C.c_int32), ("pixel_mask", C.POINTER(C.c_int16)),
        ("sbin_mask", C.POINTER(C.c_int32)), ("flatfield", C.POINTER(C.c_double)),
    ]


class _Rows(C.Structure):
    _fields_ = [
        ("pixels", C.c_int32), ("row_ptr", C.POINTER(C.c_int64)),
        ("frame", C.POINTER(C.c_int32)), ("value", C.POINTER(C.c_float)),
    ]


class _Side(C.Structure):
    _fields_ = [
        ("pixels_sum", C.POINTER(C.c_float)), ("frames_sum", C.POINTER(C.c_float)),
        ("partitions_mean", C.POINTER(C.c_float)), ("partial_mean", C.POINTER(C.c_float)),
        ("timestamp_clock", C.POINTER(C.c_double)), ("timestamp_ticks", C.POINTER(C.c_double)),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB))
        L.xo_level_max.restype = C.c_int
        L.xo_delays.restype = C.c_int
        L.xo_build_qmap.restype = C.c_int
        L.xo_sparse_filter.restype = C.c_int
        L.xo_dense_filter.restype = C.c_int
        L.xo_multitau2.restype = C.c_int
        L.xo_normalize_f32.restype = C.c_int
        L.xo_normalize_f64.restype = C.c_int
        _lib = L
    return _lib


def _p(a, ct):
    return a.ctypes.data_as(C.POINTER(ct))


def _copy(ptr, n, dtype):
    if n == 0:
        return np.zeros(0, dtype=dtype)
    return np.ctypeslib.as_array(ptr, shape=(n,)).astype(dtype, copy=True)


def delays(frames: int, dpl: int) -> tuple[np.ndarray, np.ndarray]:
    """(level, tau) of Corr::delaysPerLevel (src/xpcs/corr.cpp:1133)."""
    cap = 4096
    lv = np.zeros(cap, np.int32)
    tau = np.zeros(cap, np.int32)
    n = lib().xo_delays(frames, dpl, _p(lv, C.c_int32), _p(tau, C.c_int32), cap)
    return lv[:n].copy(), tau[:n].copy()


class QMap:
    """Configuration::BuildQMap restated (src/xpcs/configuration.cpp:244)."""

    def __init__(self, dqmap: np.ndarray, sqmap: np.ndarray):
        dq = np.ascontiguousarray(dqmap, np.int32).ravel()
        sq = np.ascontiguousarray(sqmap, np.int32).ravel()
        self._s = _QMap()
        lib().xo_build_qmap(_p(dq, C.c_int32), _p(sq, C.c_int32), dq.size, C.byref(self._s))
        s = self._s
        self.pixels = s.pixels
        self.total_static = s.total_static
        self.total_dynamic = s.total_dynamic
        self.nq = s.nq
        self.error = s.error
        self.valid = _copy(s.valid, s.pixels, np.int16)
        self.sbin_mask = _copy(s.sbin_mask, s.pixels, np.int32)
        self.pixels_per_bin = _copy(s.pixels_per_bin, s.total_static, np.int32)
        self.q_ids = _copy(s.q_ids, s.nq, np.int32)
        self.q_sb_ptr = _copy(s.q_sb_ptr, s.nq + 1, np.int32)
        self.sb_ids = _copy(s.sb_ids, s.nsb, np.int32)
        self.sb_pix_ptr = _copy(s.sb_pix_ptr, s.nsb + 1, np.int32)
        self.pix = _copy(s.pix, s.npix, np.int32)

    def __del__(self):
        try:
            lib().xo_free_qmap(C.byref(self._s))
        except Exception:
            pass


class Rows:
    """Pixel-major event lists (CSR)."""

    def __init__(self, row_ptr, frame, value):
        self.row_ptr = np.ascontiguousarray(row_ptr, np.int64)
        self.frame = np.ascontiguousarray(frame, np.int32)
        self.value = np.ascontiguousarray(value, np.float32)
        self.pixels = self.row_ptr.size - 1

    def _struct(self):
        r = _Rows()
        r.pixels = self.pixels
        r.row_ptr = _p(self.row_ptr, C.c_int64)
        r.frame = _p(self.frame, C.c_int32)
        r.value = _p(self.value, C.c_float)
        return r


def _filter_params(qm: QMap, frames, real_frames, stride, average, static_window, flat):
    fp = _FilterParams()
    fp.pixels = qm.pixels
    fp.frames = frames
    fp.real_frames = real_frames
    fp.stride = stride
    fp.average = average
    fp.static_window = static_window
    fp.total_static = qm.total_static
    fp.pixel_mask = _p(qm.valid, C.c_int16)
    fp.sbin_mask = _p(qm.sbin_mask, C.c_int32)
    fp.flatfield = _p(flat, C.c_double)
    return fp


def _collect(rows_s: _Rows, side_s: _Side, fp: _FilterParams, qm: QMap, finish: bool):
    P = rows_s.pixels
    rp = _copy(rows_s.row_ptr, P + 1, np.int64)
    E = int(rp[-1])
    rows = Rows(rp, _copy(rows_s.frame, E, np.int32), _copy(rows_s.value, E, np.float32))
    if finish:
        lib().xo_finish_side(C.byref(fp), _p(qm.pixels_per_bin, C.c_int32), C.byref(side_s))
    F, S, R = fp.frames, fp.total_static, fp.real_frames
    nparts = -(-F // fp.static_window)
    side = {
        "pixels_sum": _copy(side_s.pixels_sum, P, np.float32),
        "frames_sum": _copy(side_s.frames_sum, 2 * F, np.float32).reshape(2, F),
        "partitions_mean": _copy(side_s.partitions_mean, S, np.float32),
        "partial_mean": _copy(side_s.partial_mean, nparts * S, np.float32).reshape(nparts, S),
        "timestamp_clock": _copy(side_s.timestamp_clock, 2 * R, np.float64).reshape(2, R),
        "timestamp_tick": _copy(side_s.timestamp_ticks, 2 * R, np.float64).reshape(2, R),
    }
    lib().xo_free_rows(C.byref(rows_s))
    lib().xo_free_side(C.byref(side_s))
    return rows, side


def sparse_filter(qm: QMap, nnz, idx, val, frames, real_frames=None, stride=1, average=1,
                  static_window=None, flat=None, clock=None, ticks=None, finish=True):
    """SparseFilter::Apply over a series (src/xpcs/filter/sparse_filter.cpp:115)."""
    nnz = np.ascontiguousarray(nnz, np.uint32)
    idx = np.ascontiguousarray(idx, np.int32)
    val = np.ascontiguousarray(val, np.int16)
    real_frames = real_frames if real_frames is not None else nnz.size
    static_window = static_window or max(frames // 10, 1)
    flat = np.ascontiguousarray(flat if flat is not None else np.ones(qm.pixels), np.float64)
    fp = _filter_params(qm, frames, real_frames, stride, average, static_window, flat)
    rows_s, side_s = _Rows(), _Side()
    ck = np.ascontiguousarray(clock, np.float64) if clock is not None else None
    tk = np.ascontiguousarray(ticks, np.float64) if ticks is not None else None
    bad = lib().xo_sparse_filter(
        C.byref(fp), _p(idx, C.c_int32), _p(val, C.c_int16), _p(nnz, C.c_uint32),
        _p(ck, C.c_double) if ck is not None else None,
        _p(tk, C.c_double) if tk is not None else None, C.byref(rows_s), C.byref(side_s))
    rows, side = _collect(rows_s, side_s, fp, qm, finish)
    side["bad_index"] = bool(bad)
    return rows, side


def dark_image(dark: np.ndarray, flat: np.ndarray):
    """DarkImage::Compute (src/xpcs/data_structure/dark_image.cpp:81)."""
    dark = np.ascontiguousarray(dark, np.int16)
    nd, P = dark.shape
    flat = np.ascontiguousarray(flat, np.float64)
    avg = np.zeros(P, np.float64)
    std = np.zeros(P, np.float64)
    lib().xo_dark_image(_p(dark, C.c_int16), nd, P, _p(flat, C.c_double),
                        _p(avg, C.c_double), _p(std, C.c_double))
    return avg, std


def dense_filter(qm: QMap, raw, frames, dark_avg=None, dark_std=None, lld=0.0, sigma=0.0,
                 real_frames=None, stride=1, average=1, static_window=None, flat=None,
                 clock=None, ticks=None, finish=True):
    """DenseFilter::Apply over a series (src/xpcs/filter/dense_filter.cpp:121)."""
    raw = np.ascontiguousarray(raw, np.int16)
    real_frames = real_frames if real_frames is not None else raw.shape[0]
    static_window = static_window or max(frames // 10, 1)
    flat = np.ascontiguousarray(flat if flat is not None else np.ones(qm.pixels), np.float64)
    fp = _filter_params(qm, frames, real_frames, stride, average, static_window, flat)
    rows_s, side_s = _Rows(), _Side()
    da = np.ascontiguousarray(dark_avg, np.float64) if dark_avg is not None else None
    ds = np.ascontiguousarray(dark_std, np.float64) if dark_std is not None else None
    ck = np.ascontiguousarray(clock, np.float64) if clock is not None else None
    tk = np.ascontiguousarray(ticks, np.float64) if ticks is not None else None
    lib().xo_dense_filter(
        C.byref(fp), _p(raw, C.c_int16),
        _p(da, C.c_double) if da is not None else None,
        _p(ds, C.c_double) if ds is not None else None,
        C.c_float(lld), C.c_float(sigma), _p(ck, C.c_double) if ck is not None else None,
        _p(tk, C.c_double) if tk is not None else None, C.byref(rows_s), C.byref(side_s))
    return _collect(rows_s, side_s, fp, qm, finish)


def framesum_normalize(rows: Rows, frames_sum, frames: int) -> Rows:
    """The normalize_by_framesum pre-pass (src/xpcs/main.cpp:314-337): every
    value divided by (frameSum[F+f] / mean), mean = the float sum of
    frameSum[F..2F) in frame order divided by the frame count; all float32."""
    fs = np.ascontiguousarray(frames_sum, np.float32).ravel()[frames:2 * frames]
    acc = np.float32(0.0)
    for x in fs:
        acc = np.float32(acc + x)
    mean = np.float32(acc / np.float32(frames))
    q = (fs / mean).astype(np.float32)
    value = (rows.value / q[rows.frame]).astype(np.float32)
    return Rows(rows.row_ptr, rows.frame, value)


def _seq_sum_f32(x) -> np.float32:
    """Left-to-right float32 sum (the reference's `acc += x` loops)."""
    x = np.ascontiguousarray(x, np.float32)
    return np.add.accumulate(x)[-1] if x.size else np.float32(0.0)


def twotime(qm: QMap, rows: Rows, frames: int, qlist, static_map: bool, average: bool,
            wsize: int, sort_pixels: bool = False):
    """Corr::twotime (src/xpcs/corr.cpp:433-924, 1166-1305), float32 throughout
    in the reference's operation order.

    Smoothing (SmoothingStaticMap / SmoothingSymmetric, :433-547): sg per
    static bin of the processed q bins (static map) or per processed q bin
    (symmetric), per frame: the float sum over the bin's pixels in mapping
    order of the value at that frame, divided by the pixel count; with the
    average filter sg is then the float mean over frames.  Every value of a
    pixel of a processed q bin is divided by its sg.
    Per processed q bin (twotimeQBinThreading, :781-924): for every pixel in
    mapping order (ascending pixel index with frame threading, :573-779), for
    every pair of its events j <= k, C[f_j][f_k] += v_j * v_k; then C /= the
    pixel count.  g2full[ff] = mean of diagonal ff (float sum in order),
    g2partials[ff][w] = the diagonal's sum over window w of `wsize` entries
    divided by wsize (ff < wsize, w < (frames - wsize) / wsize).
    Returns dict(sg, c2t {q: F x F}, g2full [F][Q'], g2partials [wsize][TP][Q'])."""
    F = frames
    qset = set(int(q) for q in qlist)
    value = rows.value.copy()
    bins = []  # (q, [pixel lists of the bins]) for static map; (q, [plist]) for symmetric
    for i, q in enumerate(qm.q_ids):
        if int(q) not in qset:
            continue
        lists = [qm.pix[qm.sb_pix_ptr[k]:qm.sb_pix_ptr[k + 1]]
                 for k in range(qm.q_sb_ptr[i], qm.q_sb_ptr[i + 1])]
        bins.append((int(q), lists))
    groups = ([l for _, lists in bins for l in lists] if static_map
              else [np.concatenate(lists) for _, lists in bins])
    sg = np.zeros((len(groups), F), np.float32)
    for g, pl in enumerate(groups):
        for p in pl:
            a, b = rows.row_ptr[p], rows.row_ptr[p + 1]
            sg[g, rows.frame[a:b]] = (sg[g, rows.frame[a:b]] + value[a:b]).astype(np.float32)
        sg[g] = (sg[g] / np.float32(len(pl))).astype(np.float32)
    if average:
        sg = np.array([[_seq_sum_f32(sg[g]) / np.float32(F)] for g in range(len(groups))],
                      np.float32)
    for g, pl in enumerate(groups):
        for p in pl:
            a, b = rows.row_ptr[p], rows.row_ptr[p + 1]
            den = sg[g, 0] if average else sg[g, rows.frame[a:b]]
            value[a:b] = (value[a:b] / den).astype(np.float32)
    tp = (F - wsize) // wsize
    c2t, full, part = {}, [], []
    for q, lists in bins:
        plist = np.concatenate(lists)
        if sort_pixels:
            plist = np.sort(plist)
        C = np.zeros((F, F), np.float32)
        for p in plist:
            a, b = rows.row_ptr[p], rows.row_ptr[p + 1]
            t, v = rows.frame[a:b], value[a:b]
            j, k = np.triu_indices(t.size)
            C[t[j], t[k]] = (C[t[j], t[k]] + (v[j] * v[k]).astype(np.float32)).astype(np.float32)
        C = (C / np.float32(plist.size)).astype(np.float32)
        c2t[q] = C
        g2f = np.zeros(F, np.float32)
        g2p = np.zeros((wsize, max(tp, 0)), np.float32)
        for ff in range(F):
            diag = np.diagonal(C, ff).astype(np.float32)
            g2f[ff] = _seq_sum_f32(diag) / np.float32(diag.size)
            if ff < wsize:
                for w in range(tp):
                    seg = diag[w * wsize:(w + 1) * wsize]
                    g2p[ff, w] = _seq_sum_f32(seg) / np.float32(wsize)
        full.append(g2f)
        part.append(g2p)
    return dict(sg=sg, c2t=c2t, g2full=np.stack(full, 1) if full else np.zeros((F, 0), np.float32),
                g2partials=np.stack(part, 2) if part else np.zeros((wsize, tp, 0), np.float32))


def multitau2(rows: Rows, frames: int, dpl: int, mode: int = 0, threads: int = 0):
    """Corr::multiTau2 (src/xpcs/corr.cpp:315). mode 0 = reference, 1 = exact."""
    lv, _ = delays(frames, dpl)
    D, P = lv.size, rows.pixels
    G2 = np.zeros((D, P), np.float32)
    IP = np.zeros((D, P), np.float32)
    IF = np.zeros((D, P), np.float32)
    rs = rows._struct()
    lib().xo_multitau2(C.byref(rs), frames, dpl, mode, threads, _p(G2, C.c_float),
                       _p(IP, C.c_float), _p(IF, C.c_float))
    return G2, IP, IF


def normalize_f32(qm: QMap, G2, IP, IF):
    """Corr::normalizeG2s in float32 (src/xpcs/corr.cpp:927)."""
    D = G2.shape[0]
    g2 = np.zeros((D, qm.nq), np.float32)
    se = np.zeros((D, qm.nq), np.float32)
    args = [np.ascontiguousarray(a, np.float32) for a in (G2, IP, IF)]
    lib().xo_normalize_f32(C.byref(qm._s), D, *[_p(a, C.c_float) for a in args],
                           _p(g2, C.c_float), _p(se, C.c_float))
    return g2, se


def normalize_f64(qm: QMap, G2, IP, IF):
    """Corr::normalizeG2s formulas in double precision."""
    D = G2.shape[0]
    g2 = np.zeros((D, qm.nq), np.float64)
    se = np.zeros((D, qm.nq), np.float64)
    args = [np.ascontiguousarray(a, np.float32) for a in (G2, IP, IF)]
    lib().xo_normalize_f64(C.byref(qm._s), D, *[_p(a, C.c_float) for a in args],
                           _p(g2, C.c_double), _p(se, C.c_double))
    return g2, se


def cpu_count() -> int:
    return len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()
