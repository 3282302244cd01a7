"""Python front end of libxpcs_gpu through its C ABI (include/xpcs_gpu.h).

This is a thin ctypes binding: every call goes to the CUDA library, and the
import fails loudly when the library cannot be loaded -- there is no CPU
fallback.  The structure mirrors the reference's `corr` flow:

    s = Series(width, height, frames, dpl, dqmap, sqmap, ...)  # Configuration::init
    s.ingest_sparse(nnz, idx, val)                             # Imm + SparseFilter
    s.multitau(MODE_REFERENCE)                                 # Corr::multiTau2
    G2, IP, IF = s.g2ipif()                                    # --g2out datasets
    g2, se, g2f, sef = s.normalize()                           # Corr::normalizeG2s
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libxpcs_gpu.so"

MODE_REFERENCE = 0
MODE_EXACT = 1

STATUS = {0: "OK", 1: "INVALID_ARGUMENT", 2: "CUDA", 3: "OUT_OF_MEMORY", 4: "STATE", 5: "QMAP",
          6: "INPUT", 7: "NO_DEVICE"}

# Exported symbols of include/xpcs_gpu.h (checked by the CPU test suite).
EXPORTS = [
    "xpcs_abi_version", "xpcs_last_error", "xpcs_delay_schedule", "xpcs_series_create",
    "xpcs_series_destroy", "xpcs_series_reset", "xpcs_series_get_info", "xpcs_ingest_sparse",
    "xpcs_ingest_sparse_device", "xpcs_multitau", "xpcs_get_g2ipif", "xpcs_normalize",
    "xpcs_synchronize", "xpcs_get_stage_times", "xpcs_multitau2", "xpcs_pin_host",
    "xpcs_unpin_host", "xpcs_multitau2_noalloc", "xpcs_set_dark", "xpcs_ingest_dense",
    "xpcs_ingest_dense_device", "xpcs_get_dark", "xpcs_side_stats", "xpcs_get_normalized",
    "xpcs_batch_create", "xpcs_batch_run", "xpcs_batch_stats", "xpcs_batch_destroy",
    "xpcs_autotune", "xpcs_server_create", "xpcs_server_destroy", "xpcs_server_submit",
    "xpcs_server_push_sparse", "xpcs_server_finish", "xpcs_server_state", "xpcs_server_result",
    "xpcs_server_release", "xpcs_server_get_stats", "xpcs_twotime", "xpcs_get_twotime",
    "xpcs_set_device_memory_limit", "xpcs_get_device_memory", "xpcs_series_set_block_frames",
    "xpcs_batch_timeline", "xpcs_series_get_tuning", "xpcs_series_set_tuning",
    "xpcs_batch_set_form", "xpcs_batch_get_form", "xpcs_device_properties",
]

BATCH_F64 = 1
BATCH_F32 = 2
BATCH_AUTOTUNE = 4
TWOTIME_EXACT_CUDA_CORES = 2

NOALLOC_MAX_EVENTS = 4194304
NOALLOC_MAX_DELAYS = 512


class TwoTimeDesc(C.Structure):
    _fields_ = [("qbins", C.POINTER(C.c_int32)), ("nqbins", C.c_int32),
                ("static_map", C.c_int32), ("average", C.c_int32), ("window", C.c_int32),
                ("frame_threading", C.c_int32)]


class TwoTimeInfo(C.Structure):
    _fields_ = [("qbins", C.c_int32), ("frames", C.c_int32), ("window", C.c_int32),
                ("partials", C.c_int32), ("sg_rows", C.c_int32), ("sg_cols", C.c_int32),
                ("gram_ms", C.c_float), ("gram_flop", C.c_double),
                ("gram_flop_algorithmic", C.c_double)]


class ServerStats(C.Structure):
    _fields_ = [
        ("frames_ingested", C.c_int64), ("series_finished", C.c_int64),
        ("ingest_p50_ms", C.c_double), ("ingest_p99_ms", C.c_double),
        ("ingest_max_ms", C.c_double), ("final_p50_ms", C.c_double),
        ("final_p99_ms", C.c_double), ("active", C.c_int32), ("pending", C.c_int32),
        ("peak_active", C.c_int32), ("reserved", C.c_int32), ("used_bytes", C.c_uint64),
        ("peak_used_bytes", C.c_uint64),
    ]


ACQ_STATES = {0: "pending", 1: "active", 2: "finishing", 3: "done", 4: "failed"}


class XpcsError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"xpcs {STATUS.get(code, code)}: {msg}")
        self.code = code


class Tuning(C.Structure):
    _fields_ = [("thread_cap", C.c_int32), ("scratch_extra", C.c_int32),
                ("radix_items_per_lane", C.c_int32)]


class SeriesDesc(C.Structure):
    _fields_ = [
        ("width", C.c_int32), ("height", C.c_int32), ("frames", C.c_int32),
        ("delays_per_level", C.c_int32), ("stride_frames", C.c_int32), ("avg_frames", C.c_int32),
        ("static_window", C.c_int32), ("dqmap", C.POINTER(C.c_int32)),
        ("sqmap", C.POINTER(C.c_int32)), ("flatfield", C.POINTER(C.c_double)),
        ("dense", C.c_int32), ("lld", C.c_float), ("sigma", C.c_float), ("device", C.c_int32),
        ("normalize_by_framesum", C.c_int32),
    ]


class SeriesInfo(C.Structure):
    _fields_ = [
        ("pixels", C.c_int32), ("delays", C.c_int32), ("total_static", C.c_int32),
        ("total_dynamic", C.c_int32), ("qbins", C.c_int32), ("raw_frames", C.c_int32),
        ("raw_events", C.c_int64), ("events", C.c_int64), ("valid_pixels", C.c_int32),
        ("float_path_pixels", C.c_int32),
    ]


class StageTimes(C.Structure):
    _fields_ = [(n, C.c_float) for n in ("h2d_ms", "filter_ms", "multitau_ms", "normalize_ms",
                                         "d2h_ms", "multitau_int_ms", "multitau_float_ms",
                                         "step_ms")] + [("launches", C.c_int32)]


_lib = None


def lib() -> C.CDLL:
    """Load libxpcs_gpu.so (building it first if it is missing)."""
    global _lib
    if _lib is None:
        if not LIB.exists():
            import sys
            sys.path.insert(0, str(HERE))
            from build import build_gpu
            build_gpu()
        L = C.CDLL(str(LIB))
        L.xpcs_last_error.restype = C.c_char_p
        L.xpcs_series_create.argtypes = [C.POINTER(SeriesDesc), C.POINTER(C.c_void_p)]
        L.xpcs_series_destroy.argtypes = [C.c_void_p]
        for name in ("xpcs_series_reset", "xpcs_synchronize"):
            getattr(L, name).argtypes = [C.c_void_p]
        L.xpcs_series_get_info.argtypes = [C.c_void_p, C.POINTER(SeriesInfo)]
        L.xpcs_get_stage_times.argtypes = [C.c_void_p, C.POINTER(StageTimes)]
        L.xpcs_ingest_sparse.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32]
        L.xpcs_ingest_sparse_device.argtypes = L.xpcs_ingest_sparse.argtypes
        L.xpcs_multitau.argtypes = [C.c_void_p, C.c_int32]
        L.xpcs_set_dark.argtypes = [C.c_void_p, C.c_void_p, C.c_int32]
        L.xpcs_ingest_dense.argtypes = [C.c_void_p, C.c_void_p, C.c_int32]
        L.xpcs_ingest_dense_device.argtypes = [C.c_void_p, C.c_void_p, C.c_int32]
        L.xpcs_get_dark.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.xpcs_side_stats.argtypes = [C.c_void_p] + [C.c_void_p] * 4
        L.xpcs_get_g2ipif.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.xpcs_normalize.argtypes = [C.c_void_p] + [C.c_void_p] * 4
        L.xpcs_get_normalized.argtypes = [C.c_void_p] + [C.c_void_p] * 4
        L.xpcs_batch_create.argtypes = [C.c_void_p, C.c_int32, C.POINTER(C.c_void_p)]
        L.xpcs_batch_run.argtypes = [C.c_void_p, C.c_int32, C.c_uint32]
        L.xpcs_batch_stats.argtypes = [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_int64),
                                       C.POINTER(C.c_int32)]
        L.xpcs_batch_destroy.argtypes = [C.c_void_p]
        L.xpcs_autotune.argtypes = [C.c_void_p, C.c_int32, C.POINTER(C.c_int32)]
        L.xpcs_server_create.argtypes = [C.c_int32, C.c_uint64, C.POINTER(C.c_void_p)]
        L.xpcs_server_destroy.argtypes = [C.c_void_p]
        L.xpcs_server_submit.argtypes = [C.c_void_p, C.POINTER(SeriesDesc), C.c_int64,
                                         C.POINTER(C.c_int64)]
        L.xpcs_server_push_sparse.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p,
                                              C.c_void_p, C.c_int32]
        L.xpcs_server_finish.argtypes = [C.c_void_p, C.c_int64, C.c_int32]
        L.xpcs_server_state.argtypes = [C.c_void_p, C.c_int64, C.POINTER(C.c_int32)]
        L.xpcs_server_result.argtypes = [C.c_void_p, C.c_int64] + [C.c_void_p] * 5
        L.xpcs_server_release.argtypes = [C.c_void_p, C.c_int64]
        L.xpcs_server_get_stats.argtypes = [C.c_void_p, C.POINTER(ServerStats)]
        L.xpcs_twotime.argtypes = [C.c_void_p, C.POINTER(TwoTimeDesc), C.c_int32,
                                   C.POINTER(TwoTimeInfo)]
        L.xpcs_get_twotime.argtypes = [C.c_void_p] + [C.c_void_p] * 5
        L.xpcs_multitau2_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32,
                                             C.c_int64, C.c_int32, C.c_int32, C.c_int32,
                                             C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.xpcs_set_device_memory_limit.argtypes = [C.c_int32, C.c_uint64]
        L.xpcs_series_set_block_frames.argtypes = [C.c_void_p, C.c_int32]
        L.xpcs_batch_timeline.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.xpcs_series_get_tuning.argtypes = [C.c_void_p, C.POINTER(Tuning)]
        L.xpcs_batch_set_form.argtypes = [C.c_void_p, C.c_int32]
        L.xpcs_device_properties.argtypes = [C.c_int32] + [C.POINTER(C.c_int32)] * 3
        L.xpcs_batch_get_form.argtypes = [C.c_void_p, C.POINTER(C.c_int32),
                                          C.POINTER(C.c_int32)]
        L.xpcs_series_set_tuning.argtypes = [C.c_void_p, C.POINTER(Tuning)]
        L.xpcs_get_device_memory.argtypes = [C.c_int32, C.POINTER(C.c_uint64),
                                             C.POINTER(C.c_uint64)]
        L.xpcs_pin_host.argtypes = [C.c_void_p, C.c_uint64]
        L.xpcs_unpin_host.argtypes = [C.c_void_p]
        L.xpcs_multitau2.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32,
                                     C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p,
                                     C.c_void_p]
        _lib = L
    return _lib


def check(rc: int):
    if rc != 0:
        raise XpcsError(rc, lib().xpcs_last_error().decode(errors="replace"))


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def delay_schedule(frames: int, dpl: int):
    cap = 4096
    lv = np.zeros(cap, np.int32)
    tau = np.zeros(cap, np.int32)
    n = C.c_int32(0)
    check(lib().xpcs_delay_schedule(frames, dpl, _ptr(lv), _ptr(tau), cap, C.byref(n)))
    return lv[:n.value].copy(), tau[:n.value].copy()


class Series:
    """One XPCS series on one GPU (an xpcs_series handle)."""

    def __init__(self, width, height, frames, dpl, dqmap, sqmap, flatfield=None, stride=1,
                 average=1, static_window=None, device=0, dense=False, lld=0.0, sigma=0.0,
                 normalize_by_framesum=False):
        self._dq = np.ascontiguousarray(dqmap, np.int32).ravel()
        self._sq = np.ascontiguousarray(sqmap, np.int32).ravel()
        self._flat = (None if flatfield is None
                      else np.ascontiguousarray(flatfield, np.float64).ravel())
        d = SeriesDesc()
        d.width, d.height, d.frames, d.delays_per_level = width, height, frames, dpl
        d.stride_frames, d.avg_frames = stride, average
        d.static_window = static_window or max(frames // 10, 1)
        d.dqmap = self._dq.ctypes.data_as(C.POINTER(C.c_int32))
        d.sqmap = self._sq.ctypes.data_as(C.POINTER(C.c_int32))
        d.flatfield = (self._flat.ctypes.data_as(C.POINTER(C.c_double))
                       if self._flat is not None else None)
        d.device = device
        d.dense, d.lld, d.sigma = int(dense), lld, sigma
        d.normalize_by_framesum = int(bool(normalize_by_framesum))
        self._h = C.c_void_p()
        check(lib().xpcs_series_create(C.byref(d), C.byref(self._h)))
        self.width, self.height, self.frames = width, height, frames
        self.info()

    def close(self):
        if getattr(self, "_h", None):
            lib().xpcs_series_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def info(self) -> SeriesInfo:
        i = SeriesInfo()
        check(lib().xpcs_series_get_info(self._h, C.byref(i)))
        self.P, self.D, self.nq = i.pixels, i.delays, i.qbins
        return i

    def reset(self):
        check(lib().xpcs_series_reset(self._h))

    def tuning(self) -> dict:
        """The series' kernel knobs (xpcs_series_get_tuning)."""
        t = Tuning()
        check(lib().xpcs_series_get_tuning(self._h, C.byref(t)))
        return {n: getattr(t, n) for n, _ in Tuning._fields_}

    def set_tuning(self, thread_cap=80, scratch_extra=0, radix_items_per_lane=0):
        t = Tuning(thread_cap, scratch_extra, radix_items_per_lane)
        check(lib().xpcs_series_set_tuning(self._h, C.byref(t)))

    def set_block_frames(self, block_frames: int):
        """Transpose frames in blocks of this many filter frames as they are
        ingested (xpcs_series_set_block_frames); 0 = all at multitau()."""
        check(lib().xpcs_series_set_block_frames(self._h, int(block_frames)))

    def ingest_sparse(self, nnz, idx, val):
        nnz = np.ascontiguousarray(nnz, np.uint32)
        idx = np.ascontiguousarray(idx, np.int32)
        val = np.ascontiguousarray(val, np.int16)
        check(lib().xpcs_ingest_sparse(self._h, _ptr(idx), _ptr(val), _ptr(nnz), nnz.size))

    def ingest_sparse_device(self, nnz, idx_dev_ptr: int, val_dev_ptr: int):
        nnz = np.ascontiguousarray(nnz, np.uint32)
        check(lib().xpcs_ingest_sparse_device(self._h, C.c_void_p(idx_dev_ptr),
                                              C.c_void_p(val_dev_ptr), _ptr(nnz), nnz.size))

    def set_dark(self, dark):
        dark = np.ascontiguousarray(dark, np.int16)
        n = dark.shape[0] if dark.ndim > 1 else (1 if dark.size else 0)
        check(lib().xpcs_set_dark(self._h, _ptr(dark), n))

    def ingest_dense(self, frames):
        frames = np.ascontiguousarray(frames, np.int16)
        n = frames.size // (self.width * self.height)
        check(lib().xpcs_ingest_dense(self._h, _ptr(frames), n))

    def ingest_dense_device(self, frames_dev_ptr: int, nframes: int):
        """Dense frames already on this series' device: int16 [nframes][P]."""
        check(lib().xpcs_ingest_dense_device(self._h, C.c_void_p(frames_dev_ptr), nframes))

    def dark(self):
        avg = np.empty(self.width * self.height, np.float64)
        std = np.empty_like(avg)
        check(lib().xpcs_get_dark(self._h, _ptr(avg), _ptr(std)))
        return avg, std

    def multitau(self, mode=MODE_REFERENCE):
        check(lib().xpcs_multitau(self._h, mode))

    def synchronize(self):
        check(lib().xpcs_synchronize(self._h))

    def g2ipif(self, out=None):
        if out is None:
            out = tuple(np.empty((self.D, self.P), np.float32) for _ in range(3))
        check(lib().xpcs_get_g2ipif(self._h, *[_ptr(a) for a in out]))
        return out

    def side_stats(self, static_window):
        """pixelSum [H][W], frameSum [2][F], partition-mean-total [1][S],
        partition-mean-partial [F // static_window][S] (float32)."""
        i = self.info()
        S = i.total_static
        nwin = self.frames // static_window
        ps = np.empty((self.height, self.width), np.float32)
        fs = np.empty((2, self.frames), np.float32)
        tot = np.empty((1, S), np.float32)
        part = np.empty((nwin, S), np.float32)
        check(lib().xpcs_side_stats(self._h, _ptr(ps), _ptr(fs), _ptr(tot), _ptr(part)))
        return ps, fs, tot, part

    def normalize(self, f64=True, f32=True, out=None):
        if out is None:
            shp = (self.D, self.nq)
            out = (np.empty(shp, np.float64) if f64 else None,
                   np.empty(shp, np.float64) if f64 else None,
                   np.empty(shp, np.float32) if f32 else None,
                   np.empty(shp, np.float32) if f32 else None)
        check(lib().xpcs_normalize(self._h, *[_ptr(a) for a in out]))
        return out

    def twotime(self, qbins, static_map=False, average=False, window=1, frame_threading=False,
                mode=MODE_REFERENCE, fetch=True) -> dict:
        """xpcs_twotime + xpcs_get_twotime: sg, C2T per q bin, g2full, g2partials
        (fetch=False: compute only, results stay on the device)."""
        q = np.ascontiguousarray(qbins, np.int32)
        d = TwoTimeDesc(q.ctypes.data_as(C.POINTER(C.c_int32)), q.size, int(static_map),
                        int(average), int(window), int(frame_threading))
        info = TwoTimeInfo()
        check(lib().xpcs_twotime(self._h, C.byref(d), mode, C.byref(info)))
        if not fetch:
            return dict(gram_ms=info.gram_ms, gram_flop=info.gram_flop,
                        gram_flop_algorithmic=info.gram_flop_algorithmic, qbins=info.qbins,
                        frames=info.frames)
        Q, F = info.qbins, info.frames
        qs = np.empty(Q, np.int32)
        sg = np.empty((info.sg_rows, info.sg_cols), np.float32)
        c2t = np.empty((Q, F, F), np.float32)
        full = np.empty((F, Q), np.float32)
        part = np.empty((info.window, info.partials, Q), np.float32)
        check(lib().xpcs_get_twotime(self._h, _ptr(qs), _ptr(sg), _ptr(c2t), _ptr(full),
                                     _ptr(part)))
        return dict(qbins=qs, sg=sg, c2t={int(k): c2t[i] for i, k in enumerate(qs)},
                    g2full=full, g2partials=part, gram_ms=info.gram_ms,
                    gram_flop=info.gram_flop,
                    gram_flop_algorithmic=info.gram_flop_algorithmic)

    def autotune(self, mode=MODE_REFERENCE) -> int:
        """xpcs_autotune: search this series' kernel knobs (row capacity of the
        thread kernel, scratch words, transpose tile); returns the row capacity
        (tuning() gives all three)."""
        c = C.c_int32(0)
        check(lib().xpcs_autotune(self._h, mode, C.byref(c)))
        return c.value

    def normalized(self, f64=True, f32=False, out=None):
        """Results of the last normalisation (xpcs_normalize or a batch run)."""
        if out is None:
            shp = (self.D, self.nq)
            out = (np.empty(shp, np.float64) if f64 else None,
                   np.empty(shp, np.float64) if f64 else None,
                   np.empty(shp, np.float32) if f32 else None,
                   np.empty(shp, np.float32) if f32 else None)
        check(lib().xpcs_get_normalized(self._h, *[_ptr(a) for a in out]))
        return out

    def stage_times(self) -> dict:
        t = StageTimes()
        check(lib().xpcs_get_stage_times(self._h, C.byref(t)))
        return {n: getattr(t, n) for n, _ in StageTimes._fields_}


class Batch:
    """Several series of one device run as one CUDA graph (an xpcs_batch handle).
    The member Series objects must stay open while the batch exists."""

    def __init__(self, series):
        self.series = list(series)
        arr = (C.c_void_p * len(self.series))(*[s._h for s in self.series])
        self._arr = arr
        self._h = C.c_void_p()
        check(lib().xpcs_batch_create(arr, len(self.series), C.byref(self._h)))

    def run(self, mode=MODE_REFERENCE, f64=True, f32=False, autotune=False):
        flags = ((BATCH_F64 if f64 else 0) | (BATCH_F32 if f32 else 0)
                 | (BATCH_AUTOTUNE if autotune else 0))
        check(lib().xpcs_batch_run(self._h, mode, flags))

    def stats(self):
        """(device ms of the last run, kernels in the graph, concurrent chains)."""
        ms = C.c_float(0)
        k = C.c_int64(0)
        lanes = C.c_int32(0)
        check(lib().xpcs_batch_stats(self._h, C.byref(ms), C.byref(k), C.byref(lanes)))
        return ms.value, k.value, lanes.value

    def set_form(self, work_queue: bool):
        """Work-queue form (True) or chains form (False) for the next runs."""
        check(lib().xpcs_batch_set_form(self._h, 1 if work_queue else 0))

    def form(self):
        """(work_queue, chains) of the graph in use."""
        q, c = C.c_int32(0), C.c_int32(0)
        check(lib().xpcs_batch_get_form(self._h, C.byref(q), C.byref(c)))
        return bool(q.value), c.value

    def timeline(self):
        """(start_ms, end_ms) of every member's work in the last run, from the launch."""
        a = np.zeros(len(self.series), np.float32)
        b = np.zeros(len(self.series), np.float32)
        check(lib().xpcs_batch_timeline(self._h, _ptr(a), _ptr(b)))
        return a, b

    def close(self):
        if getattr(self, "_h", None):
            lib().xpcs_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def _desc(width, height, frames, dpl, dq, sq, flat=None, stride=1, average=1,
          static_window=None, device=0):
    d = SeriesDesc()
    d.width, d.height, d.frames, d.delays_per_level = width, height, frames, dpl
    d.stride_frames, d.avg_frames = stride, average
    d.static_window = static_window or max(frames // 10, 1)
    d.dqmap = dq.ctypes.data_as(C.POINTER(C.c_int32))
    d.sqmap = sq.ctypes.data_as(C.POINTER(C.c_int32))
    d.flatfield = flat.ctypes.data_as(C.POINTER(C.c_double)) if flat is not None else None
    d.device = device
    return d


class Server:
    """Streaming front end (an xpcs_server handle): acquisitions admitted by
    device-memory budget, frames pushed as they arrive."""

    def __init__(self, memory_budget: int, device=0):
        self._h = C.c_void_p()
        check(lib().xpcs_server_create(device, int(memory_budget), C.byref(self._h)))
        self.device = device
        self._shape = {}

    def submit(self, width, height, frames, dpl, dqmap, sqmap, expected_events, flatfield=None,
               stride=1, average=1, static_window=None) -> int:
        dq = np.ascontiguousarray(dqmap, np.int32).ravel()
        sq = np.ascontiguousarray(sqmap, np.int32).ravel()
        flat = None if flatfield is None else np.ascontiguousarray(flatfield, np.float64).ravel()
        d = _desc(width, height, frames, dpl, dq, sq, flat, stride, average, static_window,
                  self.device)
        i = C.c_int64(0)
        check(lib().xpcs_server_submit(self._h, C.byref(d), int(expected_events), C.byref(i)))
        lv, _ = delay_schedule(frames, dpl)
        nq = int(np.unique(dq[(dq > 0) & (sq > 0)]).size)
        self._shape[i.value] = (lv.size, nq, width * height)
        return i.value

    def push(self, acq_id, nnz, idx, val):
        nnz = np.ascontiguousarray(nnz, np.uint32)
        idx = np.ascontiguousarray(idx, np.int32)
        val = np.ascontiguousarray(val, np.int16)
        check(lib().xpcs_server_push_sparse(self._h, acq_id, _ptr(idx), _ptr(val), _ptr(nnz),
                                            nnz.size))

    def finish(self, acq_id, mode=MODE_REFERENCE):
        check(lib().xpcs_server_finish(self._h, acq_id, mode))

    def state(self, acq_id) -> str:
        st = C.c_int32(0)
        check(lib().xpcs_server_state(self._h, acq_id, C.byref(st)))
        return ACQ_STATES[st.value]

    def result(self, acq_id, g2ipif=False):
        D, Q, P = self._shape[acq_id]
        g2 = np.empty((D, Q))
        se = np.empty((D, Q))
        arrs = [np.empty((D, P), np.float32) for _ in range(3)] if g2ipif else [None] * 3
        check(lib().xpcs_server_result(self._h, acq_id, _ptr(g2), _ptr(se),
                                       *[_ptr(a) for a in arrs]))
        return (g2, se, *arrs) if g2ipif else (g2, se)

    def release(self, acq_id):
        check(lib().xpcs_server_release(self._h, acq_id))
        self._shape.pop(acq_id, None)

    def stats(self) -> dict:
        st = ServerStats()
        check(lib().xpcs_server_get_stats(self._h, C.byref(st)))
        return {n: getattr(st, n) for n, _ in ServerStats._fields_ if n != "reserved"}

    def close(self):
        if getattr(self, "_h", None):
            lib().xpcs_server_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def device_sm_count(device: int = 0) -> int:
    """Streaming multiprocessors of a device (xpcs_device_properties)."""
    n = C.c_int32(0)
    check(lib().xpcs_device_properties(device, C.byref(n), None, None))
    return n.value


def set_device_memory_limit(device: int, nbytes: int) -> None:
    """Cap the device memory the library may hold on `device` (0: no cap)."""
    check(lib().xpcs_set_device_memory_limit(device, int(nbytes)))


def device_memory(device: int = 0) -> tuple[int, int]:
    """(bytes the library holds on `device`, its limit; 0 = none)."""
    used, limit = C.c_uint64(0), C.c_uint64(0)
    check(lib().xpcs_get_device_memory(device, C.byref(used), C.byref(limit)))
    return used.value, limit.value


def pin(a: np.ndarray) -> np.ndarray:
    """Page-lock a numpy array in place (xpcs_pin_host); returns it."""
    if a.nbytes:
        check(lib().xpcs_pin_host(a.ctypes.data_as(C.c_void_p), a.nbytes))
    return a


def unpin(a: np.ndarray) -> None:
    if a.nbytes:
        check(lib().xpcs_unpin_host(a.ctypes.data_as(C.c_void_p)))


def multitau2(row_ptr, frame, value, frames, dpl, mode=MODE_REFERENCE, device=0):
    """Corr::multiTau2 on caller-held pixel-major rows (xpcs_multitau2)."""
    row_ptr = np.ascontiguousarray(row_ptr, np.int64)
    frame = np.ascontiguousarray(frame, np.int32)
    value = np.ascontiguousarray(value, np.float32)
    P = row_ptr.size - 1
    lv, _ = delay_schedule(frames, dpl)
    out = tuple(np.empty((lv.size, P), np.float32) for _ in range(3))
    check(lib().xpcs_multitau2(_ptr(row_ptr), _ptr(frame), _ptr(value), P, frames, dpl, mode,
                               device, *[_ptr(a) for a in out]))
    return out


def multitau2_noalloc(row_ptr_dev: int, frame_dev: int, value_dev: int, pixels: int,
                      events: int, frames: int, dpl: int, mode: int, G2_dev: int, IP_dev: int,
                      IF_dev: int, stream: int = 0) -> None:
    """xpcs_multitau2_noalloc on device buffers the caller owns (raw device
    addresses); allocates nothing on the device.  Raises XpcsError on failure."""
    check(lib().xpcs_multitau2_noalloc(
        C.c_void_p(row_ptr_dev), C.c_void_p(frame_dev), C.c_void_p(value_dev), pixels, events,
        frames, dpl, mode, C.c_void_p(G2_dev), C.c_void_p(IP_dev), C.c_void_p(IF_dev),
        C.c_void_p(stream or None)))
