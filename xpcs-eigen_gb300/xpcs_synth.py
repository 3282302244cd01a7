"""ctypes front end of libxpcs_synth (seeded synthetic XPCS acquisitions).

Workload presets follow the benchmark configurations of the multi-tau path:
``c0`` 512x512 x 1000 sparse frames (mean 0.01, tau_c 20, 18/9 rings, dpl 4),
``c1`` 1024x1024 x 10000 sparse frames (mean 0.005, tau_c log-uniform [5,500],
36/18 rings, dpl 8), ``c2`` 960x960 x 20000 dense frames + 100 darks (mean
0.02, 35 ADU/photon, dark N(100, 8^2), read noise 4, gain U[0.9,1.1], 3 sigma).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libxpcs_synth.so"
LIB_GPU = HERE / "_build" / "libxpcs_synth_gpu.so"


class _Params(C.Structure):
    _fields_ = [
        ("width", C.c_int32), ("height", C.c_int32), ("frames", C.c_int32),
        ("n_static", C.c_int32), ("n_dynamic", C.c_int32),
        ("center_x", C.c_double), ("center_y", C.c_double), ("mask_fraction", C.c_double),
        ("mean", C.c_double), ("tau_min", C.c_double), ("tau_max", C.c_double),
        ("seed", C.c_uint64), ("dark_frames", C.c_int32), ("dark_mean", C.c_double),
        ("dark_sigma", C.c_double), ("read_noise", C.c_double), ("adu_per_photon", C.c_double),
        ("gain_min", C.c_double), ("gain_max", C.c_double),
    ]


@dataclass
class Acquisition:
    width: int
    height: int
    frames: int
    n_static: int = 18
    n_dynamic: int = 9
    center_x: float | None = None
    center_y: float | None = None
    mask_fraction: float = 0.05
    mean: float = 0.01
    tau_min: float = 20.0
    tau_max: float = 20.0
    seed: int = 1234
    dpl: int = 4
    dense: bool = False
    dark_frames: int = 0
    dark_mean: float = 100.0
    dark_sigma: float = 8.0
    read_noise: float = 4.0
    adu_per_photon: float = 35.0
    gain_min: float = 1.0
    gain_max: float = 1.0
    lld: float = 0.0
    sigma: float = 3.0
    extra: dict = field(default_factory=dict)

    def _struct(self) -> _Params:
        p = _Params()
        p.width, p.height, p.frames = self.width, self.height, self.frames
        p.n_static, p.n_dynamic = self.n_static, self.n_dynamic
        p.center_x = self.width / 2 if self.center_x is None else self.center_x
        p.center_y = self.height / 2 if self.center_y is None else self.center_y
        p.mask_fraction, p.mean = self.mask_fraction, self.mean
        p.tau_min, p.tau_max, p.seed = self.tau_min, self.tau_max, self.seed
        p.dark_frames, p.dark_mean, p.dark_sigma = self.dark_frames, self.dark_mean, self.dark_sigma
        p.read_noise, p.adu_per_photon = self.read_noise, self.adu_per_photon
        p.gain_min, p.gain_max = self.gain_min, self.gain_max
        return p


PRESETS = {
    "c0": dict(width=512, height=512, frames=1000, n_static=18, n_dynamic=9, mean=0.01,
               tau_min=20.0, tau_max=20.0, dpl=4),
    "c1": dict(width=1024, height=1024, frames=10000, n_static=36, n_dynamic=18, mean=0.005,
               tau_min=5.0, tau_max=500.0, dpl=8),
    "c2": dict(width=960, height=960, frames=20000, n_static=36, n_dynamic=18, mean=0.02,
               tau_min=5.0, tau_max=500.0, dpl=8, dense=True, dark_frames=100,
               gain_min=0.9, gain_max=1.1, lld=0.0, sigma=3.0),
}


def preset(name: str, **overrides) -> Acquisition:
    kw = dict(PRESETS[name])
    kw.update(overrides)
    return Acquisition(**kw)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not LIB.exists():
            from build import build_synth  # noqa: E402  (package-local build recipe)
            build_synth()
        L = C.CDLL(str(LIB))
        L.xs_make_maps.restype = C.c_int
        L.xs_sparse.restype = C.c_int64
        L.xs_sparse.argtypes = [C.POINTER(_Params), C.POINTER(C.c_uint32),
                                C.POINTER(C.POINTER(C.c_int32)), C.POINTER(C.POINTER(C.c_int16))]
        L.xs_dense_create.restype = C.c_void_p
        L.xs_dense_create.argtypes = [C.POINTER(_Params)]
        L.xs_dense_next.argtypes = [C.c_void_p, C.c_int32, C.POINTER(C.c_int16)]
        L.xs_dense_destroy.argtypes = [C.c_void_p]
        L.xs_free.argtypes = [C.c_void_p]
        L.xs_pixel_fields.argtypes = [C.POINTER(_Params), C.c_void_p, C.c_void_p]
        _lib = L
    return _lib


def maps(acq: Acquisition):
    """dqmap, sqmap (int32 [H][W]), flatfield (float64 [H][W]), tau_c per ring."""
    p = acq._struct()
    P = acq.width * acq.height
    dq = np.zeros(P, np.int32)
    sq = np.zeros(P, np.int32)
    flat = np.zeros(P, np.float64)
    tau = np.zeros(max(acq.n_dynamic, 1), np.float64)
    lib().xs_make_maps(C.byref(p), dq.ctypes.data_as(C.POINTER(C.c_int32)),
                       sq.ctypes.data_as(C.POINTER(C.c_int32)),
                       flat.ctypes.data_as(C.POINTER(C.c_double)),
                       tau.ctypes.data_as(C.POINTER(C.c_double)))
    shape = (acq.height, acq.width)
    return dq.reshape(shape), sq.reshape(shape), flat.reshape(shape), tau


def sparse_frames(acq: Acquisition):
    """(nnz[frames] uint32, idx int32, val int16) in frame-major order."""
    p = acq._struct()
    nnz = np.zeros(acq.frames, np.uint32)
    pi = C.POINTER(C.c_int32)()
    pv = C.POINTER(C.c_int16)()
    n = lib().xs_sparse(C.byref(p), nnz.ctypes.data_as(C.POINTER(C.c_uint32)), C.byref(pi),
                        C.byref(pv))
    if n < 0:
        raise MemoryError("xs_sparse allocation failed")
    idx = np.ctypeslib.as_array(pi, shape=(max(n, 1),))[:n].copy()
    val = np.ctypeslib.as_array(pv, shape=(max(n, 1),))[:n].copy()
    lib().xs_free(C.cast(pi, C.c_void_p))
    lib().xs_free(C.cast(pv, C.c_void_p))
    return nnz, idx, val


_glib = None


def glib():
    """libxpcs_synth_gpu: the same sparse frames drawn on the current CUDA device."""
    global _glib
    if _glib is None:
        if not LIB_GPU.exists():
            from build import build_synth_gpu  # noqa: E402
            build_synth_gpu()
        L = C.CDLL(str(LIB_GPU))
        L.xsg_sparse.restype = C.c_int64
        L.xsg_sparse.argtypes = [C.POINTER(_Params), C.c_void_p, C.c_void_p,
                                 C.POINTER(C.c_uint32), C.POINTER(C.c_void_p),
                                 C.POINTER(C.c_void_p)]
        L.xsg_dense.restype = C.c_int
        L.xsg_dense.argtypes = [C.POINTER(_Params), C.c_void_p, C.c_void_p, C.c_void_p,
                                C.POINTER(C.c_void_p)]
        L.xsg_free.argtypes = [C.c_void_p]
        L.xsg_to_host.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64]
        _glib = L
    return _glib


def pixel_fields(acq: Acquisition):
    """Per-pixel AR(1) coefficients (a, s) of the speckle field, float32 [P] each."""
    p = acq._struct()
    P = acq.width * acq.height
    a = np.zeros(P, np.float32)
    s = np.zeros(P, np.float32)
    lib().xs_pixel_fields(C.byref(p), a.ctypes.data_as(C.c_void_p), s.ctypes.data_as(C.c_void_p))
    return a, s


class DeviceFrames:
    """Sparse frames of ``sparse_frames(acq)`` drawn on the current CUDA device:
    ``nnz`` (host uint32 [frames]), ``idx`` / ``val`` device pointers of
    ``events`` int32 / int16 entries.  Free with close()."""

    def __init__(self, acq: Acquisition):
        p = acq._struct()
        a, s = pixel_fields(acq)
        self.nnz = np.zeros(acq.frames, np.uint32)
        pi, pv = C.c_void_p(), C.c_void_p()
        n = glib().xsg_sparse(C.byref(p), a.ctypes.data_as(C.c_void_p),
                              s.ctypes.data_as(C.c_void_p),
                              self.nnz.ctypes.data_as(C.POINTER(C.c_uint32)), C.byref(pi),
                              C.byref(pv))
        if n < 0:
            raise MemoryError("xsg_sparse failed")
        self.events, self.idx, self.val = int(n), pi.value, pv.value

    def to_host(self):
        idx = np.empty(self.events, np.int32)
        val = np.empty(self.events, np.int16)
        if self.events:
            glib().xsg_to_host(idx.ctypes.data_as(C.c_void_p), self.idx, idx.nbytes)
            glib().xsg_to_host(val.ctypes.data_as(C.c_void_p), self.val, val.nbytes)
        return self.nnz, idx, val

    def close(self):
        if getattr(self, "idx", None):
            glib().xsg_free(self.idx)
            glib().xsg_free(self.val)
            self.idx = self.val = None

    def __del__(self):
        self.close()


class DeviceDenseFrames:
    """The dense frames of ``DenseStream(acq)`` (``dark_frames`` darks, then
    ``frames`` data frames) drawn on the current CUDA device: ``ptr`` is an
    int16 [dark_frames + frames][P] device array.  Free with close()."""

    def __init__(self, acq: Acquisition):
        p = acq._struct()
        a, s = pixel_fields(acq)
        _, _, flat, _ = maps(acq)
        flat = np.ascontiguousarray(flat.ravel(), np.float64)
        out = C.c_void_p()
        if glib().xsg_dense(C.byref(p), a.ctypes.data_as(C.c_void_p), s.ctypes.data_as(C.c_void_p),
                            flat.ctypes.data_as(C.c_void_p), C.byref(out)) != 0:
            raise MemoryError("xsg_dense failed")
        self.P = acq.width * acq.height
        self.dark_frames, self.frames = acq.dark_frames, acq.frames
        self.ptr = out.value

    def frame_ptr(self, k: int) -> int:
        """Device address of sequence frame k (darks first)."""
        return self.ptr + 2 * self.P * k

    def to_host(self, first: int, count: int) -> np.ndarray:
        out = np.empty((count, self.P), np.int16)
        if count:
            glib().xsg_to_host(out.ctypes.data_as(C.c_void_p), C.c_void_p(self.frame_ptr(first)),
                               out.nbytes)
        return out

    def close(self):
        if getattr(self, "ptr", None):
            glib().xsg_free(self.ptr)
            self.ptr = None

    def __del__(self):
        self.close()


class DenseStream:
    """Dense frames in order: ``dark_frames`` darks, then ``frames`` data frames."""

    def __init__(self, acq: Acquisition):
        self.acq = acq
        self._p = acq._struct()
        self._h = lib().xs_dense_create(C.byref(self._p))

    def next(self, count: int) -> np.ndarray:
        out = np.empty((count, self.acq.width * self.acq.height), np.int16)
        lib().xs_dense_next(self._h, count, out.ctypes.data_as(C.POINTER(C.c_int16)))
        return out

    def close(self):
        if self._h:
            lib().xs_dense_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()
