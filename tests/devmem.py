"""Device buffers for tests that act as a caller owning its own GPU memory.

The CUDA runtime's C API through ctypes (cudaMalloc / cudaMemcpy / streams),
so these tests need no framework to hold device memory.  Pointers made here
live in the same CUDA context as the library's own (the primary context of
the device).
"""
from __future__ import annotations

import ctypes as C
import glob
import os

import numpy as np

_rt = None

H2D, D2H = 1, 2


def _cudart():
    global _rt
    if _rt is None:
        home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
        cands = [os.path.join(home, "lib64", "libcudart.so")]
        cands += sorted(glob.glob(os.path.join(home, "lib64", "libcudart.so.*")))
        cands += sorted(glob.glob(os.path.join(home, "targets", "*", "lib", "libcudart.so*")))
        err = None
        for c in cands:
            try:
                _rt = C.CDLL(c)
                break
            except OSError as e:
                err = e
        if _rt is None:
            raise RuntimeError(f"libcudart not found under {home}: {err}")
        _rt.cudaMalloc.argtypes = [C.POINTER(C.c_void_p), C.c_size_t]
        _rt.cudaFree.argtypes = [C.c_void_p]
        _rt.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
        _rt.cudaSetDevice.argtypes = [C.c_int]
        _rt.cudaStreamCreate.argtypes = [C.POINTER(C.c_void_p)]
        _rt.cudaStreamDestroy.argtypes = [C.c_void_p]
        _rt.cudaStreamSynchronize.argtypes = [C.c_void_p]
        _rt.cudaGetErrorString.restype = C.c_char_p
    return _rt


def _check(rc, what):
    if rc != 0:
        raise RuntimeError(f"{what}: {_cudart().cudaGetErrorString(rc).decode()}")


def set_device(dev: int) -> None:
    _check(_cudart().cudaSetDevice(dev), "cudaSetDevice")


class Buffer:
    """A device allocation of `nbytes` (at least 1 byte)."""

    def __init__(self, nbytes: int):
        self.nbytes = int(nbytes)
        p = C.c_void_p()
        _check(_cudart().cudaMalloc(C.byref(p), max(self.nbytes, 1)), "cudaMalloc")
        self.ptr = p.value

    @classmethod
    def from_array(cls, a: np.ndarray) -> "Buffer":
        a = np.ascontiguousarray(a)
        b = cls(a.nbytes)
        if a.nbytes:
            _check(_cudart().cudaMemcpy(b.ptr, a.ctypes.data, a.nbytes, H2D), "cudaMemcpy H2D")
        return b

    def upload(self, a: np.ndarray) -> None:
        a = np.ascontiguousarray(a)
        assert a.nbytes <= self.nbytes
        if a.nbytes:
            _check(_cudart().cudaMemcpy(self.ptr, a.ctypes.data, a.nbytes, H2D), "cudaMemcpy H2D")

    def download(self, dtype, shape) -> np.ndarray:
        out = np.empty(shape, dtype)
        assert out.nbytes <= self.nbytes
        if out.nbytes:
            _check(_cudart().cudaMemcpy(out.ctypes.data, self.ptr, out.nbytes, D2H),
                   "cudaMemcpy D2H")
        return out

    def free(self) -> None:
        if self.ptr:
            _cudart().cudaFree(self.ptr)
            self.ptr = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.free()


class Stream:
    def __init__(self):
        s = C.c_void_p()
        _check(_cudart().cudaStreamCreate(C.byref(s)), "cudaStreamCreate")
        self.handle = s.value

    def synchronize(self) -> None:
        _check(_cudart().cudaStreamSynchronize(self.handle), "cudaStreamSynchronize")

    def close(self) -> None:
        if self.handle:
            _cudart().cudaStreamDestroy(self.handle)
            self.handle = None
