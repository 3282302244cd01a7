"""Build recipe for the native parts of xpcs-eigen_gb300.

  libxpcs_gpu.so    CUDA kernels + C ABI (include/xpcs_gpu.h), sm_103a only
  libxpcs_synth.so  seeded synthetic acquisitions (benchmark/test inputs)
  libxpcs_synth_gpu.so  the same sparse frames drawn on the GPU (large benchmark inputs)
  corr              C++ command-line driver with the reference's flags

Everything is compiled in-tree into xpcs-eigen_gb300/_build/.  Translation
units are compiled in parallel; no cmake.  Float code is compiled without
fused multiply-add contraction (-fmad=false, -ffp-contract=off) because the
kernels reproduce the reference's float arithmetic bit for bit.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
BUILD = PKG / "_build"
OBJ = BUILD / "obj"
INCLUDE = ROOT / "include"
CSRC = PKG / "csrc"

NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC",
                     "-I", str(INCLUDE), "-I", str(CSRC)]
GPU_SOURCES = ["abi.cu", "scan.cu", "k_transpose.cu", "k_multitau.cu", "k_normalize.cu",
               "qmap.cpp", "noalloc.cu", "k_dense.cu", "k_side.cu", "batch.cu",
               "server.cpp", "k_twotime.cu", "k_twotime_tc.cu"]

LIB_GPU = BUILD / "libxpcs_gpu.so"
LIB_SYNTH = BUILD / "libxpcs_synth.so"
CORR = BUILD / "corr"
HOST = PKG / "host"


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(map(str, cmd)) + "\n" + r.stdout + r.stderr)
    return r


def _stale(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def build_gpu(force: bool = False, verbose: bool = False) -> Path:
    OBJ.mkdir(parents=True, exist_ok=True)
    headers = [INCLUDE / "xpcs_gpu.h", CSRC / "xpcs_internal.h", CSRC / "f64emu.cuh",
               CSRC / "mt_replay.cuh",
               CSRC / "classify.cuh"]
    jobs = []
    objs = []
    for src in GPU_SOURCES:
        s = CSRC / src
        o = OBJ / (s.stem + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            cmd = [NVCC] + NVCC_FLAGS + (["-Xptxas", "-v"] if verbose else []) + [
                "-c", str(s), "-o", str(o)]
            if src.endswith(".cpp"):
                cmd = [NVCC] + NVCC_FLAGS + ["-x", "cu", "-c", str(s), "-o", str(o)]
            jobs.append(cmd)
    if jobs:
        with ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            for r in ex.map(_run, jobs):
                if verbose and r.stderr:
                    print(r.stderr, file=sys.stderr)
    if force or _stale(LIB_GPU, objs):
        _run([NVCC] + ARCH + ["-shared", "-o", str(LIB_GPU)] + [str(o) for o in objs])
    return LIB_GPU


def build_synth(force: bool = False) -> Path:
    BUILD.mkdir(parents=True, exist_ok=True)
    src = PKG / "synth" / "xpcs_synth.cpp"
    if force or _stale(LIB_SYNTH, [src, PKG / "synth" / "xpcs_synth.h"]):
        _run(["g++", "-std=c++17", "-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
              "-o", str(LIB_SYNTH), str(src)])
    return LIB_SYNTH


LIB_SYNTH_GPU = BUILD / "libxpcs_synth_gpu.so"


def build_synth_gpu(force: bool = False) -> Path:
    """The GPU draw of the synthetic sparse frames (benchmark inputs)."""
    BUILD.mkdir(parents=True, exist_ok=True)
    src = PKG / "synth" / "xpcs_synth_gpu.cu"
    if force or _stale(LIB_SYNTH_GPU, [src, PKG / "synth" / "xpcs_synth.h"]):
        _run([NVCC] + ARCH + ["-O3", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC",
                              "-shared", "-I", str(PKG / "synth"), "-o", str(LIB_SYNTH_GPU),
                              str(src)])
    return LIB_SYNTH_GPU


# AddressSanitizer + UndefinedBehaviorSanitizer builds of the host programs
# (tests/test_host_sanitizers.py); every undefined behaviour ends the run.
SANITIZE = ["-fsanitize=address,undefined", "-fno-sanitize-recover=undefined",
            "-fno-omit-frame-pointer", "-g", "-O1"]


def build_corr(force: bool = False, sanitize: bool = False) -> Path:
    """The C++ `corr` driver, linked against libxpcs_gpu.so (rpath $ORIGIN);
    with sanitize, the host code built with the sanitizers as corr_sanitized."""
    srcs = [HOST / "corr_main.cpp", HOST / "xh5c.cpp", HOST / "h5lite.cpp", HOST / "imm.cpp"]
    deps = srcs + [HOST / "xh5c.h", HOST / "h5lite.h", HOST / "imm.h", INCLUDE / "xpcs_gpu.h",
                   LIB_GPU]
    out = BUILD / "corr_sanitized" if sanitize else CORR
    if force or _stale(out, deps):
        opt = SANITIZE if sanitize else ["-O2"]
        _run(["g++", "-std=c++17"] + opt + ["-ffp-contract=off", "-I", str(INCLUDE), "-o", str(out)]
             + [str(x) for x in srcs] + ["-L", str(BUILD), "-lxpcs_gpu",
                                         "-Wl,-rpath,$ORIGIN"])
    return out


H5TOOL = BUILD / "h5lite_tool"


def build_h5tool(force: bool = False, sanitize: bool = False) -> Path:
    """The h5lite command line (dump / create / put / from-xh5c) used by the
    tests; with sanitize, built with the sanitizers as h5lite_tool_sanitized."""
    BUILD.mkdir(parents=True, exist_ok=True)
    srcs = [HOST / "h5lite_tool.cpp", HOST / "h5lite.cpp", HOST / "xh5c.cpp"]
    out = BUILD / "h5lite_tool_sanitized" if sanitize else H5TOOL
    if force or _stale(out, srcs + [HOST / "h5lite.h", HOST / "xh5c.h"]):
        opt = SANITIZE if sanitize else ["-O2"]
        _run(["g++", "-std=c++17"] + opt + ["-Wall", "-o", str(out)] + [str(x) for x in srcs])
    return out


def build_all(force: bool = False) -> None:
    with ThreadPoolExecutor(max_workers=3) as ex:
        futs = [ex.submit(build_gpu, force), ex.submit(build_synth, force),
                ex.submit(build_synth_gpu, force)]
        for f in futs:
            f.result()
    build_corr(force)
    build_h5tool(force)


if __name__ == "__main__":
    build_all(force="--force" in sys.argv)
    print("built", LIB_GPU, LIB_SYNTH, CORR)
