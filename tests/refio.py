"""File I/O of the reference `corr` contract, for tests and fixture generation.

* XH5C containers: the flat HDF5 stand-in read and written by the oracle build
  of the reference (format in oracle/ref_build/shim/fakeh5.cpp).
* IMM files: 1024-byte header per frame (compression @4, rows @108, cols @112,
  bytes @116, elapsed @128 (f64), dlen @152 (u32), buffer_number @160,
  corecotick @620; layout of class Header, src/xpcs/io/imm.h:63-144), then
  int32 indices + int16 values (sparse) or int16 values (dense).
* The analysis configuration entries that Configuration::init reads
  (src/xpcs/configuration.cpp:80-242).
"""
from __future__ import annotations

import struct
import subprocess
from pathlib import Path

import numpy as np

XH5C_TYPES = {1: np.int32, 2: np.int64, 3: np.float32, 4: np.float64, 6: np.uint32,
              7: np.int16, 8: np.uint16}
_DTYPE_CODE = {np.dtype(v): k for k, v in XH5C_TYPES.items()}


def write_xh5c(path, entries: dict):
    recs = []
    for name, value in entries.items():
        if isinstance(value, str):
            b = value.encode()
            code, dims = 5, [1]
        else:
            a = np.asarray(value)
            code = _DTYPE_CODE[a.dtype]
            dims = list(a.shape) if a.ndim else [1]
            b = np.ascontiguousarray(a).tobytes()
        recs.append(struct.pack("<I", len(name)) + name.encode()
                    + struct.pack("<II", code, len(dims)) + struct.pack("<%dQ" % len(dims), *dims)
                    + struct.pack("<Q", len(b)) + b)
    with open(path, "wb") as f:
        f.write(b"XH5C" + struct.pack("<II", 1, len(recs)) + b"".join(recs))


def read_xh5c(path) -> dict:
    data = Path(path).read_bytes()
    assert data[:4] == b"XH5C"
    _, n = struct.unpack_from("<II", data, 4)
    o, out = 12, {}
    for _ in range(n):
        (pl,) = struct.unpack_from("<I", data, o)
        o += 4
        name = data[o:o + pl].decode()
        o += pl
        code, rank = struct.unpack_from("<II", data, o)
        o += 8
        dims = struct.unpack_from("<%dQ" % rank, data, o)
        o += 8 * rank
        (nb,) = struct.unpack_from("<Q", data, o)
        o += 8
        raw = data[o:o + nb]
        o += nb
        if code == 5:
            out[name] = raw.decode(errors="replace")
        else:
            out[name] = np.frombuffer(raw, dtype=XH5C_TYPES[code]).reshape(dims).copy()
    return out


def _header(compression: int, rows: int, cols: int, dlen: int, frame: int, elapsed: float,
            tick: int) -> bytes:
    h = bytearray(1024)
    struct.pack_into("<i", h, 4, compression)
    struct.pack_into("<ii", h, 108, rows, cols)
    struct.pack_into("<i", h, 116, 2)
    struct.pack_into("<d", h, 128, elapsed)
    struct.pack_into("<I", h, 152, dlen)
    struct.pack_into("<i", h, 160, frame)
    struct.pack_into("<i", h, 620, tick)
    return bytes(h)


def write_imm_sparse(path, rows, cols, nnz, idx, val, clock=None, ticks=None):
    nnz = np.asarray(nnz, np.uint32)
    off = np.concatenate([[0], np.cumsum(nnz.astype(np.int64))])
    with open(path, "wb") as f:
        for t in range(nnz.size):
            a, b = off[t], off[t + 1]
            f.write(_header(6, rows, cols, int(nnz[t]), t,
                            float(clock[t]) if clock is not None else t * 0.005,
                            int(ticks[t]) if ticks is not None else t))
            f.write(np.asarray(idx[a:b], np.int32).tobytes())
            f.write(np.asarray(val[a:b], np.int16).tobytes())


def write_imm_dense(path, rows, cols, frames: np.ndarray, clock=None, ticks=None):
    frames = np.asarray(frames, np.int16).reshape(-1, rows * cols)
    with open(path, "wb") as f:
        for t in range(frames.shape[0]):
            f.write(_header(0, rows, cols, rows * cols, t,
                            float(clock[t]) if clock is not None else t * 0.005,
                            int(ticks[t]) if ticks is not None else t))
            f.write(frames[t].tobytes())


def config_entries(width, height, dqmap, sqmap, imm_path, first=1, last=None, dpl=4,
                   stride=1, average=1, static_window=None, compression=True, flat=None,
                   dark=(0, 0), lld=0.0, sigma=0.0, entry="/xpcs", output="/exchange",
                   normalize_by_framesum=0, twotime=None) -> dict:
    """The /xpcs and /measurement datasets Configuration::init reads.  Scalars
    are int32 (getInteger reads into a 4-byte int, quirk Q10); tables are 2-D."""
    assert last is not None
    frames = (last - first + 1) // (stride * average)
    e = {
        entry + "/compression": "ENABLED" if compression else "DISABLED",
        entry + "/output_data": output,
        "/measurement/instrument/detector/x_dimension": np.int32(width),
        "/measurement/instrument/detector/y_dimension": np.int32(height),
        entry + "/dqmap": np.asarray(dqmap, np.int32).reshape(height, width),
        entry + "/sqmap": np.asarray(sqmap, np.int32).reshape(height, width),
        entry + "/transposed": "DISABLED",
        entry + "/data_begin": np.int32(first),
        entry + "/data_end": np.int32(last),
        entry + "/data_begin_todo": np.int32(first),
        entry + "/data_end_todo": np.int32(last),
        entry + "/delays_per_level": np.int32(dpl),
        entry + "/dark_begin_todo": np.int32(dark[0]),
        entry + "/dark_end_todo": np.int32(dark[1]),
        entry + "/twotime2onetime_window_size": np.int32(1),
        entry + "/normalize_by_framesum": np.int32(normalize_by_framesum),
        entry + "/static_mean_window_size": np.int32(static_window or max(frames // 10, 1)),
        entry + "/stride_frames": np.int32(stride),
        entry + "/avg_frames": np.int32(average),
        "/measurement/instrument/detector/x_pixel_size": np.float32(0.075),
        "/measurement/instrument/detector/y_pixel_size": np.float32(0.075),
        "/measurement/instrument/detector/adu_per_photon": np.float32(1.0),
        "/measurement/instrument/detector/exposure_time": np.float32(0.005),
        "/measurement/instrument/detector/efficiency": np.float32(1.0),
        "/measurement/instrument/detector/distance": np.float32(5000.0),
        "/measurement/instrument/source_begin/beam_intensity_transmitted": np.float32(1.0),
        "/measurement/sample/thickness": np.float32(1.0),
        entry + "/flatfield_enabled": "ENABLED" if flat is not None else "DISABLED",
        entry + "/analysis_type": "Multitau",
        entry + "/input_file_local": str(imm_path),
    }
    if flat is not None:
        e["/measurement/instrument/detector/flatfield"] = np.asarray(flat, np.float64).reshape(
            height, width)
    if twotime is not None:  # (q bins to process, smoothing method, smoothing filter, window)
        qlist, method, filt, wsize = twotime
        e[entry + "/analysis_type"] = "Twotime"
        e[entry + "/smoothing_method"] = method
        e[entry + "/smoothing_filter"] = filt
        e[entry + "/qphi_bin_to_process"] = np.asarray(qlist, np.int64).reshape(-1, 1)
        e[entry + "/twotime2onetime_window_size"] = np.int32(wsize)
    if dark[0] != dark[1]:
        e[entry + "/lld"] = np.float32(lld)
        e[entry + "/sigma"] = np.float32(sigma)
    return e


def run_reference(corr: Path, config: Path, workdir: Path, threads: int | None = None,
                  g2out: bool = True, timeout: int = 3600, extra_args=()) -> dict:
    """Run the reference `corr` on an XH5C config; return its /exchange datasets
    and the stdout (stage timers)."""
    import os
    env = dict(os.environ)
    if threads:
        env["OMP_NUM_THREADS"] = str(threads)
    args = [str(corr), str(config)] + (["--g2out"] if g2out else []) + list(extra_args)
    r = subprocess.run(args, cwd=workdir, env=env, capture_output=True, text=True,
                       timeout=timeout)
    if r.returncode != 0:
        raise RuntimeError(f"reference corr failed ({r.returncode}): {r.stderr[-2000:]}")
    out = read_xh5c(config)
    res = {k.split("/")[-1]: v for k, v in out.items() if k.startswith("/exchange/")}
    res["_stdout"] = r.stdout
    return res
