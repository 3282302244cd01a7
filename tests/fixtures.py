"""Golden fixtures (tests/golden/*.npz) and their replay through the oracle.

A fixture holds the inputs of one `corr` run and every dataset the reference
wrote (keys ref_*).  params = [W, H, frames, real_frames, dpl, stride, avg,
static_window, dark_frames, dense]."""
from __future__ import annotations

from pathlib import Path

import numpy as np

import oracle

GOLDEN = Path(__file__).resolve().parent / "golden"
CASES = sorted(p.stem for p in GOLDEN.glob("*.npz") if not p.stem.startswith("twotime"))
TWOTIME_CASES = sorted(p.stem for p in GOLDEN.glob("twotime*.npz"))
SPARSE_CASES = [c for c in CASES if not c.startswith("dense")]


def load(name: str) -> dict:
    with np.load(GOLDEN / f"{name}.npz") as z:
        fx = {k: z[k] for k in z.files}
    W, H, F, real, dpl, stride, avg, swin, ndark, dense = (int(x) for x in fx["params"])
    fx.update(W=W, H=H, F=F, real=real, dpl=dpl, stride=stride, avg=avg, swin=swin,
              ndark=ndark, dense=bool(dense))
    fx["flatfield"] = fx["flat"] if fx["flat"].size else None
    fx["framesum"] = int(fx["framesum"]) if "framesum" in fx else 0
    return fx


def load_twotime(name: str) -> dict:
    with np.load(GOLDEN / f"{name}.npz") as z:
        fx = {k: z[k] for k in z.files}
    W, H, F, wsize, frame_threading, static_map, average = (int(x) for x in fx["params"])
    fx.update(W=W, H=H, F=F, wsize=wsize, frame_threading=bool(frame_threading),
              static_map=bool(static_map), average=bool(average))
    return fx


def oracle_twotime(fx):
    qm = oracle.QMap(fx["dqmap"], fx["sqmap"])
    rows, side = oracle.sparse_filter(qm, fx["nnz"], fx["idx"], fx["val"], fx["F"])
    return oracle.twotime(qm, rows, fx["F"], fx["qlist"], fx["static_map"], fx["average"],
                          fx["wsize"], sort_pixels=fx["frame_threading"]), side


def oracle_filter(fx):
    qm = oracle.QMap(fx["dqmap"], fx["sqmap"])
    flat = fx["flatfield"]
    if fx["dense"]:
        raw = fx["raw"]
        nd = fx["ndark"]
        f = flat.ravel() if flat is not None else np.ones(fx["W"] * fx["H"])
        da, ds = oracle.dark_image(raw[:nd], f)
        rows, side = oracle.dense_filter(
            qm, raw[nd:], fx["F"], da, ds, float(fx["lld_sigma"][0]), float(fx["lld_sigma"][1]),
            real_frames=fx["real"], stride=fx["stride"], average=fx["avg"],
            static_window=fx["swin"], flat=flat.ravel() if flat is not None else None,
            clock=fx["clock"][nd:], ticks=fx["ticks"][nd:])
    else:
        rows, side = oracle.sparse_filter(
            qm, fx["nnz"], fx["idx"], fx["val"], fx["F"], real_frames=fx["real"],
            stride=fx["stride"], average=fx["avg"], static_window=fx["swin"],
            flat=flat.ravel() if flat is not None else None, clock=fx["clock"],
            ticks=fx["ticks"])
    if fx["framesum"]:
        rows = oracle.framesum_normalize(rows, side["frames_sum"], fx["F"])
    return qm, rows, side


def oracle_run(fx, mode=0):
    qm, rows, side = oracle_filter(fx)
    G2, IP, IF = oracle.multitau2(rows, fx["F"], fx["dpl"], mode)
    g2, se = oracle.normalize_f32(qm, G2, IP, IF)
    g64, s64 = oracle.normalize_f64(qm, G2, IP, IF)
    return dict(qm=qm, rows=rows, side=side, G2=G2, IP=IP, IF=IF, g2=g2, se=se, g64=g64, s64=s64)


def same_bits(a, b) -> bool:
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b)
    return a.shape == b.shape and a.dtype == b.dtype and bool(
        np.array_equal(a.view(np.uint8), b.view(np.uint8)))


def same_bits_nan(a, b) -> bool:
    """Bit-identical except that any NaN matches any NaN (x86 and CUDA produce
    different NaN payloads for 0/0)."""
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b)
    if a.shape != b.shape or a.dtype != b.dtype:
        return False
    na, nb = np.isnan(a), np.isnan(b)
    if not np.array_equal(na, nb):
        return False
    return bool(np.array_equal(a[~na].view(np.uint8), b[~nb].view(np.uint8)))


def max_rel_err(a, b) -> float:
    """Max relative error over finite entries; NaN/inf positions must agree."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    fa, fb = np.isfinite(a), np.isfinite(b)
    assert np.array_equal(fa, fb), "non-finite positions differ"
    assert np.array_equal(np.isnan(a), np.isnan(b))
    if not fa.any():
        return 0.0
    d = np.abs(a[fa] - b[fa])
    s = np.maximum(np.abs(b[fa]), 1e-300)
    return float(np.max(np.where(d == 0, 0.0, d / s)))


def frames_of(fx, chunks=1):
    """Split the fixture's raw sparse frames into `chunks` ingest calls."""
    nnz = fx["nnz"]
    off = np.concatenate([[0], np.cumsum(nnz.astype(np.int64))])
    bounds = np.linspace(0, nnz.size, chunks + 1).astype(int)
    for a, b in zip(bounds[:-1], bounds[1:]):
        yield nnz[a:b], fx["idx"][off[a]:off[b]], fx["val"][off[a]:off[b]]
