"""Generate the golden fixtures of tests/golden/ from the reference itself.

Each case writes a synthetic acquisition (IMM frames + an XH5C analysis
config), runs xpcs-eigen's own `corr --g2out` (built from its unmodified
sources by oracle/ref_build) and stores inputs and every /exchange dataset in
<case>.npz.  Run where the upstream checkout is mounted:

    python tests/golden/make_golden.py [--ref CHECKOUT] [--only CASE]

CHECKOUT defaults to $XPCS_REFERENCE_SRC, else to the checkout the reference
build recipe (oracle/ref_build/Makefile) reads.

The fixtures pin the oracle (tests/test_oracle_golden.py) and the GPU path
(tests/test_gpu_parity.py) to the reference's outputs.
"""
from __future__ import annotations

import argparse
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path[:0] = [str(ROOT / "xpcs-eigen_gb300"), str(ROOT / "oracle"), str(ROOT / "tests")]

import oracle  # noqa: E402
import refio  # noqa: E402
import xpcs_synth as xs  # noqa: E402


def _sparse(acq):
    return xs.sparse_frames(acq)


def case_sparse_basic():
    acq = xs.Acquisition(width=48, height=40, frames=300, n_static=8, n_dynamic=4, mean=0.05,
                         tau_min=10, tau_max=10, seed=11, dpl=4)
    nnz, idx, val = _sparse(acq)
    return acq, dict(nnz=nnz, idx=idx, val=val), {}


def case_sparse_quirk():
    # dense bursts of events followed by sparse ones: level compaction leaves an
    # unsorted stale tail, so the reference's lower_bound misses products (Q1)
    acq = xs.Acquisition(width=32, height=32, frames=512, n_static=8, n_dynamic=4, mean=0.35,
                         tau_min=200, tau_max=200, seed=12, dpl=4)
    nnz, idx, val = _sparse(acq)
    return acq, dict(nnz=nnz, idx=idx, val=val), {}


def case_sparse_stride_avg():
    acq = xs.Acquisition(width=36, height=36, frames=601, n_static=6, n_dynamic=3, mean=0.08,
                         tau_min=30, tau_max=30, seed=13, dpl=4)
    nnz, idx, val = _sparse(acq)
    return acq, dict(nnz=nnz, idx=idx, val=val), dict(stride=2, average=3)


def case_sparse_flat():
    acq = xs.Acquisition(width=40, height=30, frames=257, n_static=10, n_dynamic=5, mean=0.1,
                         tau_min=15, tau_max=15, seed=14, dpl=8, gain_min=0.9, gain_max=1.1)
    nnz, idx, val = _sparse(acq)
    return acq, dict(nnz=nnz, idx=idx, val=val), dict(flat=True)


def case_sparse_hot():
    # hot pixels (large counts, sums beyond the integer path's exactness bound),
    # counts above 32767 that the reference reads as negative int16 (Q3), a
    # pixel lit in every frame and one lit only in the last frame
    acq = xs.Acquisition(width=24, height=24, frames=400, n_static=6, n_dynamic=3, mean=0.05,
                         tau_min=20, tau_max=20, seed=15, dpl=4)
    nnz, idx, val = _sparse(acq)
    rng = np.random.default_rng(15)
    P = acq.width * acq.height
    frames = []
    off = np.concatenate([[0], np.cumsum(nnz.astype(np.int64))])
    hot = [5, 77, 300]
    for t in range(acq.frames):
        ii = list(idx[off[t]:off[t + 1]])
        vv = list(val[off[t]:off[t + 1]])
        d = dict(zip(ii, vv))
        d[hot[0]] = int(rng.integers(200, 3000))
        if t % 3 == 0:
            d[hot[1]] = np.int16(np.uint16(40000 + t).view(np.int16))
        if t % 2 == 0:
            d[hot[2]] = int(rng.integers(1, 40))
        if t == acq.frames - 1:
            d[P - 1] = 7
        keys = sorted(d)
        frames.append((keys, [d[k] for k in keys]))
    nnz = np.array([len(k) for k, _ in frames], np.uint32)
    idx = np.concatenate([np.array(k, np.int32) for k, _ in frames])
    val = np.concatenate([np.array(v, np.int64).astype(np.int16) for _, v in frames])
    return acq, dict(nnz=nnz, idx=idx, val=val), {}


def case_sparse_dups():
    # repeated pixel indices inside a frame (summed by the filter) and
    # unsorted indices within frames
    acq = xs.Acquisition(width=20, height=20, frames=200, n_static=4, n_dynamic=2, mean=0.2,
                         tau_min=8, tau_max=8, seed=16, dpl=4, gain_min=0.95, gain_max=1.05)
    nnz, idx, val = _sparse(acq)
    rng = np.random.default_rng(16)
    off = np.concatenate([[0], np.cumsum(nnz.astype(np.int64))])
    out_i, out_v, out_n = [], [], []
    for t in range(acq.frames):
        ii = idx[off[t]:off[t + 1]].copy()
        vv = val[off[t]:off[t + 1]].copy()
        if ii.size:
            k = rng.integers(0, ii.size, size=max(1, ii.size // 4))
            ii = np.concatenate([ii, ii[k], ii[k[:1]]])
            vv = np.concatenate([vv, (vv[k] % 5 + 1).astype(np.int16), np.array([2], np.int16)])
            perm = rng.permutation(ii.size)
            ii, vv = ii[perm], vv[perm]
        out_i.append(ii)
        out_v.append(vv)
        out_n.append(ii.size)
    return acq, dict(nnz=np.array(out_n, np.uint32), idx=np.concatenate(out_i).astype(np.int32),
                     val=np.concatenate(out_v).astype(np.int16)), dict(flat=True)


def case_qmap_shared_sbin():
    # static bin 3 appears under two dynamic bins (quirk Q6 drops part of it)
    acq = xs.Acquisition(width=30, height=30, frames=256, n_static=8, n_dynamic=4, mean=0.06,
                         tau_min=12, tau_max=12, seed=17, dpl=4)
    nnz, idx, val = _sparse(acq)
    dq, sq, _, _ = xs.maps(acq)
    dq = dq.copy()
    sel = (sq == 3) & (np.arange(dq.size).reshape(dq.shape) % 3 == 0)
    dq[sel] = 3
    return acq, dict(nnz=nnz, idx=idx, val=val, dqmap=dq, sqmap=sq), {}


def case_dense_dark():
    acq = xs.Acquisition(width=24, height=20, frames=160, n_static=6, n_dynamic=3, mean=0.15,
                         tau_min=10, tau_max=10, seed=18, dpl=4, dense=True, dark_frames=12,
                         gain_min=0.9, gain_max=1.1)
    ds = xs.DenseStream(acq)
    raw = ds.next(acq.dark_frames + acq.frames)
    ds.close()
    return acq, dict(raw=raw), dict(flat=True, dense=True, lld=2.0, sigma=3.0)


def case_sparse_framesum():
    # values divided by (frame sum / mean frame sum) before multi-tau (main.cpp:314-337)
    acq = xs.Acquisition(width=36, height=36, frames=400, n_static=10, n_dynamic=5, mean=0.05,
                         tau_min=4, tau_max=60, seed=19, dpl=4)
    nnz, idx, val = _sparse(acq)
    return acq, dict(nnz=nnz, idx=idx, val=val), dict(framesum=True)


CASES = {f.__name__[5:]: f for f in [case_sparse_basic, case_sparse_quirk, case_sparse_stride_avg,
                                      case_sparse_flat, case_sparse_hot, case_sparse_dups,
                                      case_qmap_shared_sbin, case_dense_dark,
                                      case_sparse_framesum]}


def make(name, corr: Path):
    acq, data, opt = CASES[name]()
    W, H = acq.width, acq.height
    dq, sq, flat, _ = xs.maps(acq)
    dq = data.pop("dqmap", dq)
    sq = data.pop("sqmap", sq)
    stride, average = opt.get("stride", 1), opt.get("average", 1)
    use_flat = opt.get("flat", False)
    with tempfile.TemporaryDirectory() as td:
        wd = Path(td)
        imm = wd / "frames.imm"
        clock = np.arange(1, 10 ** 6, dtype=np.float64) * 0.00125
        ticks = np.arange(10 ** 6, dtype=np.int64) * 3 + 17
        if opt.get("dense"):
            raw = data["raw"]
            nd = acq.dark_frames
            refio.write_imm_dense(imm, H, W, raw, clock=clock, ticks=ticks)
            cfg = refio.config_entries(W, H, dq, sq, imm, first=nd + 1, last=nd + acq.frames,
                                       dpl=acq.dpl, compression=False,
                                       flat=flat if use_flat else None, dark=(1, nd),
                                       lld=opt["lld"], sigma=opt["sigma"])
            real = acq.frames
        else:
            nnz = data["nnz"]
            real = nnz.size
            refio.write_imm_sparse(imm, H, W, nnz, data["idx"], data["val"], clock=clock,
                                   ticks=ticks)
            cfg = refio.config_entries(W, H, dq, sq, imm, first=1, last=real, dpl=acq.dpl,
                                       stride=stride, average=average,
                                       flat=flat if use_flat else None,
                                       normalize_by_framesum=1 if opt.get("framesum") else 0)
        cpath = wd / "config.h5"
        refio.write_xh5c(cpath, cfg)
        out = refio.run_reference(corr, cpath, wd)
    frames = real // (stride * average)
    arrays = dict(data)
    arrays.update(dqmap=dq, sqmap=sq, flat=flat if use_flat else np.zeros(0),
                  clock=clock[:real + acq.dark_frames], ticks=ticks[:real + acq.dark_frames],
                  params=np.array([W, H, frames, real, acq.dpl, stride, average,
                                   int(cfg["/xpcs/static_mean_window_size"]), acq.dark_frames,
                                   1 if opt.get("dense") else 0], np.int64),
                  lld_sigma=np.array([opt.get("lld", 0.0), opt.get("sigma", 0.0)], np.float32),
                  framesum=np.int32(1 if opt.get("framesum") else 0))
    for k, v in out.items():
        if k != "_stdout":
            arrays["ref_" + k.replace("-", "_")] = v
    np.savez_compressed(HERE / f"{name}.npz", **arrays)
    return arrays


# two-time cases: (acquisition, q bins to process, smoothing method, filter, window, threading)
TWOTIME = {
    "twotime_symmetric_avg": (dict(width=40, height=40, frames=256, n_static=8, n_dynamic=4,
                                   mean=0.05, tau_min=5, tau_max=40, seed=21, dpl=4),
                              [1, 3], "symmetric", "Average", 4, False),
    "twotime_staticmap": (dict(width=48, height=40, frames=300, n_static=12, n_dynamic=6,
                               mean=0.03, tau_min=3, tau_max=100, seed=22, dpl=4),
                          [2, 4, 5], "StaticMap", "None", 3, False),
    "twotime_frame_threading": (dict(width=36, height=36, frames=200, n_static=8, n_dynamic=4,
                                     mean=0.06, tau_min=4, tau_max=30, seed=23, dpl=4),
                                [1, 2, 4], "symmetric", "None", 5, True),
}


def make_twotime(name, corr: Path):
    kw, qlist, method, filt, wsize, frame_threading = TWOTIME[name]
    acq = xs.Acquisition(**kw)
    W, H = acq.width, acq.height
    dq, sq, _, _ = xs.maps(acq)
    nnz, idx, val = xs.sparse_frames(acq)
    with tempfile.TemporaryDirectory() as td:
        wd = Path(td)
        imm = wd / "frames.imm"
        refio.write_imm_sparse(imm, H, W, nnz, idx, val)
        cfg = refio.config_entries(W, H, dq, sq, imm, first=1, last=acq.frames, dpl=acq.dpl,
                                   twotime=(qlist, method, filt, wsize))
        cpath = wd / "config.h5"
        refio.write_xh5c(cpath, cfg)
        out = refio.run_reference(corr, cpath, wd, g2out=False,
                                  extra_args=["--frame_threading"] if frame_threading else [])
    arrays = dict(nnz=nnz, idx=idx, val=val, dqmap=dq, sqmap=sq,
                  params=np.array([W, H, acq.frames, wsize, 1 if frame_threading else 0,
                                   1 if method.lower() == "staticmap" else 0,
                                   1 if filt.lower() == "average" else 0], np.int64),
                  qlist=np.asarray(qlist, np.int32))
    for k, v in out.items():
        if k != "_stdout":
            arrays["ref_" + k.replace("-", "_")] = v
    np.savez_compressed(HERE / f"{name}.npz", **arrays)
    return arrays


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=None)
    ap.add_argument("--only", default=None)
    a = ap.parse_args()
    ref = a.ref or str(oracle.reference_root())
    corr = oracle.build_reference(ref)
    if corr is None:
        sys.exit("reference sources not found at " + ref)
    for name in CASES:
        if a.only and name != a.only:
            continue
        arr = make(name, corr)
        G2 = arr["ref_G2"]
        print(f"{name}: D={G2.shape[0]} P={G2.shape[1]} -> {name}.npz")
    for name in TWOTIME:
        if a.only and name != a.only:
            continue
        arr = make_twotime(name, corr)
        print(f"{name}: " + ", ".join(f"{k} {v.shape}" for k, v in arr.items()
                                      if k.startswith("ref_")) + f" -> {name}.npz")


if __name__ == "__main__":
    main()
