"""The C++ `corr` driver end to end: for every golden case the IMM frames and
the analysis file are rebuilt from the fixture's inputs, `corr --g2out
--darkout` runs on them, and every dataset it writes must be bit-identical to
what the reference's own `corr` wrote for the same inputs.  The analysis file
is an HDF5 file (written into, as the reference does, and read back with the
independent walk of tests/h5walk.py) or the XH5C container."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

import build
import h5walk
import refio
from fixtures import CASES, TWOTIME_CASES, load, load_twotime, same_bits_nan

FORMATS = ["hdf5", "xh5c"]


def _as_format(cfg: Path, fmt: str) -> Path:
    """The analysis file in the given format (the XH5C file converted)."""
    if fmt == "xh5c":
        return cfg
    h5 = cfg.with_suffix(".hdf5.h5")
    r = subprocess.run([str(build.build_h5tool()), "from-xh5c", str(cfg), str(h5)],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    return h5


def _exchange(cfg: Path, fmt: str) -> dict:
    sets = h5walk.read(cfg) if fmt == "hdf5" else refio.read_xh5c(cfg)
    return {k.split("/")[-1]: v for k, v in sets.items() if k.startswith("/exchange/")}

DATASETS = ["G2", "IP", "IF", "norm-0-g2", "norm-0-stderr", "pixelSum", "frameSum",
            "partition-mean-total", "partition-mean-partial", "timestamp_clock",
            "timestamp_tick", "tau", "partition_norm_factor"]


def _write_inputs(fx, wd: Path):
    imm = wd / "frames.imm"
    W, H = fx["W"], fx["H"]
    flat = fx["flatfield"]
    if fx["dense"]:
        nd = fx["ndark"]
        refio.write_imm_dense(imm, H, W, fx["raw"], clock=fx["clock"], ticks=fx["ticks"])
        cfg = refio.config_entries(W, H, fx["dqmap"], fx["sqmap"], imm, first=nd + 1,
                                   last=nd + fx["F"], dpl=fx["dpl"], compression=False,
                                   flat=flat, dark=(1, nd), lld=float(fx["lld_sigma"][0]),
                                   sigma=float(fx["lld_sigma"][1]), static_window=fx["swin"])
    else:
        refio.write_imm_sparse(imm, H, W, fx["nnz"], fx["idx"], fx["val"], clock=fx["clock"],
                               ticks=fx["ticks"])
        cfg = refio.config_entries(W, H, fx["dqmap"], fx["sqmap"], imm, first=1, last=fx["real"],
                                   dpl=fx["dpl"], stride=fx["stride"], average=fx["avg"],
                                   flat=flat, static_window=fx["swin"],
                                   normalize_by_framesum=fx["framesum"])
    path = wd / "analysis.h5"
    refio.write_xh5c(path, cfg)
    return path


@pytest.fixture(scope="module")
def corr():
    return build.build_corr()


@pytest.mark.gpu
@pytest.mark.parametrize("fmt", FORMATS)
@pytest.mark.parametrize("case", CASES)
def test_corr_matches_reference_outputs(corr, case, fmt, tmp_path):
    fx = load(case)
    cfg = _as_format(_write_inputs(fx, tmp_path), fmt)
    r = subprocess.run([str(corr), str(cfg), "--g2out", "--darkout"], cwd=tmp_path,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    out = _exchange(cfg, fmt)
    for name in DATASETS:
        ref = fx["ref_" + name.replace("-", "_")]
        assert name in out, name
        assert same_bits_nan(np.asarray(out[name]).reshape(ref.shape), ref), name
    if fx["dense"]:
        n = fx["W"] * fx["H"]
        assert out["DarkAvg"].size == n and out["DarkStd"].size == n


@pytest.mark.gpu
@pytest.mark.parametrize("fmt", FORMATS)
@pytest.mark.parametrize("case", TWOTIME_CASES)
def test_corr_twotime_matches_reference_outputs(corr, case, fmt, tmp_path):
    fx = load_twotime(case)
    imm = tmp_path / "frames.imm"
    refio.write_imm_sparse(imm, fx["H"], fx["W"], fx["nnz"], fx["idx"], fx["val"])
    tt = (fx["qlist"], "StaticMap" if fx["static_map"] else "symmetric",
          "Average" if fx["average"] else "None", fx["wsize"])
    cfg = tmp_path / "analysis.h5"
    refio.write_xh5c(cfg, refio.config_entries(fx["W"], fx["H"], fx["dqmap"], fx["sqmap"], imm,
                                               first=1, last=fx["F"], dpl=4, twotime=tt))
    cfg = _as_format(cfg, fmt)
    args = [str(corr), str(cfg)] + (["--frame_threading"] if fx["frame_threading"] else [])
    r = subprocess.run(args, cwd=tmp_path, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    out = _exchange(cfg, fmt)
    names = ["sg", "g2full", "g2partials", "pixelSum", "frameSum"] + \
        [k[4:] for k in fx if k.startswith("ref_g2_")]
    for name in names:
        ref = fx["ref_" + name]
        assert name in out, name
        assert same_bits_nan(np.asarray(out[name]).reshape(ref.shape), ref), name
    assert "tau" not in out


def test_corr_rejects_unsupported_reader_flags(corr, tmp_path):
    r = subprocess.run([str(corr), str(tmp_path / "x.h5"), "--ufxc"], capture_output=True,
                       text=True)
    assert r.returncode != 0 and "outside the multi-tau IMM path" in r.stderr


def test_corr_rejects_unsupported_analyses(corr, tmp_path):
    fx = load("sparse_basic")
    cfg = _write_inputs(fx, tmp_path)
    ent = refio.read_xh5c(cfg)
    ent["/xpcs/analysis_type"] = "Twotime"
    ent["/xpcs/smoothing_method"] = "boxcar"
    ent["/xpcs/smoothing_filter"] = "None"
    ent["/xpcs/qphi_bin_to_process"] = np.ones((1, 1), np.int64)
    refio.write_xh5c(cfg, ent)
    r = subprocess.run([str(corr), str(cfg)], capture_output=True, text=True)
    assert r.returncode != 0 and "Smoothing method is not valid" in r.stderr


def test_corr_reads_config_and_frames_without_a_device(corr, tmp_path):
    """On a machine without a GPU the driver parses the analysis file and the
    IMM headers, then fails at series creation with the library's status."""
    import shutil
    if shutil.which("nvidia-smi"):
        pytest.skip("a GPU is present")
    for case in ("sparse_stride_avg", "dense_dark"):
        fx = load(case)
        cfg = _write_inputs(fx, tmp_path)
        r = subprocess.run([str(corr), str(cfg)], capture_output=True, text=True)
        assert r.returncode == 1
        assert f"{fx['F']} frames (stride {fx['stride']}, average {fx['avg']})" in r.stdout
        assert "(7): no CUDA device" in r.stderr
