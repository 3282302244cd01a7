"""Host-side failure handling of the `corr` driver, on the CPU (no GPU needed).

Faults are made on the host: IMM files cut short or with a corrupt frame
length, configurations with a field missing, pixel indices outside the
detector.  `corr --dry-run` reads the configuration and every frame the
analysis would use and stops before any GPU work, so each fault must end the
run with exit status 1 and a message naming it -- where the reference's own
reader trusts dlen and carries on after a short read (src/xpcs/io/imm.cpp:
70-118)."""
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

import refio
from fixtures import load

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT / "xpcs-eigen_gb300"))


@pytest.fixture(scope="module")
def corr():
    from build import build_corr
    return build_corr()


def _case(tmp, name="sparse_basic", dense=False, **cfg_over):
    fx = load(name)
    imm = tmp / "frames.imm"
    if dense:
        refio.write_imm_dense(imm, fx["H"], fx["W"], fx["raw"])
    else:
        refio.write_imm_sparse(imm, fx["H"], fx["W"], fx["nnz"], fx["idx"], fx["val"])
    cfg = refio.config_entries(fx["W"], fx["H"], fx["dqmap"], fx["sqmap"], imm, first=1,
                               last=fx["real"], dpl=fx["dpl"], compression=not dense)
    for k, v in cfg_over.items():
        if v is None:
            cfg.pop(k)
        else:
            cfg[k] = v
    path = tmp / "analysis.h5"
    refio.write_xh5c(path, cfg)
    return fx, imm, path


def _run(corr, path):
    r = subprocess.run([str(corr), str(path), "--dry-run"], capture_output=True, text=True,
                       timeout=120)
    return r.returncode, r.stdout + r.stderr


def test_valid_input_passes_the_dry_run(corr, tmp_path):
    fx, _, path = _case(tmp_path)
    rc, out = _run(corr, path)
    assert rc == 0, out
    assert f"{int(fx['nnz'].sum())} events" in out and "input is valid" in out


def test_hdf5_analysis_file_passes_the_dry_run(corr, tmp_path):
    """The analysis file as HDF5 (the XH5C case converted by h5lite): the
    driver reads the configuration from it and validates the frames."""
    from build import build_h5tool
    fx, _, path = _case(tmp_path)
    h5 = tmp_path / "analysis_hdf5.h5"
    r = subprocess.run([str(build_h5tool()), "from-xh5c", str(path), str(h5)],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    rc, out = _run(corr, h5)
    assert rc == 0, out
    assert f"{int(fx['nnz'].sum())} events" in out and "input is valid" in out
    # a chunk of the file cut away: a reading error naming HDF5, not a crash
    b = h5.read_bytes()
    h5.write_bytes(b[: len(b) // 3])
    rc, out = _run(corr, h5)
    assert rc == 1 and "HDF5" in out


def test_dense_input_passes_the_dry_run(corr, tmp_path):
    fx = load("dense_dark")
    imm = tmp_path / "frames.imm"
    refio.write_imm_dense(imm, fx["H"], fx["W"], fx["raw"])
    cfg = refio.config_entries(fx["W"], fx["H"], fx["dqmap"], fx["sqmap"], imm,
                               first=fx["ndark"] + 1, last=fx["ndark"] + fx["real"],
                               dpl=fx["dpl"], compression=False, dark=(1, fx["ndark"]),
                               lld=float(fx["lld_sigma"][0]), sigma=float(fx["lld_sigma"][1]))
    path = tmp_path / "analysis.h5"
    refio.write_xh5c(path, cfg)
    rc, out = _run(corr, path)
    assert rc == 0, out


def test_truncated_imm_file_is_an_error(corr, tmp_path):
    _, imm, path = _case(tmp_path)
    data = imm.read_bytes()
    for cut in (len(data) - 3, len(data) - 1024 - 7, 1024 + 2):  # values, header, indices
        imm.write_bytes(data[:cut])
        rc, out = _run(corr, path)
        assert rc == 1, out
        assert "truncated" in out or "ends after" in out, out


def test_missing_frames_are_an_error(corr, tmp_path):
    fx, imm, path = _case(tmp_path)
    data = imm.read_bytes()
    # drop the last frame whole: a clean end of file, but fewer frames than configured
    last = 1024 + 6 * int(fx["nnz"][-1])
    imm.write_bytes(data[:len(data) - last])
    rc, out = _run(corr, path)
    assert rc == 1 and "ends after" in out, out


def test_corrupt_frame_length_is_an_error(corr, tmp_path):
    fx, imm, path = _case(tmp_path)
    data = bytearray(imm.read_bytes())
    # the first frame's dlen (uint32 at byte 152) beyond the detector's pixels
    data[152:156] = np.uint32(fx["W"] * fx["H"] + 1).tobytes()
    imm.write_bytes(bytes(data))
    rc, out = _run(corr, path)
    assert rc == 1 and "dlen" in out, out


def test_dense_frame_length_must_equal_the_detector(corr, tmp_path):
    fx = load("dense_dark")
    imm = tmp_path / "frames.imm"
    refio.write_imm_dense(imm, fx["H"], fx["W"], fx["raw"])
    data = bytearray(imm.read_bytes())
    frame_bytes = 1024 + 2 * fx["W"] * fx["H"]
    # frame 3's dlen one short: the reader would misalign every later frame
    data[3 * frame_bytes + 152:3 * frame_bytes + 156] = np.uint32(fx["W"] * fx["H"] - 1).tobytes()
    imm.write_bytes(bytes(data))
    cfg = refio.config_entries(fx["W"], fx["H"], fx["dqmap"], fx["sqmap"], imm,
                               first=fx["ndark"] + 1, last=fx["ndark"] + fx["real"],
                               dpl=fx["dpl"], compression=False, dark=(1, fx["ndark"]),
                               lld=float(fx["lld_sigma"][0]), sigma=float(fx["lld_sigma"][1]))
    path = tmp_path / "analysis.h5"
    refio.write_xh5c(path, cfg)
    rc, out = _run(corr, path)
    assert rc == 1 and "dense dlen" in out, out


def test_pixel_index_outside_the_detector_is_an_error(corr, tmp_path):
    fx, imm, path = _case(tmp_path)
    data = bytearray(imm.read_bytes())
    # first event of the first frame with events
    t = int(np.argmax(fx["nnz"] > 0))
    off = t * 1024 + int(np.sum(fx["nnz"][:t], dtype=np.int64)) * 6 + 1024
    data[off:off + 4] = np.int32(fx["W"] * fx["H"] + 3).tobytes()
    imm.write_bytes(bytes(data))
    rc, out = _run(corr, path)
    assert rc == 1 and "outside the detector" in out, out


@pytest.mark.parametrize("field", ["/xpcs/delays_per_level", "/xpcs/dqmap",
                                   "/measurement/instrument/detector/x_dimension",
                                   "/xpcs/output_data", "/xpcs/input_file_local"])
def test_missing_configuration_field_is_an_error(corr, tmp_path, field):
    _, _, path = _case(tmp_path, **{field: None})
    rc, out = _run(corr, path)
    assert rc == 1 and field in out, out


def test_wrong_map_size_and_missing_imm_file(corr, tmp_path):
    fx = load("sparse_basic")
    _, _, path = _case(tmp_path, **{"/xpcs/dqmap": np.ones((2, 3), np.int32)})
    rc, out = _run(corr, path)
    assert rc == 1 and "dqmap" in out, out
    _, imm, path = _case(tmp_path)
    imm.unlink()
    rc, out = _run(corr, path)
    assert rc == 1 and "cannot open" in out, out
    assert fx["W"] > 0
