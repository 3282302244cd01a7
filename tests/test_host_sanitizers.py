"""The host C++ of the drop-in driver -- the IMM reader, the HDF5 reader and
writer, the analysis-file layer and corr's input checks -- built with
AddressSanitizer and UndefinedBehaviorSanitizer (build.py SANITIZE) and run on
the CPU over valid inputs and over the faults the host tests make: IMM files
cut short or with a corrupt frame length, a configuration with a field
missing, pixel indices outside the detector, HDF5 files with bytes flipped at
random.  Every run must end with its normal status (0, or 1 with a message)
and with no sanitizer report.  `corr --dry-run` stops before any GPU work."""
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

import refio
from fixtures import load

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT / "xpcs-eigen_gb300"))

ENV = dict(os.environ, ASAN_OPTIONS="detect_leaks=0:abort_on_error=0:exitcode=86",
           UBSAN_OPTIONS="print_stacktrace=1:halt_on_error=1:exitcode=87")
REPORTS = ("ERROR: AddressSanitizer", "runtime error:", "ERROR: UndefinedBehaviorSanitizer")


def _sanitizers_available(tmp: Path) -> bool:
    src = tmp / "probe.cpp"
    src.write_text("int main() { return 0; }\n")
    r = subprocess.run(["g++", "-fsanitize=address,undefined", str(src), "-o",
                        str(tmp / "probe")], capture_output=True)
    return r.returncode == 0


@pytest.fixture(scope="module")
def tools(tmp_path_factory):
    if not _sanitizers_available(tmp_path_factory.mktemp("probe")):
        pytest.skip("the compiler has no sanitizer runtimes")
    from build import build_corr, build_h5tool
    return str(build_corr(sanitize=True)), str(build_h5tool(sanitize=True))


def _run(*args):
    r = subprocess.run([str(a) for a in args], capture_output=True, timeout=300, env=ENV)
    # a corrupted file's names are arbitrary bytes
    out = (r.stdout + r.stderr).decode(errors="replace")
    assert not any(s in out for s in REPORTS), out[-3000:]
    assert r.returncode in (0, 1), (r.returncode, out[-3000:])
    return r.returncode, out


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


def test_corr_input_checks_under_the_sanitizers(tools, tmp_path):
    corr, h5tool = tools
    # valid sparse input, then the same analysis file converted to HDF5
    _, imm, path = _case(tmp_path)
    assert _run(corr, path, "--dry-run")[0] == 0
    h5 = tmp_path / "analysis_hdf5.h5"
    assert _run(h5tool, "from-xh5c", path, h5)[0] == 0
    assert _run(corr, h5, "--dry-run")[0] == 0
    data = imm.read_bytes()
    # cut short inside a frame's data
    imm.write_bytes(data[: len(data) * 2 // 3])
    assert _run(corr, path, "--dry-run")[0] == 1
    # a corrupt frame length (the first header's dlen field, bytes 152-155)
    bad = bytearray(data)
    bad[152:156] = np.uint32(0x7FFFFFFF).tobytes()
    imm.write_bytes(bytes(bad))
    assert _run(corr, path, "--dry-run")[0] == 1
    # a pixel index outside the detector
    fx = load("sparse_basic")
    idx = fx["idx"].copy()
    idx[len(idx) // 3] = fx["W"] * fx["H"] + 5
    refio.write_imm_sparse(imm, fx["H"], fx["W"], fx["nnz"], idx, fx["val"])
    assert _run(corr, path, "--dry-run")[0] == 1
    # the HDF5 analysis file with a chunk cut away
    b = h5.read_bytes()
    h5.write_bytes(b[: len(b) // 3])
    assert _run(corr, h5, "--dry-run")[0] == 1


def test_dense_frames_under_the_sanitizers(tools, tmp_path):
    corr, _ = tools
    fx = load("dense_dark")
    imm = tmp_path / "frames.imm"
    refio.write_imm_dense(imm, fx["H"], fx["W"], fx["raw"])
    cfg = refio.config_entries(fx["W"], fx["H"], fx["dqmap"], fx["sqmap"], imm,
                               first=fx["ndark"] + 1, last=fx["ndark"] + fx["real"],
                               dpl=fx["dpl"], compression=False, dark=(1, fx["ndark"]),
                               lld=float(fx["lld_sigma"][0]), sigma=float(fx["lld_sigma"][1]))
    path = tmp_path / "analysis.h5"
    refio.write_xh5c(path, cfg)
    assert _run(corr, path, "--dry-run")[0] == 0
    # frame 3's dlen one short of the detector
    data = bytearray(imm.read_bytes())
    frame_bytes = 1024 + 2 * fx["W"] * fx["H"]
    data[3 * frame_bytes + 152:3 * frame_bytes + 156] = np.uint32(fx["W"] * fx["H"] - 1).tobytes()
    imm.write_bytes(bytes(data))
    assert _run(corr, path, "--dry-run")[0] == 1


@pytest.mark.parametrize("field", ["/xpcs/delays_per_level", "/xpcs/dqmap",
                                   "/measurement/instrument/detector/x_dimension"])
def test_missing_configuration_field_under_the_sanitizers(tools, tmp_path, field):
    corr, _ = tools
    _, _, path = _case(tmp_path, **{field: None})
    assert _run(corr, path, "--dry-run")[0] == 1


def test_hdf5_writer_and_corrupted_files_under_the_sanitizers(tools, tmp_path):
    _, h5tool = tools
    f = tmp_path / "base.h5"
    _run(h5tool, "create", f)
    puts = {"/a/i16": ("i16", "2,2", [-32768, 7, 8, 32767]),
            "/a/u32": ("u32", "1", [4294967295]),
            "/b/c/f32": ("f32", "3", [1.5, -0.25, 3.0e38]),
            "/b/c/f64": ("f64", "2,1,2", [1e-300, -2.5, 3.141592653589793, 0.0]),
            "/b/s": ("str", "scalar", ["/exchange"])}
    for path, (kind, dims, vals) in puts.items():
        assert _run(h5tool, "put", f, path, kind, dims, *vals)[0] == 0
    # an overwrite in place, and a refused change of shape
    assert _run(h5tool, "put", f, "/b/c/f32", "f32", "3", 1, 2, 3)[0] == 0
    assert _run(h5tool, "put", f, "/b/c/f32", "f32", "4", 1, 2, 3, 4)[0] == 1
    rc, out = _run(h5tool, "dump", f)
    assert rc == 0 and "/b/c/f32" in out
    base = f.read_bytes()
    rng = np.random.default_rng(11)
    bad = tmp_path / "bad.h5"
    for trial in range(60):
        b = bytearray(base)
        for _ in range(int(rng.integers(1, 6))):
            i = int(rng.integers(0, len(b)))
            b[i] = int(rng.integers(0, 256))
        if trial % 10 == 0:
            b = b[: int(rng.integers(8, len(b)))]
        bad.write_bytes(bytes(b))
        _run(h5tool, "dump", bad)
