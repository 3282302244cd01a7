"""pytest configuration: the `gpu` marker and import paths.

Tests marked `gpu` need a CUDA device (run with -m gpu); everything else runs
on CPU only.  The native libraries are built in-tree on first use."""
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
for p in (ROOT / "xpcs-eigen_gb300", ROOT / "oracle", ROOT / "tests"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
