import pathlib
import sys

import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]
PKG = ROOT / "gpu-cpm_gb300"
for p in (str(ROOT), str(PKG)):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line(
        "markers", "gpu: needs a CUDA GPU (GB300) and the built libgpucpm_gb300.so")


@pytest.fixture(scope="session")
def engine_lib():
    """Build (if stale) and load the CUDA engine library."""
    import build as engine_build  # gpu-cpm_gb300/build.py
    engine_build.build()
    import gpucpm
    return gpucpm.library()
