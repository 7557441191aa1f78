import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: larger inputs")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Builds libfbk.so and the oracle once per session (no-op when up to date)."""
    from fastbact_gb300.build import build
    from oracle import orc

    build()
    orc.build()
    yield


def _has_gpu() -> bool:
    try:
        import ctypes

        from fastbact_gb300 import _native as N

        h = ctypes.c_void_p()
        st = N.lib().fbk_ctx_create(0, 0, ctypes.byref(h))
        if st == 0:
            N.lib().fbk_ctx_destroy(h)
            return True
        return False
    except Exception:
        return False


@pytest.fixture(scope="session")
def ctx():
    """A device context; GPU tests fail (not skip) when no device is present, so
    a missing GPU on a GPU run is loud."""
    from fastbact_gb300.api import Context

    c = Context(0)
    yield c
    c.close()


def pytest_collection_modifyitems(config, items):
    # When the run did not select GPU tests explicitly and no device exists, skip them.
    markexpr = config.getoption("-m") or ""
    if "gpu" in markexpr and "not gpu" not in markexpr:
        return
    if _has_gpu():
        return
    skip = pytest.mark.skip(reason="no CUDA device in this environment")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)
