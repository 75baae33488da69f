import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "mojo-petsc4py_gb300"), os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (runs on the GB300)")
    config.addinivalue_line(
        "markers", "fma: run in the fused multiply-add arithmetic (GPU tests default to exact)"
    )


@pytest.fixture(autouse=True)
def _arithmetic(request):
    """GPU parity tests run in the exact arithmetic, where every kernel's
    result is bit-identical to the reference's sequential loops; tests marked
    `fma` run in the (default) fused form and compare within a tolerance."""
    if request.node.get_closest_marker("gpu") is None:
        yield
        return
    from mojopetsc4py import _lib

    before = _lib.get_arithmetic()
    _lib.set_arithmetic("fma" if request.node.get_closest_marker("fma") else "exact")
    yield
    _lib.set_arithmetic(before)


def has_gpu() -> bool:
    try:
        from mojopetsc4py import _lib

        return _lib.device_count() > 0
    except Exception:
        return False
