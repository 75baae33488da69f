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
        "markers", "fma: run in the fused multiply-add arithmetic (GPU tests default to ordered)"
    )
    config.addinivalue_line(
        "markers", "exact: run in the exact arithmetic with tree reductions"
    )


@pytest.fixture(autouse=True)
def _arithmetic(request):
    """GPU parity tests run in the ordered arithmetic: every kernel rounds
    each product and sum separately in the reference's order and every
    reduction follows the reference's blocked summation, so whole solves are
    bit-identical to the oracle's.  Tests marked `exact` run the exact form
    (parallel tree reductions), tests marked `fma` the default fused form
    (the one bench.py times)."""
    if request.node.get_closest_marker("gpu") is None:
        yield
        return
    from mojopetsc4py import _lib

    mode = "ordered"
    if request.node.get_closest_marker("fma"):
        mode = "fma"
    elif request.node.get_closest_marker("exact"):
        mode = "exact"
    before = _lib.get_arithmetic()
    _lib.set_arithmetic(mode)
    yield
    _lib.set_arithmetic(before)


def has_gpu() -> bool:
    try:
        from mojopetsc4py import _lib

        return _lib.device_count() > 0
    except Exception:
        return False
