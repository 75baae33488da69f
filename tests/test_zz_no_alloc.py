"""gp_vec_reduce_static: the reductions of gp_vec_reduce with scratch in the
library's static device memory and the result in a caller-owned device buffer
(nothing allocated).  Compared with gp_vec_reduce on the same inputs, two
calls in a row (the ticket word must come back to zero after each call).
This file is collected last so that it also runs after every other suite."""
import ctypes

import numpy as np
import pytest

from mojopetsc4py import _lib
from mojopetsc4py import _device as dev

pytestmark = pytest.mark.gpu

OPS = {0: "dot", 1: "sum x^2", 2: "sum |x|", 3: "sum x", 4: "(x.y, x.x)", 5: "max |x|"}


def reduce_host(op, x, y):
    out = (ctypes.c_double * 2)()
    _lib.check(_lib.lib().gp_vec_reduce(op, x.numel(), x.data_ptr(), y.data_ptr(), out,
                                        dev.stream_ptr()))
    return np.array(out[: 2 if op == 4 else 1])


def reduce_static(op, x, y, out):
    _lib.check(_lib.lib().gp_vec_reduce_static(op, x.numel(), x.data_ptr(), y.data_ptr(),
                                               out.data_ptr(), dev.stream_ptr()))


@pytest.mark.parametrize("n", [1, 257, 100003, 3_000_001])
@pytest.mark.parametrize("op", sorted(OPS))
def test_static_scratch_reduction_matches_the_allocating_entry(op, n):
    import torch

    g = torch.Generator(device="cuda").manual_seed(n + op)
    x = torch.randn(n, dtype=torch.float64, device="cuda", generator=g)
    y = torch.randn(n, dtype=torch.float64, device="cuda", generator=g)
    want = reduce_host(op, x, y)
    # the same sums in numpy (FP64, pairwise): an independent value
    xh, yh = x.cpu().numpy(), y.cpu().numpy()
    ref = {0: [xh @ yh], 1: [xh @ xh], 2: [np.abs(xh).sum()], 3: [xh.sum()],
           4: [xh @ yh, xh @ xh], 5: [np.abs(xh).max()]}[op]
    out = torch.full((2,), float("nan"), dtype=torch.float64, device="cuda")
    for _ in range(2):
        out.fill_(float("nan"))
        reduce_static(op, x, y, out)
        got = out.cpu().numpy()[: len(want)]
        # same kernel and grid: equal to the last bit; the bound is the test's
        np.testing.assert_allclose(got, want, rtol=1e-13, atol=0)
        # sums of n terms of either sign: rounding relative to sum |terms|
        scale = {0: np.abs(xh * yh).sum(), 3: np.abs(xh).sum()}.get(op, abs(ref[0]))
        np.testing.assert_allclose(got[0], ref[0], rtol=0, atol=1e-13 * scale + 1e-300)
        if op == 4:
            np.testing.assert_allclose(got[1], ref[1], rtol=1e-13)


def test_empty_vector_gives_zero():
    import torch

    x = torch.empty(0, dtype=torch.float64, device="cuda")
    out = torch.full((2,), 7.0, dtype=torch.float64, device="cuda")
    reduce_static(4, x, x, out)
    assert out.cpu().tolist() == [0.0, 0.0]


def test_rejects_sizes_beyond_the_limit_and_bad_ops():
    import torch

    x = torch.zeros(4, dtype=torch.float64, device="cuda")
    out = torch.zeros(2, dtype=torch.float64, device="cuda")
    lib = _lib.lib()
    st = lib.gp_vec_reduce_static(0, 2**31, x.data_ptr(), x.data_ptr(), out.data_ptr(), None)
    assert st == 1 and b"2^31" in lib.gp_last_error()
    st = lib.gp_vec_reduce_static(9, 4, x.data_ptr(), x.data_ptr(), out.data_ptr(), None)
    assert st == 1
    st = lib.gp_vec_reduce_static(0, 4, x.data_ptr(), x.data_ptr(), None, None)
    assert st == 1
