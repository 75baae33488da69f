"""Host logic of the batched and mixed forms (no GPU): stacking systems into
one block-diagonal CSR, the rank sharding, option validation and the ctypes
layouts of the form options."""
import ctypes

import numpy as np
import pytest

from mojopetsc4py import _lib, gallery
from mojopetsc4py.batch import BatchOptions, shard_systems, stack_systems


def test_stacking_keeps_each_system_in_its_own_rows_and_columns():
    rng = np.random.default_rng(0)
    systems = [gallery.rgg_laplacian(n, rng) for n in (30, 1, 57)]
    sys_rows, indptr, indices, data = stack_systems(systems)
    assert sys_rows.tolist() == [0, 30, 31, 88]
    assert indptr[-1] == len(indices) == len(data) == sum(int(ip[-1]) for ip, _, _ in systems)
    for s, (ip, ix, v) in enumerate(systems):
        r0, r1 = sys_rows[s], sys_rows[s + 1]
        for i in range(r0, r1):
            cols = indices[indptr[i]:indptr[i + 1]]
            assert np.all((cols >= r0) & (cols < r1))
            li = i - r0
            np.testing.assert_array_equal(cols - r0, ix[ip[li]:ip[li + 1]])
            np.testing.assert_array_equal(data[indptr[i]:indptr[i + 1]], v[ip[li]:ip[li + 1]])


@pytest.mark.parametrize("world", [1, 2, 3, 8])
def test_sharding_covers_every_system_once_and_balances(world):
    costs = [int(c) for c in np.random.default_rng(world).integers(1, 1000, size=97)]
    shards = shard_systems(costs, world)
    assert len(shards) == world
    flat = sorted(s for sh in shards for s in sh)
    assert flat == list(range(97))
    loads = [sum(costs[s] for s in sh) for sh in shards]
    assert max(loads) - min(loads) <= max(costs)
    assert shard_systems(costs, world) == shards  # deterministic on every rank


def test_option_structs_match_the_c_layout():
    # gp_batch_options: 4 int32 then 4 doubles; gp_mixed_options: 4 int32, 2 doubles
    assert ctypes.sizeof(BatchOptions) == 4 * 4 + 4 * 8
    from mojopetsc4py.mixed import MixedOptions, MixedResult

    assert ctypes.sizeof(MixedOptions) == 4 * 4 + 2 * 8
    assert ctypes.sizeof(MixedResult) == 4 * 4 + 8
    o = BatchOptions()
    _lib.lib().gp_batch_options_default(ctypes.byref(o))
    assert (o.pc_type, o.precision, o.rtol) == (2, 0, 1e-8)
    m = MixedOptions()
    _lib.lib().gp_mixed_options_default(ctypes.byref(m))
    assert (m.restart, m.tri_sweeps, m.rtol) == (30, 4, 1e-10)


def test_batch_rejects_bad_shapes_before_touching_a_device():
    lib = _lib.lib()
    h = ctypes.c_void_p()
    rows = np.array([0, 2], dtype=np.int64)
    ip = np.array([0, 1, 2], dtype=np.int64)
    ix = np.array([0, 1], dtype=np.int64)
    v = np.ones(2)
    # 3 right-hand sides is not a supported count
    st = lib.gp_batch_create(ctypes.byref(h), 1, rows.ctypes.data, ip.ctypes.data,
                             ix.ctypes.data, v.ctypes.data, 3, None)
    assert st == 1 and b"right-hand sides" in lib.gp_last_error()
    # a row coupling outside its system
    rows2 = np.array([0, 1, 2], dtype=np.int64)
    ix2 = np.array([1, 1], dtype=np.int64)
    st = lib.gp_batch_create(ctypes.byref(h), 2, rows2.ctypes.data, ip.ctypes.data,
                             ix2.ctypes.data, v.ctypes.data, 1, None)
    assert st == 1 and b"own system" in lib.gp_last_error()
