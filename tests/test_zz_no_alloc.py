"""lpg_count_seirp_static: the count_SEIRP entry point that allocates nothing.

Its scratch is a file-scope device array; this file is collected last so
that it runs both after every other test and, on its own, in a fresh
process.  It calls both entry points through the C ABI and requires equal
outputs on two calls in a row, with different shapes in between, so that
nothing left in the static scratch by one call can leak into the next.
"""

import ctypes as C

import numpy as np
import pytest

from test_count_seirp import NAMES
from test_count_seirp import _gpu_count
from test_count_seirp import random_columns

pytestmark = pytest.mark.gpu


def _same(a, b):
    for name, x, y in zip(NAMES + ("n_invalid",), a, b):
        np.testing.assert_array_equal(x, y, err_msg=name)


@pytest.mark.parametrize(
    "n,G,ns,offset",
    [
        (1_000_003, 774, 3, 0),
        (2_000_000, 4096, 4, 0),  # largest histogram: the grid shrinks to fit the static scratch
        (300_001, 14, 1, 1),
        (0, 7, 2, 0),
    ],
)
def test_static_matches_allocating_twice(n, G, ns, offset):
    cols = random_columns(n, G, ns, seed=100 + G, bad_nodes=7 if n else 0)
    ref = _gpu_count("lpg_count_seirp", cols, G, ns, n, offset)
    first = _gpu_count("lpg_count_seirp_static", cols, G, ns, n, offset)
    second = _gpu_count("lpg_count_seirp_static", cols, G, ns, n, offset)
    _same(ref, first)
    _same(ref, second)


def test_static_after_a_different_shape():
    big = random_columns(600_000, 4096, 4, seed=1)
    small = random_columns(50_000, 3, 2, seed=2)
    _gpu_count("lpg_count_seirp_static", big, 4096, 4, 600_000)
    ref = _gpu_count("lpg_count_seirp", small, 3, 2, 50_000)
    _same(ref, _gpu_count("lpg_count_seirp_static", small, 3, 2, 50_000))


def test_static_rejects_sizes_beyond_the_limit():
    from laser_polio_gb300 import _lib

    lib = _lib.load()
    z = C.c_void_p(0)
    rc = lib.lpg_count_seirp_static(*([z] * 5), 4097, 3, 0, *([z] * 10))
    assert rc == -1
    assert b"n_nodes 4097" in lib.lpg_op_last_error()


def _pool_bytes():
    """(free device bytes, the default memory pool's used and reserved bytes
    now, its used high-water mark) from the CUDA driver."""
    import torch

    cu = C.CDLL("libcuda.so.1")
    dev = C.c_int(0)
    assert cu.cuDeviceGet(C.byref(dev), torch.cuda.current_device()) == 0
    pool = C.c_void_p(0)
    assert cu.cuDeviceGetDefaultMemPool(C.byref(pool), dev) == 0
    out = []
    for attr in (7, 5, 8):  # CU_MEMPOOL_ATTR_USED_MEM_CURRENT, _RESERVED_MEM_CURRENT, _USED_MEM_HIGH
        v = C.c_uint64(0)
        assert cu.cuMemPoolGetAttribute(pool, attr, C.byref(v)) == 0
        out.append(v.value)
    free, _ = torch.cuda.mem_get_info()
    return (free, *out)


def _reset_pool_high_water():
    import torch

    cu = C.CDLL("libcuda.so.1")
    dev = C.c_int(0)
    assert cu.cuDeviceGet(C.byref(dev), torch.cuda.current_device()) == 0
    pool = C.c_void_p(0)
    assert cu.cuDeviceGetDefaultMemPool(C.byref(pool), dev) == 0
    zero = C.c_uint64(0)
    assert cu.cuMemPoolSetAttribute(pool, 8, C.byref(zero)) == 0  # resets the used high-water mark


def _prepared(entry, cols, G, ns, n):
    """Device inputs and outputs allocated once; returns call() (one launch
    of `entry`, synchronised) and read() (the outputs on the host)."""
    import torch

    from laser_polio_gb300 import _lib

    lib = _lib.load()
    dev = [torch.from_numpy(c).cuda() for c in cols]
    outs = [torch.zeros((G,), dtype=torch.int32, device="cuda") for _ in range(4)]
    outs += [torch.zeros((G, ns), dtype=torch.int32, device="cuda") for _ in range(2)]
    outs += [torch.zeros((G,), dtype=torch.int32, device="cuda") for _ in range(2)]
    bad = torch.zeros((1,), dtype=torch.int64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream

    def call():
        rc = getattr(lib, entry)(*[c.data_ptr() for c in dev], G, ns, n, *[o.data_ptr() for o in outs],
                                 bad.data_ptr(), C.c_void_p(stream))
        assert rc == 0, lib.lpg_op_last_error()
        torch.cuda.synchronize()

    def read():
        return tuple(o.cpu().numpy() for o in outs) + (int(bad.item()),)

    return call, read


def test_static_calls_allocate_nothing():
    """Around two static calls (after one that set up the device, which may
    load the module that holds the array) neither the device's free memory
    nor the default memory pool's used or reserved bytes change, and the
    pool's used high-water mark does not rise: a scratch allocation slipped
    into the entry point, freed or not, would fail here."""
    import torch

    cols = random_columns(500_000, 774, 3, seed=9)
    want = _gpu_count("lpg_count_seirp", cols, 774, 3, 500_000)
    call, read = _prepared("lpg_count_seirp_static", cols, 774, 3, 500_000)
    call()
    torch.cuda.synchronize()
    _reset_pool_high_water()
    free0, used0, res0, high0 = _pool_bytes()
    got = []
    for _ in range(2):
        call()
        got.append(read())
    free1, used1, res1, high1 = _pool_bytes()
    for g in got:
        _same(want, g)
    assert (used1, res1) == (used0, res0)
    assert high1 <= used0
    assert free1 == free0
