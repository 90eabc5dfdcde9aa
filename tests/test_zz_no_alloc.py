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
