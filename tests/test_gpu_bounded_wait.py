"""The single-pass scans' bounded waits end with a status instead of a hang:
a look-back against a status word that nothing writes gives up at its poll
limit, raises RTA_DEV_SPIN_TIMEOUT, and the context keeps working (a tree
built right after it equals the oracle's)."""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import oracle as O
from rta_gb300 import lib as L, plugin as P, scenes as S

pytestmark = pytest.mark.gpu


def test_lookback_wait_gives_up_with_a_status_and_the_context_survives():
    lib = L.load()
    flags = C.c_uint32(0)
    assert lib.rta_selftest_bounded_wait(P._stream(), C.byref(flags)) == L.OK
    assert flags.value & L.DEV_SPIN_TIMEOUT
    assert flags.value & ~L.DEV_SPIN_TIMEOUT == 0
    # the device still runs work correctly afterwards
    tris = S.clusters(2, 3000, seed=5)
    lb = O.lbvh_build(tris, 30)
    bvh = P.lbvh_constructor(morton_bits=30).build(P.cuda_ftl(tris))
    np.testing.assert_array_equal(bvh.codes(), lb.codes.astype(np.uint32))
    np.testing.assert_array_equal(bvh.index_buffer, lb.ids)
    assert bvh.status() == 0
