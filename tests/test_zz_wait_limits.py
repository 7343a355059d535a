"""Bounded waits on the GPU: the run kernel's grid barrier, met by one block fewer than
the launch holds (a block that never arrives), gives up after its poll limit instead of
waiting forever, every block leaves, and the host reads OXG_ERR_TIMEOUT; the context
stays usable afterwards. No fault, trap or hang is made: the stall is a barrier arrival
that never happens, and every wait in the kernel is bounded.

Collected after the other GPU tests (file name), since the stalled launch takes a few
seconds."""

import ctypes as C
import time

import pytest

pytestmark = pytest.mark.gpu


def test_grid_barrier_gives_up_and_reports_timeout(native):
    from oxdna import _abi
    L = native
    n = 8
    res = (C.c_int * n)()
    # every block arrives: the barrier passes
    assert L.oxg_selftest_barrier(n, -1, res, None) == _abi.OK
    assert list(res) == [1] * n
    # block 3 never arrives: the others give up (poll limit, then the abort word)
    t0 = time.perf_counter()
    rc = L.oxg_selftest_barrier(n, 3, res, None)
    waited = time.perf_counter() - t0
    assert rc == _abi.ERR_TIMEOUT, (rc, L.oxg_last_error())
    assert list(res) == [0, 0, 0, -1, 0, 0, 0, 0]
    assert waited < 60.0
    # block 0 (the one that adds the phase bit) missing: the same
    assert L.oxg_selftest_barrier(n, 0, res, None) == _abi.ERR_TIMEOUT
    assert list(res) == [-1] + [0] * (n - 1)
    # the context still works
    assert L.oxg_selftest_barrier(n, -1, res, None) == _abi.OK
    assert list(res) == [1] * n
