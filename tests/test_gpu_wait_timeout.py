"""The time-out path of the kernels' bounded device waits, without a fault: a
self-test kernel waits on an mbarrier that nothing arrives at (no copy issued,
nothing in flight), gives up after a short limit and raises the handle's
device flag; dg_sync must then report DG_ERR_CUDA once, and the handle must
go on stepping correctly."""
import ctypes

import pytest

import pydugks
from _cases import make_pair, run_both
from seeded import rel_err

pytestmark = pytest.mark.gpu


def test_bounded_wait_times_out_and_the_handle_recovers():
    eng, orc, f0 = make_pair("walls", "fp32")  # a TMA-fed form
    eng.sync()
    cycles = ctypes.c_longlong(0)
    assert pydugks.lib().dg_selftest_wait_timeout(eng._h, 1024, ctypes.byref(cycles)) == pydugks.DG_OK
    print(f"1024 polls of an mbarrier that never completes: {cycles.value} SM cycles")
    assert cycles.value > 0
    with pytest.raises(pydugks.DugksError) as e:
        eng.sync()
    assert e.value.code == pydugks.DG_ERR_CUDA and "timed out" in str(e.value)
    eng.sync()  # reading the flag cleared it
    got, want = run_both(eng, orc, f0, 1, 5)
    assert rel_err(got, want) <= 2e-5
    eng.sync()


def test_selftest_rejects_out_of_range_limits():
    eng, _, _ = make_pair("walls", "fp64")
    for bad in (0, -1, (1 << 22) + 1):
        assert pydugks.lib().dg_selftest_wait_timeout(eng._h, bad, None) == pydugks.DG_ERR_ARG
