"""The allocation-free statistics entry point (dg_stats_values_noalloc).

It exists for callers that cannot allocate device memory when they ask for
statistics -- hosts whose own allocator owns all of the device memory, or
whose memory budget the state arrays have already spent -- and keeps its
scratch in a fixed array of the library instead.  It must give the statistics
of dg_stats_values (the entry point that allocates its scratch) on the same
state, within the tolerance of
tests/test_gpu_parity.py::test_stats_match_oracle, call after call: the state
changes between the two calls checked here, so a stale scratch array would
show.  Collected last so that a failure here leaves the rest of a -x run done.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

import pydugks  # noqa: E402
from _cases import make_pair  # noqa: E402
from seeded import rel_err, seeded_state  # noqa: E402

TOL = 1e-13


def _noalloc(eng, out, stream):
    info = eng.info
    f = eng.device_ptr(pydugks.DG_BUF_F)
    rc = pydugks.lib().dg_stats_values_noalloc(
        ctypes.c_void_p(f), eng.nx, eng.ny, eng.nz, info.pitch, info.pop_stride, info.dt / 2.0,
        info.ambient[0], info.ambient[1], info.ambient[2], ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream))
    assert rc == 0, pydugks.lib().dg_noalloc_last_error().decode()


def test_noalloc_statistics_equal_the_allocating_entry_point_on_two_calls_in_a_row():
    eng, _, _ = make_pair("walls", "fp64", seed=5)
    stream = torch.cuda.current_stream().cuda_stream
    eng.set_stream(stream)
    nx = eng.nx
    out = torch.full((12 + 9 * nx + 1,), float("nan"), dtype=torch.float64, device="cuda")
    for call in range(2):
        eng.run(1 + 7 * call, 7)
        diag_ref, prof_ref = eng.stats_values()
        _noalloc(eng, out, stream)
        torch.cuda.synchronize()
        o = out.cpu().numpy()
        diag, prof, bad = o[:12], o[12:12 + 9 * nx].reshape(nx, 9), o[12 + 9 * nx]
        assert bad == 0
        assert rel_err(diag, diag_ref) <= TOL, call
        assert np.max(np.abs(prof - prof_ref)) <= TOL * max(1.0, np.max(np.abs(prof_ref))), call


def test_noalloc_statistics_at_the_largest_accepted_nx():
    """nx = 512 (two x blocks of the first pass, the most scratch) with ny*nz = 128
    rows, more than the 64 row blocks, so every block sums several rows."""
    cfg = pydugks.make_config(nx=512, ny=16, nz=8, xwidth=512, ywidth=16, zwidth=8, periods_x=0, CFL=0.5,
                              visc=0.02, ambient_fz=1e-5)
    eng = pydugks.Engine(cfg)
    eng.set_state(seeded_state(512, 16, 8, seed=21))
    stream = torch.cuda.current_stream().cuda_stream
    eng.set_stream(stream)
    nx = eng.nx
    out = torch.full((12 + 9 * nx + 1,), float("nan"), dtype=torch.float64, device="cuda")
    for call in range(2):
        eng.run(1 + 3 * call, 3)
        diag_ref, prof_ref = eng.stats_values()
        _noalloc(eng, out, stream)
        torch.cuda.synchronize()
        o = out.cpu().numpy()
        diag, prof, bad = o[:12], o[12:12 + 9 * nx].reshape(nx, 9), o[12 + 9 * nx]
        assert bad == 0
        assert rel_err(diag, diag_ref) <= TOL, call
        assert np.max(np.abs(prof - prof_ref)) <= TOL * max(1.0, np.max(np.abs(prof_ref))), call
    eng.close()


def test_noalloc_rejects_grids_beyond_its_maximum():
    eng, _, _ = make_pair("walls", "fp64", seed=5)
    out = torch.zeros(16, dtype=torch.float64, device="cuda")
    rc = pydugks.lib().dg_stats_values_noalloc(
        ctypes.c_void_p(eng.device_ptr(pydugks.DG_BUF_F)), 513, 1, 1, 1024, 1 << 20, 0.1, 0.0, 0.0, 0.0,
        ctypes.c_void_p(out.data_ptr()), None)
    assert rc == pydugks.DG_ERR_SHAPE
    assert "maximum" in pydugks.lib().dg_noalloc_last_error().decode()
