"""Spectral statistics of a periodic box (dg_spectral_stats /
dg_output_spectral; the reference's Fortran decaying-turbulence statistics,
src/fortran/dhit/src/stat.f90:5-205) against the numpy restatement
oracle/spectral.py on the same state: relative agreement <= 1e-10 for every
value and shell (FP64 on both sides; the FFTs differ in rounding only).
The FP32 form reads its own state; the files carry the same values in the
reference's formats.
"""
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

import pydugks  # noqa: E402
from seeded import seeded_state  # noqa: E402

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "oracle"))
import spectral  # noqa: E402


def _box(nx=24, ny=20, nz=16, precision="fp64", workdir="."):
    cfg = pydugks.make_config(case="tg_eq", nx=nx, ny=ny, nz=nz, xwidth=nx, ywidth=ny, zwidth=nz, periods_x=1,
                              CFL=0.5, visc=0.004, ambient_fz=0.0, precision=precision)
    return pydugks.Engine(cfg, workdir=workdir)


def _check(eng, f):
    vals, spec = eng.spectral_stats(nbins=2 * eng.nx + 1)
    u, v, w = spectral.velocity(f)
    ref, ett = spectral.stat_te(u, v, w, eng.info.xwidth, eng.info.visc)
    for key in spectral.KEYS:
        if key == "ediss_total":
            assert vals[key] == 0.0
            continue
        rel = abs(vals[key] - ref[key]) / max(abs(ref[key]), 1e-300)
        print(f"{key}: engine {vals[key]:.12e} oracle {ref[key]:.12e} rel {rel:.1e}")
        assert rel <= 1e-10 or (key == "skew" and abs(vals[key] - ref[key]) < 1e-10)
    assert np.allclose(spec, ett[:len(spec)], rtol=1e-10, atol=1e-12 * ett.max())
    return vals, spec


@pytest.mark.parametrize("shape", [(24, 20, 16), (32, 32, 32)])
def test_spectral_statistics_match_the_oracle(shape):
    eng = _box(*shape)
    f = seeded_state(*shape, seed=17, umax=0.05, eps=0.0)
    eng.set_state(f)
    _check(eng, eng.get_state())


def test_taylor_green_start():
    """The tg_eq start: one Fourier mode per component (shell sqrt(3) -> 2)."""
    eng = _box(32, 32, 32)
    vals, spec = _check(eng, eng.get_state())
    assert np.argmax(spec) == 2
    assert spec[2] / spec.sum() > 0.99


def test_fp32_form_reads_its_own_state():
    eng = _box(24, 20, 16, precision="fp32")
    eng.set_state(seeded_state(24, 20, 16, seed=18, umax=0.05, eps=0.0))
    _check(eng, eng.get_state())


def test_output_files_carry_the_values(tmp_path):
    eng = _box(24, 20, 16, workdir=str(tmp_path))
    eng.set_state(seeded_state(24, 20, 16, seed=19, umax=0.05, eps=0.0))
    vals, spec = eng.spectral_stats(nbins=25)
    eng.output_spectral(50)
    eng.output_spectral(100)
    ke = (tmp_path / "KE.dat").read_text().splitlines()
    assert len(ke) == 2 and ke[0].split()[0] == "000050"
    assert float(ke[0].split()[2]) == pytest.approx(vals["te"], rel=1e-9)
    st = (tmp_path / "stat_te.dat").read_text().splitlines()
    assert int(st[1].split()[0]) == 100 and float(st[1].split()[2]) == pytest.approx(vals["te"], rel=1e-6)
    sp = (tmp_path / "stat_te_spectral.dat").read_text().splitlines()[0].split()
    assert len(sp) == 13
    got = [float(x) for x in sp[2:]]
    want = [vals[k] for k in ("etotal", "ediss", "ediss_total", "eta", "vk", "tk", "uprm", "tmse", "retms", "xl",
                              "kmxeta")]
    assert np.allclose(got, want, rtol=1e-6, atol=0)
    sf = (tmp_path / "skew-flat.dat").read_text().splitlines()[0].split()
    assert float(sf[3]) == pytest.approx(vals["flat"], rel=1e-6)
    lines = (tmp_path / "spe000000050.dat").read_text().splitlines()
    assert len(lines) == 25 and lines[0].split()[0] == "0"
    assert np.allclose([float(l.split()[1]) for l in lines], spec, rtol=1e-6, atol=1e-300)


def test_walls_are_refused():
    cfg = pydugks.make_config(nx=16, ny=8, nz=8, xwidth=16, ywidth=8, zwidth=8, periods_x=0)
    eng = pydugks.Engine(cfg)
    with pytest.raises(pydugks.DugksError) as e:
        eng.spectral_stats()
    assert e.value.code == pydugks.DG_ERR_UNSUPPORTED
