"""The numpy restatement of the reference's spectral statistics
(src/fortran/dhit/src/stat.f90:5-205, oracle/spectral.py) against closed
forms for a single Fourier mode: u = A sin(k x), v = w = 0 on a periodic box.

  kinetic energy = spectral energy = A^2/4, all of it in shell m;
  dissipation = 2 nu k^2 A^2/4 (k = 2 pi m / L with the reference's pi);
  longitudinal derivative A k cos(k x): skewness 0, flatness
  <cos^4> / (<cos^2>^2 / 3) ... = (3/8)/3 / ((1/2)/3)^2 = 4.5 (the three
  derivative fields are pooled, two of them zero).
"""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "oracle"))
import spectral  # noqa: E402


@pytest.mark.parametrize("shape,m", [((8, 12, 16), 2), ((16, 16, 16), 5)])
def test_single_mode_closed_forms(shape, m):
    nz, ny, nx = shape
    L, nu, A = float(nx), 0.01, 0.03
    x = (np.arange(nx) + 0.5) * L / nx
    k = 2 * np.pi * m / L
    u = np.broadcast_to(A * np.sin(k * x), shape).copy()
    z = np.zeros(shape)
    vals, ett = spectral.stat_te(u, z, z, L, nu)
    kr = 2 * spectral.PI * m / L
    assert vals["te"] == pytest.approx(A * A / 4, rel=1e-12)
    assert vals["etotal"] == pytest.approx(A * A / 4, rel=1e-12)
    assert ett[m] == pytest.approx(A * A / 4, rel=1e-12)
    assert np.sum(np.abs(np.delete(ett, m))) < 1e-20
    assert vals["ediss"] == pytest.approx(2 * nu * kr * kr * A * A / 4, rel=1e-12)
    assert abs(vals["skew"]) < 1e-9
    assert vals["flat"] == pytest.approx(4.5, rel=1e-9)
    assert vals["uprm"] == pytest.approx(np.sqrt(2.0 / 3.0 * A * A / 4), rel=1e-12)
    assert vals["eta"] == pytest.approx((nu ** 3 / vals["ediss"]) ** 0.25, rel=1e-12)


def test_mean_velocity_is_removed():
    rng = np.random.default_rng(3)
    u, v, w = (rng.uniform(-0.01, 0.01, (6, 8, 10)) for _ in range(3))
    a, sa = spectral.stat_te(u, v, w, 10.0, 0.02)
    b, sb = spectral.stat_te(u + 0.05, v - 0.02, w, 10.0, 0.02)
    for key in ("etotal", "ediss", "skew", "flat"):
        assert b[key] == pytest.approx(a[key], rel=1e-10)
    assert np.allclose(sa, sb, rtol=1e-10, atol=1e-30)
    assert b["te"] > a["te"]  # the physical-space energy keeps the mean (stat.f90:60)
