"""Tanh wall-normal mesh of the stretched-mesh channel
(src/fortran/channel/run/mesh.py:21-25, dugks.cuf:107-121)."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def tanh_faces(n, L, alpha):
    eta = -1.0 + 2.0 * np.arange(n + 1) / n
    return L / (2 * alpha) * np.tanh(eta * 0.5 * (np.log(1 + alpha) - np.log(1 - alpha))) + 0.5 * L


def test_formula_matches_reference_mesh_file():
    ref = np.loadtxt(os.path.join(GOLDEN, "mesh_tanh_128.txt"))
    ours = tanh_faces(128, 61.72, 0.85)
    assert np.max(np.abs(ours - ref)) < 1e-12


def test_mesh_is_symmetric_and_clustered():
    xf = tanh_faces(128, 2.0, 0.85)
    d = np.diff(xf)
    assert np.allclose(d, d[::-1], rtol=1e-12)
    assert d[0] < d[64] / 2
