"""The oracle's set-up restatements on the CPU: the tanh wall-normal mesh
(src/fortran/channel/run/mesh.py:21-25, dugks.cuf:107-121) against the
reference's own run/mesh.txt, the config reading rules (src/config.h:17-74,
src/numerics.cu:62-106) and the seeded turbulent-channel start."""
import os

import numpy as np

import pyoracle
import workloads

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_oracle_tanh_faces_match_reference_mesh_file():
    ref = np.loadtxt(os.path.join(GOLDEN, "mesh_tanh_128.txt"))
    ours = pyoracle.tanh_faces(128, 61.72, 0.85)
    assert np.max(np.abs(ours - ref)) < 1e-12


def test_oracle_mesh_from_the_reference_file_has_the_fortran_ghosts():
    xf = np.loadtxt(os.path.join(GOLDEN, "mesh_tanh_128.txt"))
    xc, dxx = pyoracle.mesh_from_faces(xf, 61.72)
    assert xc[0] == -xc[1] and xc[129] == 2 * 61.72 - xc[128]
    assert dxx[0] == dxx[1] and dxx[129] == dxx[128]
    assert np.all(dxx[1:-1] > 0) and abs(dxx[1:-1].sum() - 61.72) < 1e-12
    # symmetric about the channel centre, clustered at the walls
    assert np.allclose(dxx[1:-1], dxx[1:-1][::-1], rtol=1e-12)
    assert dxx[1] < dxx[64] / 2


def test_config_reading_rules():
    kv = pyoracle.parse_config("#####\nnx=12\nnx=99\nCFL=0.7=junk\nno equals sign\nvisc =0.1\n")
    assert kv["nx"] == "12"            # first occurrence wins
    assert kv["CFL"] == "0.7"          # the field after the first '='
    assert "visc " in kv and "visc" not in kv  # no trimming
    assert pyoracle._stof("0.166") == float(np.float32(0.166))
    assert pyoracle._stoi("64abc") == 64


def test_stretched_setup_uses_the_first_cell_for_dt():
    cfg, meta = workloads.channel_config()
    s = pyoracle.setup_from_config(cfg)
    assert s["xc"] is not None
    assert s["dt"] == float(np.float32(0.5)) * s["dxx"][1] / np.sqrt(6 * (1.0 / 3.0))
    # the first cell centre sits at y+ = 0.5 (alpha chosen by bisection)
    utau = meta["utau"]
    assert abs(s["xc"][1] * utau / meta["nu"] - 0.5) < 1e-3


def test_seeded_channel_start_has_its_stated_shape():
    cfg, _ = workloads.channel_config(nx=32, ny=16, nz=24, re_tau=180.0)
    orc = pyoracle.Oracle.from_config(cfg)
    f = orc.initial_state()
    assert f.shape == (24, 16, 32, 19)
    rho = f.sum(-1)
    cz = np.array([0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1])
    w = (f * cz).sum(-1) / rho
    assert np.allclose(rho, 1.0, atol=1e-12)
    xc = orc.setup["xc"][1:-1]
    L = orc.setup["xwidth"]
    lam = 6 * 0.1 * (xc / L) * (1 - xc / L)
    dev = w - lam[None, None, :]
    # +-10 % of the bulk velocity plus streaks of 5 % at most
    assert np.max(np.abs(dev)) <= 0.1 * 0.1 + 0.05 * 0.1 + 1e-12
    assert abs(dev.mean()) < 2e-3
    # deterministic, and another seed gives another start
    assert np.array_equal(f, orc.initial_state())
    other = pyoracle.Oracle.from_config(workloads.channel_config(nx=32, ny=16, nz=24, seed=1)[0]).initial_state()
    assert not np.array_equal(f, other)
