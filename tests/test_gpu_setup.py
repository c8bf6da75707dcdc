"""The engine's set-up against the reference's, computed independently of the
engine: the stretched wall-normal mesh against the reference's own
src/fortran/channel/run/mesh.txt, the time step and coefficients against the
oracle's restatement of src/numerics.cu:62-106 / src/dugks.cu:101-125, and the
initial states of every case against the oracle's generators
(src/dugks.cu:222-281 for tg_eq and channel, the seeded turbulent-channel start
of the benchmark workloads).

Tolerances: mesh centres and widths bit-identical for a mesh file (the same
two operations on the same doubles), 1e-12 absolute for the tanh generator
(libm tanh/log against numpy's); time step and coefficients bit-identical
(1e-13 relative on a tanh mesh, where dt follows the first cell width);
initial states 1e-15 relative (the same double expressions, libm against
libm).
"""
import os

import numpy as np
import pytest

import pydugks
import pyoracle
import workloads
from _cases import CASES
from seeded import rel_err

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _reference_faces():
    return np.loadtxt(os.path.join(GOLDEN, "mesh_tanh_128.txt"))


def _fortran_mesh(xf, xwidth):
    """dugks.cuf:114-121 written out in the test: centres, widths, mirrored ghosts."""
    nx = len(xf) - 1
    xc = np.zeros(nx + 2)
    dxx = np.zeros(nx + 2)
    for i in range(1, nx + 1):
        xc[i] = 0.5 * (xf[i] + xf[i - 1])
        dxx[i] = xf[i] - xf[i - 1]
    xc[0] = -xc[1]
    xc[nx + 1] = 2 * xwidth - xc[nx]
    dxx[0] = dxx[1]
    dxx[nx + 1] = dxx[nx]
    return xc, dxx


def _channel_kw(**over):
    kw = dict(case="channel", nx=128, ny=4, nz=4, xwidth=61.72, ywidth=387.79, zwidth=129.26, periods_x=0,
              CFL=0.5, visc=0.0012, ambient_fz=1e-6)
    kw.update(over)
    return kw


def test_mesh_file_equals_the_reference_mesh(tmp_path):
    """mesh=file on the reference's mesh.txt: centres, widths and both ghosts as dugks.cuf:107-121."""
    xf = _reference_faces()
    with open(tmp_path / "mesh.txt", "w") as fh:
        for v in xf:
            fh.write(repr(float(v)) + "\n")
    cfg = pydugks.make_config(**_channel_kw(mesh="file", mesh_file="mesh.txt"))
    with pydugks.Engine(cfg, workdir=str(tmp_path)) as eng:
        xc, dxx = eng.mesh()
        info = eng.info
    want_xc, want_dxx = _fortran_mesh(xf, 61.72)
    assert np.array_equal(xc, want_xc)
    assert np.array_equal(dxx, want_dxx)
    # dt from the first cell width (dugks.cuf:138, CFL read as the reference reads reals)
    assert info.dt == pyoracle.setup_from_config(cfg, workdir=str(tmp_path))["dt"]


def test_mesh_tanh_matches_the_reference_mesh():
    """mesh=tanh with alpha = 0.85 and L = 61.72 reproduces run/mesh.txt (written by run/mesh.py)."""
    cfg = pydugks.make_config(**_channel_kw(mesh="tanh", mesh_alpha=0.85))
    with pydugks.Engine(cfg) as eng:
        xc, dxx = eng.mesh()
    want_xc, want_dxx = _fortran_mesh(_reference_faces(), 61.72)
    assert np.max(np.abs(xc - want_xc)) <= 1e-12
    assert np.max(np.abs(dxx - want_dxx)) <= 1e-12
    oxc, odxx = pyoracle.setup_from_config(cfg)["xc"], pyoracle.setup_from_config(cfg)["dxx"]
    assert np.max(np.abs(xc - oxc)) <= 1e-12 and np.max(np.abs(dxx - odxx)) <= 1e-12


def _configs():
    out = {name: pydugks.make_config(**kw) for name, kw in CASES.items()}
    out["channel Re_tau=180 256x128x128"] = workloads.channel_config()[0]
    out["channel 192x128x96 fp32"] = workloads.channel_config(nx=128, ny=96, nz=192, precision="fp32")[0]
    out["laminar 32x64x32"] = workloads.laminar_config()
    out["Taylor-Green 64^3"] = workloads.taylor_green_config()
    out["Taylor-Green 64^3 fp32"] = workloads.taylor_green_config(precision="fp32")
    return out


@pytest.mark.parametrize("name", sorted(_configs()))
def test_time_step_and_coefficients_equal_the_oracle(name):
    cfg = _configs()[name]
    dtype = np.float32 if "precision=fp32" in cfg else np.float64
    orc = pyoracle.Oracle.from_config(cfg, dtype=dtype)
    # on a tanh mesh dt comes from the first cell width, which libm's tanh and
    # numpy's give to the last few bits (1e-13 relative); otherwise bit-identical
    rtol = 1e-13 if orc.setup["xc"] is not None else 0.0
    with pydugks.Engine(cfg) as eng:
        info = eng.info
        for key in ("dx", "dy", "dz", "dt"):
            assert abs(getattr(info, key) - orc.setup[key]) <= rtol * abs(orc.setup[key]), key
        coef = orc.coefficients()  # visc RT hdt bw0 bw1 bw2 fw0 fw1 fw2 dx dy dz dt
        for key, idx in (("bw0", 3), ("bw1", 4), ("bw2", 5), ("fw0", 6), ("fw1", 7), ("fw2", 8)):
            assert abs(getattr(info, key) - coef[idx]) <= rtol * abs(coef[idx]), key
        if orc.setup["xc"] is not None:
            xc, dxx = eng.mesh()
            assert np.max(np.abs(xc - orc.setup["xc"])) <= 1e-12
            assert np.max(np.abs(dxx - orc.setup["dxx"])) <= 1e-12


@pytest.mark.parametrize("cfg_name,kw", [
    ("tg_eq u0=0.1 (reference)", dict(case="tg_eq", nx=16, ny=12, nz=10, xwidth=16, ywidth=12, zwidth=10,
                                      periods_x=1, ambient_fz=0.0)),
    ("tg_eq u0=0.05", dict(case="tg_eq", nx=16, ny=12, nz=10, xwidth=16, ywidth=12, zwidth=10, periods_x=1,
                           ambient_fz=0.0, tg_u0=0.05)),
    ("channel", dict(case="channel", nx=20, ny=6, nz=5, xwidth=20, ywidth=6, zwidth=5)),
    ("channel_turb tanh", dict(case="channel_turb", nx=24, ny=8, nz=10, xwidth=24, ywidth=16, zwidth=12,
                               mesh="tanh", mesh_alpha=0.9, CFL=0.5, visc=0.01, ambient_fz=1e-5, seed=3)),
    ("channel_turb uniform", dict(case="channel_turb", nx=20, ny=6, nz=5, xwidth=20, ywidth=6, zwidth=5,
                                  ambient_fz=1e-5, seed=0, ub=0.05, streak_m=2)),
])
def test_initial_state_equals_the_oracle(cfg_name, kw):
    cfg = pydugks.make_config(**kw)
    orc = pyoracle.Oracle.from_config(cfg)
    with pydugks.Engine(cfg) as eng:
        got = eng.get_state()
    want = orc.initial_state()
    err = rel_err(got, want)
    print(f"{cfg_name}: initial state rel err {err:.2e}")
    assert err <= 1e-15
    if cfg_name.startswith("tg_eq u0=0.1") or cfg_name == "channel":
        # the reference-literal restatement of src/dugks.cu:222-281 (oracle_init, fixed 0.1)
        ref = pyoracle.interior(orc.init(0 if kw["case"] == "tg_eq" else 1))
        assert rel_err(got, ref) <= 1e-15


def test_tg_amplitude_scales_velocity_and_density():
    """tg_u0 = 0.05 replaces the reference's 0.1 in u and in the density term (rho - 1 ~ u0^2)."""
    base = dict(case="tg_eq", nx=16, ny=16, nz=16, xwidth=16, ywidth=16, zwidth=16, periods_x=1, ambient_fz=0.0)
    states = {}
    for u0 in (0.1, 0.05):
        with pydugks.Engine(pydugks.make_config(tg_u0=u0, **base)) as eng:
            f = eng.get_state()
        rho = f.sum(-1)
        jx = (f * np.array([0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0])).sum(-1)
        states[u0] = (rho - 1.0, jx / rho)
    assert np.allclose(states[0.05][0], states[0.1][0] / 4, rtol=1e-12, atol=1e-14)
    assert np.allclose(states[0.05][1], states[0.1][1] / 2, rtol=1e-12, atol=1e-14)
