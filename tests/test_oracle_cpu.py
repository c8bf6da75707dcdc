"""The oracle (CPU restatement of the reference step) against analytic
properties of DUGKS and against the reference's own outputs (golden
fixtures made by running the reference kernels; see tests/golden/)."""
import glob
import os

import numpy as np
import pytest

import pyoracle
from seeded import rel_err, seeded_state

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def laminar(nx=16, ny=4, nz=4, dtype=np.float64, **kw):
    # examples/laminar/config.txt scaled down: walls in x, force along z, CFL 0.7, visc 0.166
    dx = float(np.float32(nx)) / nx
    dt = float(np.float32(0.7)) * dx / np.sqrt(2.0)
    return pyoracle.Oracle(nx, ny, nz, dx, 1.0, 1.0, dt, float(np.float32(0.166)),
                           F=(0.0, 0.0, float(np.float32(3.2421875e-5))), periodic_x=0, dtype=dtype, **kw)


def test_coefficients_follow_init_dugks():
    o = laminar()
    c = o.coefficients()
    visc, RT, hdt = c[0], c[1], c[2]
    tau = visc / RT
    dt = 2 * hdt
    assert c[3] == (3. * tau * hdt) / (2. * tau + dt)
    assert c[4] == (2. * tau - hdt) / (2. * tau + dt)
    assert c[6] == tau * hdt / (2. * tau + hdt)
    assert np.float32(visc) == np.float32(0.166) and visc == float(np.float32(0.166))


def test_mass_conserved_walls_and_periodic():
    o = laminar()
    f = o.init(1)
    m0 = f[1:-1, 1:-1, 1:-1].sum()
    o.run(f, 1, 100)
    assert abs(f[1:-1, 1:-1, 1:-1].sum() - m0) / m0 < 1e-13
    p = pyoracle.Oracle(8, 8, 8, 1.0, 1.0, 1.0, 0.5 / np.sqrt(2), 0.01, periodic_x=1)
    g = pyoracle.to_ghosted(seeded_state(8, 8, 8, seed=2))
    m0 = g.sum()
    p.run(g, 1, 50)
    assert abs(pyoracle.interior(g).sum() - m0) / m0 < 1e-13


def test_poiseuille_steady_state():
    """Body-force-driven channel between bounce-back walls relaxes to the
    parabola u = F x (W - x) / (2 nu) (cf. examples/laminar/velprof.plt:21)."""
    nx = 16
    o = laminar(nx=nx, ny=2, nz=2)
    f = o.init(1)
    o.run(f, 1, 6000)
    rho, ux, uy, uz = o.macro(f)
    c = o.cfg
    x = (np.arange(nx) + 0.5) * c.dx
    W = nx * c.dx
    exact = c.Fz * x * (W - x) / (2 * c.visc)
    prof = uz[2, 2, 1:-1]
    assert np.max(np.abs(prof - exact)) / exact.max() < 0.02
    assert np.allclose(prof, prof[::-1], rtol=1e-10)


def test_fp32_tracks_fp64():
    a = laminar()
    b = laminar(dtype=np.float32)
    fa = a.init(1)
    fb = b.init(1)
    a.run(fa, 1, 100)
    b.run(fb, 1, 100)
    assert rel_err(fb, fa) < 2e-5


def test_stretched_uniform_limit():
    """The Fortran-channel formulas on a uniform mesh equal the CUDA-C ones."""
    nx, ny, nz = 12, 4, 4
    dx = 1.0
    xc = (np.arange(nx + 2) - 0.5) * dx
    dxx = np.full(nx + 2, dx)
    dt = 0.5 * dx / np.sqrt(2.0)
    u = pyoracle.Oracle(nx, ny, nz, dx, 1.0, 1.0, dt, 0.05, F=(0, 0, 1e-5))
    s = pyoracle.Oracle(nx, ny, nz, dx, 1.0, 1.0, dt, 0.05, F=(0, 0, 1e-5), xc=xc, dxx=dxx)
    f0 = pyoracle.to_ghosted(seeded_state(nx, ny, nz, seed=7))
    f1 = f0.copy()
    u.run(f0, 1, 10)
    s.run(f1, 1, 10)
    assert rel_err(f1, f0) < 1e-14


def test_fortran_face_force_differs_only_by_force_terms():
    nx, ny, nz = 12, 4, 4
    xc = (np.arange(nx + 2) - 0.5)
    dxx = np.ones(nx + 2)
    dt = 0.5 / np.sqrt(2.0)
    a = pyoracle.Oracle(nx, ny, nz, 1.0, 1.0, 1.0, dt, 0.05, F=(0, 1e-6, 0), xc=xc, dxx=dxx, face_force=0)
    b = pyoracle.Oracle(nx, ny, nz, 1.0, 1.0, 1.0, dt, 0.05, F=(0, 1e-6, 0), xc=xc, dxx=dxx, face_force=1)
    f0 = pyoracle.to_ghosted(seeded_state(nx, ny, nz, seed=8))
    f1 = f0.copy()
    a.run(f0, 1, 5)
    b.run(f1, 1, 5)
    d = rel_err(f1, f0)
    assert 1e-12 < d < 1e-5
    # without a force the two treatments coincide
    a = pyoracle.Oracle(nx, ny, nz, 1.0, 1.0, 1.0, dt, 0.05, xc=xc, dxx=dxx, face_force=0)
    b = pyoracle.Oracle(nx, ny, nz, 1.0, 1.0, 1.0, dt, 0.05, xc=xc, dxx=dxx, face_force=1)
    f0 = pyoracle.to_ghosted(seeded_state(nx, ny, nz, seed=8))
    f1 = f0.copy()
    a.run(f0, 1, 5)
    b.run(f1, 1, 5)
    assert rel_err(f1, f0) < 1e-14


def test_gradient_and_trilinear_agree_on_smooth_flow():
    o_t = laminar()
    o_g = laminar(recon=1)
    ft = o_t.init(1)
    fg = o_g.init(1)
    o_t.run(ft, 1, 100)
    o_g.run(fg, 1, 100)
    assert rel_err(fg, ft) < 1e-9


def test_stats_formulas():
    o = laminar(nx=8, ny=3, nz=2)
    f = pyoracle.to_ghosted(seeded_state(8, 3, 2, seed=9))
    diag, prof = o.stats(f)
    rho, ux, uy, uz = [a[1:-1, 1:-1, 1:-1] for a in o.macro(f)]
    assert np.isclose(diag[0], rho.mean(), rtol=1e-14)
    assert np.isclose(diag[11], uz.max())
    assert np.allclose(prof[:, 0], ux.mean(axis=(0, 1)), rtol=1e-13)
    assert np.allclose(prof[:, 3], (ux * uz).mean(axis=(0, 1)) - ux.mean(axis=(0, 1)) * uz.mean(axis=(0, 1)),
                       atol=1e-16)


GOLDEN_FILES = sorted(glob.glob(os.path.join(GOLDEN, "ref_*.npz")))


@pytest.mark.skipif(not GOLDEN_FILES, reason="no reference golden fixtures committed")
@pytest.mark.parametrize("path", GOLDEN_FILES, ids=[os.path.basename(p) for p in GOLDEN_FILES])
def test_oracle_matches_reference_golden(path):
    """Outputs of the reference's own kernels on seeded inputs
    (tests/golden/make_golden.py); the oracle must reproduce them."""
    z = np.load(path)
    m = {k: z[k].item() if z[k].shape == () else z[k] for k in z.files}
    nx, ny, nz = int(m["nx"]), int(m["ny"]), int(m["nz"])
    dtype = np.float64 if int(m["prec"]) == 0 else np.float32
    o = pyoracle.Oracle(nx, ny, nz, float(m["dx"]), float(m["dy"]), float(m["dz"]), float(m["dt"]),
                        float(m["visc"]), F=tuple(m["F"]), periodic_x=int(m["periodic_x"]),
                        xwidth=float(m["xwidth"]), ywidth=float(m["ywidth"]), zwidth=float(m["zwidth"]),
                        recon=int(m["recon"]), perturb=int(m["perturb"]), dtype=dtype)
    f = pyoracle.to_ghosted(seeded_state(nx, ny, nz, seed=int(m["seed"])), dtype=dtype)
    o.run(f, 1, int(m["nsteps"]))
    err = rel_err(pyoracle.interior(f), m["f_out"])
    tol = 1e-13 if dtype == np.float64 else 2e-6
    assert err <= tol, err


def test_stretched_gradient_reconstruction_reduces_to_the_uniform_one(tmp_path):
    """recon=gradient on a stretched mesh whose faces are evenly spaced (a mesh
    file) equals the reference's uniform calc_fx rule to rounding."""
    import pydugks
    from seeded import seeded_state
    kw = dict(nx=12, ny=5, nz=4, xwidth=12, ywidth=5, zwidth=4, periods_x=0, CFL=0.5, visc=0.02, ambient_fz=1e-5,
              recon="gradient")
    with open(tmp_path / "mesh.txt", "w") as fh:
        fh.write("\n".join(repr(float(v)) for v in np.arange(13.0)) + "\n")
    uni = pyoracle.Oracle.from_config(pydugks.make_config(**kw))
    st = pyoracle.Oracle.from_config(pydugks.make_config(mesh="file", mesh_file="mesh.txt", **kw),
                                     workdir=str(tmp_path))
    assert st.cfg.mesh == 1 and st.cfg.recon == 1 and uni.cfg.mesh == 0
    f0 = pyoracle.to_ghosted(seeded_state(12, 5, 4, seed=41))
    a, b = f0.copy(), f0.copy()
    uni.run(a, 1, 10)
    st.run(b, 1, 10)
    err = float(np.max(np.abs(a - b)) / np.max(np.abs(a)))
    print(f"stretched rule on a uniform mesh vs calc_fx: {err:.2e}")
    assert err <= 1e-13
