"""Shared parity-test cases: an engine (C ABI) and the oracle on the same seeded state."""
import numpy as np

import pydugks
import pyoracle
from seeded import seeded_state

# small grids chosen so that no dimension is a multiple of the flux tile
CASES = {
    # walls in x (bounce-back, linear-extrapolation ghosts), force along z: the reference orientation
    "walls": dict(nx=20, ny=6, nz=5, xwidth=20, ywidth=6, zwidth=5, periods_x=0, CFL=0.7, visc=0.166,
                  ambient_fz=3.2421875e-5),
    # fully periodic, force with two components
    "periodic": dict(nx=16, ny=12, nz=10, xwidth=16, ywidth=12, zwidth=10, periods_x=1, CFL=0.5, visc=0.01,
                     ambient_fx=1e-5, ambient_fy=2e-5, ambient_fz=0.0),
    # anisotropic cells, no force
    "aniso": dict(nx=33, ny=7, nz=9, xwidth=33, ywidth=14, zwidth=27, periods_x=0, CFL=0.5, visc=0.05,
                  ambient_fz=0.0),
    # tanh-stretched wall-normal mesh (Fortran channel mesh math), force along z
    "stretched": dict(nx=24, ny=8, nz=6, xwidth=24, ywidth=16, zwidth=12, periods_x=0, CFL=0.5, visc=0.02,
                      ambient_fz=1e-5, mesh="tanh", mesh_alpha=0.85),
    # perturbation forcing in stage (a) (calc_perturb_force)
    "perturb": dict(nx=32, ny=8, nz=6, xwidth=32, ywidth=8, zwidth=6, periods_x=0, CFL=0.5, visc=0.02,
                    ambient_fz=1e-5, perturb=1),
}


def make_pair(name, precision="fp64", seed=1, workdir=".", **over):
    kw = dict(CASES[name])
    kw.update(over)
    kw["precision"] = precision
    cfg = pydugks.make_config(**kw)
    eng = pydugks.Engine(cfg, workdir=workdir)
    dtype = np.float64 if precision == "fp64" else np.float32
    # the oracle is set up from the config text alone (mesh, dt and coefficients
    # restated from the reference), never from the engine's own tables
    orc = pyoracle.Oracle.from_config(cfg, dtype=dtype, workdir=workdir)
    f0 = seeded_state(eng.nx, eng.ny, eng.nz, seed=seed)
    eng.set_state(f0)
    return eng, orc, f0


def run_both(eng, orc, f0, istep0, nsteps, nthreads=0):
    eng.run(istep0, nsteps)
    got = eng.get_state()
    g = pyoracle.to_ghosted(f0, dtype=orc.dtype)
    orc.run(g, istep0, nsteps, nthreads)
    return got, pyoracle.interior(g).astype(np.float64)
