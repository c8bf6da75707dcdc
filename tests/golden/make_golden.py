"""Golden fixtures from the reference's own kernels.

Runs the reference's unmodified CUDA-C step kernels (oracle/_ref/*.cubin,
launched by oracle/ref_runner.cpp in dugks_step's order) on seeded inputs
(tests/seeded.py) and stores the resulting f-tilde with the parameters the
reference derived (dx, dt, coefficients follow src/numerics.cu:101-105).
The CPU test tests/test_oracle_cpu.py::test_oracle_matches_reference_golden
checks the oracle against them.  Needs a GPU:
    python tests/golden/make_golden.py OUTDIR
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")]
import pyoracle  # noqa: E402
from seeded import seeded_state  # noqa: E402

CASES = [
    # name, grid, widths, CFL, visc, F, periods_x, prec, recon, perturb, seed, nsteps
    ("walls_f64_1", (32, 8, 4), (32, 8, 4), 0.7, 0.166, (0, 0, 3.2421875e-5), 0, 0, 0, 0, 11, 1),
    ("walls_f64_10", (32, 8, 4), (32, 8, 4), 0.7, 0.166, (0, 0, 3.2421875e-5), 0, 0, 0, 0, 11, 10),
    ("periodic_f64_10", (16, 16, 6), (16, 16, 6), 0.5, 0.01, (1e-5, 2e-5, 0), 1, 0, 0, 0, 12, 10),
    ("aniso_f64_10", (16, 8, 4), (16, 16, 12), 0.5, 0.05, (0, 0, 0), 0, 0, 0, 0, 13, 10),
    ("walls_f32_10", (32, 8, 4), (32, 8, 4), 0.7, 0.166, (0, 0, 3.2421875e-5), 0, 1, 0, 0, 14, 10),
    ("gradient_f64_5", (32, 8, 4), (32, 8, 4), 0.7, 0.166, (0, 0, 3.2421875e-5), 0, 0, 1, 0, 15, 5),
    ("perturb_f64_5", (32, 8, 4), (32, 8, 4), 0.5, 0.02, (0, 0, 1e-5), 0, 0, 0, 1, 16, 5),
]


def main(outdir):
    os.makedirs(outdir, exist_ok=True)
    for name, (nx, ny, nz), (xw, yw, zw), cfl, visc, F, px, prec, recon, perturb, seed, nsteps in CASES:
        R = np.float64 if prec == 0 else np.float32
        f32 = np.float32
        cflr, xwr, ywr, zwr, viscr = (R(f32(v)) for v in (cfl, xw, yw, zw, visc))
        dx, dy, dz = xwr / R(nx), ywr / R(ny), zwr / R(nz)
        dt = cflr * dx / np.sqrt(R(6) * R(1.0 / 3.0))
        Ff = tuple(float(f32(v)) for v in F)
        f = pyoracle.to_ghosted(seeded_state(nx, ny, nz, seed=seed))
        pyoracle.ref_run(f, nx, ny, nz, float(f32(cfl)), float(f32(xw)), float(f32(yw)), float(f32(zw)),
                         float(f32(visc)), Ff, periods=(px, 1, 1), istep0=1, nsteps=nsteps, prec=prec,
                         perturb=perturb, recon=recon)
        out = os.path.join(outdir, f"ref_{name}.npz")
        np.savez(out, nx=nx, ny=ny, nz=nz, dx=float(dx), dy=float(dy), dz=float(dz), dt=float(dt),
                 visc=float(viscr), F=np.array(Ff), periodic_x=px, xwidth=float(xwr), ywidth=float(ywr),
                 zwidth=float(zwr), recon=recon, perturb=perturb, prec=prec, seed=seed, nsteps=nsteps,
                 f_out=pyoracle.interior(f))
        print("wrote", out)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py OUTDIR")
    main(sys.argv[1])
