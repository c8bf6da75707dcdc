"""config.txt texts of the benchmark workloads (pure Python; loads no library).

`make_config` writes the reference's keys (src/numerics.cu:70-99,
src/parallel.cu:95-97, src/cuda.cu:17) with defaults from
examples/laminar/config.txt, plus any extension keys of this engine.  The
workload builders give the channel, laminar-channel and Taylor-Green
configurations in the reference orientation (walls on the x faces, force
along z).  Used by the Python binding, the bench and the tests alike, so that
a run without the engine library (the CPU reference arm of the bench) sets up
the same workload.
"""
import math

# Keys read by the reference (src/numerics.cu:70-99, src/parallel.cu:95-97,
# src/cuda.cu:17), in the order of examples/laminar/config.txt.
REFERENCE_KEYS = ("case", "xwidth", "ywidth", "zwidth", "nx", "ny", "nz", "restart", "nrestart", "perturb",
                  "istep0", "nsteps", "noutput3", "noutput2", "ndump", "CFL", "visc", "ambient_fx",
                  "ambient_fy", "ambient_fz", "periods_x", "periods_y", "periods_z", "gpusPerThread")


def make_config(**kw):
    """Reference-format config.txt text; every reference key gets a default.

    Extension keys of this engine (precision, mesh, mesh_alpha, mesh_file,
    recon, ub, re_tau, seed, ...) are appended when given."""
    d = dict(case="channel", xwidth=64, ywidth=32, zwidth=32, nx=64, ny=32, nz=32, restart=0, nrestart=0,
             perturb=0, istep0=1, nsteps=100, noutput3=10000000, noutput2=5000, ndump=100000, CFL=0.7,
             visc=0.166, ambient_fx=0.0, ambient_fy=0.0, ambient_fz=3.2421875e-5, periods_x=0, periods_y=1,
             periods_z=1, gpusPerThread=8)
    d.update(kw)
    lines = ["#####################"]
    for k in REFERENCE_KEYS:
        lines.append(f"{k}={d.pop(k)}")
    for k, v in d.items():
        lines.append(f"{k}={v}")
    return "\n".join(lines) + "\n"


def tanh_alpha_for_first_face(nx, L, x1):
    """alpha of the tanh mesh (src/fortran/channel/run/mesh.py:21-25) whose first
    face lies at x1 from the wall (bisection; the first face moves towards the
    wall as alpha grows)."""
    lo, hi = 1e-9, 1 - 1e-12
    eta = -1.0 + 2.0 / nx
    for _ in range(200):
        a = 0.5 * (lo + hi)
        xf1 = L / (2 * a) * math.tanh(eta * 0.5 * (math.log(1 + a) - math.log(1 - a))) + 0.5 * L
        if xf1 > x1:
            lo = a
        else:
            hi = a
    return 0.5 * (lo + hi)


def channel_config(nx=128, ny=128, nz=256, precision="fp64", re_tau=180.0, ub=0.1, yplus1=0.5, cfl=0.5,
                   seed=0, **extra):
    """Turbulent channel at Re_tau in the reference orientation: walls on the
    x faces (tanh-stretched, nx cells across 2H = xwidth = nx), spanwise y,
    streamwise z with the body force.  Domain 2H x (4/3)pi H x 4 pi H.
    nu from the bulk velocity ub through Dean's correlation
    Re_tau = 0.09 Re_b^0.88 (Re_b = 2 H ub / nu); u_tau = Re_tau nu / H;
    F = u_tau^2 / H; the mesh alpha puts the first cell centre at y+ = yplus1.
    Initial state: case=channel_turb (laminar profile + seeded perturbations
    of +-10% ub + near-wall streaks of 5% ub)."""
    H = nx / 2.0
    re_b = (re_tau / 0.09) ** (1.0 / 0.88)
    nu = 2 * H * ub / re_b
    utau = re_tau * nu / H
    F = utau * utau / H
    alpha = tanh_alpha_for_first_face(nx, 2 * H, 2 * yplus1 * H / re_tau)
    kw = dict(case="channel_turb", nx=nx, ny=ny, nz=nz, xwidth=2 * H, ywidth=round(4.0 / 3.0 * math.pi * H, 4),
              zwidth=round(4.0 * math.pi * H, 4), periods_x=0, CFL=cfl, visc=f"{nu:.9g}", ambient_fz=f"{F:.9g}",
              mesh="tanh", mesh_alpha=f"{alpha:.15g}", precision=precision, ub=ub, re_tau=re_tau, seed=seed,
              noutput2=1000, ndump=100000, nsteps=50000)
    kw.update(extra)
    return make_config(**kw), dict(nu=nu, utau=utau, F=F, alpha=alpha, re_b=re_b)



def laminar_config(precision="fp64", **extra):
    """Laminar body-force channel 32 (x, periodic) x 64 (y, walls) x 32 (z), in the
    reference orientation 64 (walls) x 32 x 32: u_c = 0.1, Re_c = u_c H / nu = 100
    with H = W/2 = 32 (nu = 0.032), F = 8 nu u_c / W^2 = 6.25e-6, CFL 0.5, f = feq."""
    kw = dict(case="channel", nx=64, ny=32, nz=32, xwidth=64, ywidth=32, zwidth=32, periods_x=0, CFL=0.5,
              visc=0.032, ambient_fz=6.25e-6, precision=precision)
    kw.update(extra)
    return make_config(**kw)


def taylor_green_config(n=64, u0=0.05, re=1600.0, precision="fp64", **extra):
    """3-D Taylor-Green vortex, n^3 periodic cells, amplitude u0 in the velocity and
    the density term (extension key tg_u0), Re = u0 L / nu with L = n / (2 pi)."""
    L = n / (2 * math.pi)
    kw = dict(case="tg_eq", nx=n, ny=n, nz=n, xwidth=n, ywidth=n, zwidth=n, periods_x=1, CFL=0.5,
              visc=f"{u0 * L / re:.9g}", ambient_fz=0.0, tg_u0=u0, precision=precision)
    kw.update(extra)
    return make_config(**kw)
