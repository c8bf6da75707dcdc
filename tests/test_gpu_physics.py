"""Analytic checks of the engine's step (the reference validates by plots only,
examples/laminar/velprof.plt:21)."""
import numpy as np
import pytest

import pydugks

pytestmark = pytest.mark.gpu


def test_laminar_channel_startup_matches_the_transient_poiseuille_series():
    """Body-force-driven channel from rest, 64 cells between bounce-back walls,
    u_c = 0.1, Re_c = 100 (nu = 0.032), CFL 0.5, 20000 steps: the streamwise
    velocity follows u(x,t) = u_ss(x) - sum_{n odd} 32 u_c/(n pi)^3
    sin(n pi x/W) exp(-nu (n pi/W)^2 t)."""
    kw = dict(nx=64, ny=4, nz=4, xwidth=64, ywidth=4, zwidth=4, periods_x=0, CFL=0.5, visc=0.032,
              ambient_fz=6.25e-6)
    eng = pydugks.Engine(pydugks.make_config(**kw))
    from seeded import W as wts
    eng.set_state(np.ascontiguousarray(np.broadcast_to(wts, (4, 4, 64, 19))))
    nsteps = 20000
    eng.run(1, nsteps)
    rho, ux, uy, uz = eng.copy_vel()
    prof = uz[2, 2, 1:-1]
    info = eng.info
    t = nsteps * info.dt
    nu, F, Wd = info.visc, info.ambient[2], 64.0
    x = (np.arange(64) + 0.5) * info.dx
    uc = F * Wd * Wd / (8 * nu)
    u = F * x * (Wd - x) / (2 * nu)
    for n in range(1, 400, 2):
        u -= 32 * uc / (n * np.pi) ** 3 * np.sin(n * np.pi * x / Wd) * np.exp(-nu * (n * np.pi / Wd) ** 2 * t)
    err = np.max(np.abs(prof - u)) / uc
    print(f"transient Poiseuille at t={t:.1f}: max |u - series| / u_c = {err:.3e}, centre {prof[31]:.6f} vs {u[31]:.6f}")
    assert err < 5e-3
    assert np.allclose(prof, prof[::-1], rtol=1e-10, atol=1e-14)
