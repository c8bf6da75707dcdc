"""The hand-written adjoint against the FP64 tangent: the gradient of the
final kinetic energy of a Taylor-Green run (tg_eq with u0 = 0.05, periodic
box) with respect to the initial velocity field, from the engine's adjoint
(dugks_autograd.DugksRun with checkpoints and recomputation), paired with
seeded directions d, must equal the directional derivative dJ[d] from the
oracle's tangent-linear model (the oracle's restatement of the reference step
run on dual numbers: exact to rounding, no finite-difference truncation) to
1e-10 relative.  A wall-bounded channel with a force field control is
checked the same way in tests/test_gpu_adjoint_field.py against central
differences."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

import pydugks  # noqa: E402
import pyoracle  # noqa: E402
import workloads  # noqa: E402
import dugks_autograd as da  # noqa: E402
from seeded import CX, CY, CZ, W, uniform_sym  # noqa: E402

TOL = 1e-10


def _dfeq(rho, u, d):
    """Directional derivative of the second-order equilibrium in u along d;
    rho (...), u and d (3, ...) -> (..., 19)."""
    c = np.stack([CX, CY, CZ]).astype(np.float64)
    eu = 3.0 * np.einsum("ap,a...->...p", c, u)
    cd = np.einsum("ap,a...->...p", c, d)
    ud = (u * d).sum(0)[..., None]
    return W * rho[..., None] * (3.0 * cd + 3.0 * eu * cd - 3.0 * ud)


def _dke(f, df):
    """d(0.5 sum |j|^2 / rho) for f, df of shape (..., 19)."""
    rho, drho = f.sum(-1), df.sum(-1)
    j = [(f * c).sum(-1) for c in (CX, CY, CZ)]
    dj = [(df * c).sum(-1) for c in (CX, CY, CZ)]
    jj = sum(a * a for a in j)
    return float(np.sum(sum(a * b for a, b in zip(j, dj)) / rho - 0.5 * jj * drho / rho ** 2))


@pytest.mark.parametrize("n,nsteps,every", [(16, 30, 7), (12, 60, 16)])
def test_adjoint_gradient_equals_the_fp64_tangent(n, nsteps, every):
    cfg = workloads.taylor_green_config(n=n, u0=0.05)
    eng = pydugks.Engine(cfg)
    rho0, u0 = da.macro(torch.from_numpy(eng.get_state()).permute(3, 0, 1, 2).cuda())

    def J(u):
        f0 = da.feq(rho0, u).permute(1, 2, 3, 0)
        fN = da.run(da.from_dump_order(eng, f0), eng, 1, nsteps, every)
        return da.kinetic_energy(eng, fN)

    u = u0.clone().requires_grad_(True)
    (g,) = torch.autograd.grad(J(u), u)
    g = g.cpu().numpy()
    f0 = da.feq(rho0, u0).permute(1, 2, 3, 0).contiguous().cpu().numpy()
    rho_np, u_np = rho0.cpu().numpy(), u0.cpu().numpy()
    orc = pyoracle.Oracle.from_config(cfg)
    for k in range(4):
        d = uniform_sym(70 + k, u_np.size, 0).reshape(u_np.shape)
        f, df = pyoracle.to_ghosted(f0), pyoracle.to_ghosted(_dfeq(rho_np, u_np, d))
        orc.tangent_run(f, df, 1, nsteps)
        tan = _dke(pyoracle.interior(f), pyoracle.interior(df))
        adj = float(np.sum(g * d))
        rel = abs(adj - tan) / abs(tan)
        print(f"n={n} steps={nsteps} direction {k}: adjoint {adj:.15e} tangent {tan:.15e} rel {rel:.2e}")
        assert rel <= TOL
    eng.close()
