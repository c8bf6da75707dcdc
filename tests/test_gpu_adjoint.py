"""The hand-written adjoint of the DUGKS step (no counterpart in the
reference) against central finite differences of the forward step.

Per step: <(S(f+e d) - S(f-e d)) / 2e, lam> == <d, adjoint(lam)> for random
d, lam (the transpose identity), FP64, every boundary configuration.
Through a checkpointed multi-step run (dugks_autograd.DugksRun): gradient of
the final kinetic energy with respect to the initial velocity field against
central differences, relative agreement <= 1e-5.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

import pydugks  # noqa: E402
import dugks_autograd as da  # noqa: E402
from _cases import CASES  # noqa: E402
from seeded import seeded_state, uniform_sym  # noqa: E402


def _engine(case, precision="fp64"):
    kw = dict(CASES[case])
    kw["precision"] = precision
    return pydugks.Engine(pydugks.make_config(**kw))


@pytest.mark.parametrize("case", sorted(CASES))
def test_adjoint_is_the_transpose_of_the_step(case):
    eng = _engine(case)
    nx, ny, nz = eng.nx, eng.ny, eng.nz
    f = seeded_state(nx, ny, nz, seed=21)
    d = uniform_sym(5, f.size, 7).reshape(f.shape) * 1e-2 * f
    lam = uniform_sym(6, f.size, 9).reshape(f.shape)
    def cdiff(eps):
        eng.set_state(f + eps * d)
        eng.run(3, 1)
        fp = eng.get_state()
        eng.set_state(f - eps * d)
        eng.run(3, 1)
        fm = eng.get_state()
        return (fp - fm) / (2 * eps)

    # Richardson-extrapolated central difference: O(eps^4) truncation
    e = 1e-4
    jvp = (4 * cdiff(e / 2) - cdiff(e)) / 3
    lhs = float(np.sum(jvp * lam))
    ft = da.from_dump_order(eng, torch.from_numpy(f).cuda())
    lt = da.from_dump_order(eng, torch.from_numpy(lam).cuda())
    out = torch.zeros_like(lt)
    eng.set_stream(torch.cuda.current_stream().cuda_stream)
    eng.adjoint_step(3, ft.data_ptr(), lt.data_ptr(), out.data_ptr())
    torch.cuda.synchronize()
    vjp = da.to_dump_order(eng, out).cpu().numpy()
    rhs = float(np.sum(d * vjp))
    rel = abs(lhs - rhs) / abs(rhs)
    print(f"{case}: <Jd,l>={lhs:.12e} <d,J^T l>={rhs:.12e} rel {rel:.2e}")
    assert rel < 1e-7


def test_adjoint_in_place_equals_out_of_place():
    eng = _engine("walls")
    f = seeded_state(eng.nx, eng.ny, eng.nz, seed=22)
    lam = uniform_sym(3, f.size, 1).reshape(f.shape)
    ft = da.from_dump_order(eng, torch.from_numpy(f).cuda())
    lt = da.from_dump_order(eng, torch.from_numpy(lam).cuda())
    out = torch.zeros_like(lt)
    eng.set_stream(torch.cuda.current_stream().cuda_stream)
    eng.adjoint_step(1, ft.data_ptr(), lt.data_ptr(), out.data_ptr())
    eng.adjoint_step(1, ft.data_ptr(), lt.data_ptr(), lt.data_ptr())
    torch.cuda.synchronize()
    assert torch.equal(out, lt)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_batched_recomputation_and_adjoint_equal_the_step_loops(precision):
    """dg_run_store / dg_adjoint_run against dg_get_state_device + dg_step and
    dg_adjoint_step called one at a time: identical arrays."""
    eng = _engine("stretched", precision)
    eng.set_stream(torch.cuda.current_stream().cuda_stream)
    dt = torch.float64 if precision == "fp64" else torch.float32
    f = da.from_dump_order(eng, torch.from_numpy(seeded_state(eng.nx, eng.ny, eng.nz, seed=23)).cuda().to(dt))
    n = 5
    states = torch.zeros((n, eng.soa_len), dtype=dt, device="cuda")
    stride = states.stride(0) * states.element_size()
    eng.set_state_device(f.data_ptr())
    eng.run_store(4, n, states.data_ptr(), stride)
    ref = torch.zeros_like(states)
    eng.set_state_device(f.data_ptr())
    for s in range(n):
        eng.get_state_device(ref[s].data_ptr())
        if s + 1 < n:
            eng.step(4 + s)
    lam0 = torch.from_numpy(uniform_sym(4, eng.soa_len, 2)).cuda().to(dt)
    lam_a, lam_b = lam0.clone(), lam0.clone()
    eng.adjoint_run(4, n, states.data_ptr(), stride, lam_a.data_ptr())
    for s in reversed(range(n)):
        eng.adjoint_step(4 + s, ref[s].data_ptr(), lam_b.data_ptr(), lam_b.data_ptr())
    torch.cuda.synchronize()
    assert torch.equal(states, ref)
    assert torch.equal(lam_a, lam_b)
    with pytest.raises(RuntimeError):
        eng.adjoint_run(4, n, states.data_ptr(), stride, states[2].data_ptr())  # lam inside the states


def _tg_problem(n=16, u0=0.05):
    L = n
    visc = u0 * (L / (2 * np.pi)) / 1600.0
    cfg = pydugks.make_config(case="tg_eq", nx=n, ny=n, nz=n, xwidth=L, ywidth=L, zwidth=L, periods_x=1,
                              CFL=0.5, visc=f"{visc:.9g}", ambient_fz=0.0)
    eng = pydugks.Engine(cfg)
    f0 = eng.get_state()
    rho0, u = da.macro(torch.from_numpy(f0).permute(3, 0, 1, 2).cuda())
    return eng, rho0, u


def test_gradient_of_kinetic_energy_matches_finite_differences():
    eng, rho0, u0 = _tg_problem()
    nsteps, every = 30, 7

    def J(u):
        f0 = da.feq(rho0, u).permute(1, 2, 3, 0)
        t0 = da.from_dump_order(eng, f0)
        fN = da.run(t0, eng, 1, nsteps, every)
        return da.kinetic_energy(eng, fN)

    u = u0.clone().requires_grad_(True)
    Ju = J(u)
    (g,) = torch.autograd.grad(Ju, u)
    eps = 1e-6
    for k in range(3):
        d = torch.from_numpy(uniform_sym(40 + k, u0.numel(), 0).reshape(u0.shape)).cuda()
        with torch.no_grad():
            fd = (J(u0 + eps * d) - J(u0 - eps * d)) / (2 * eps)
        ad = float((g * d).sum())
        rel = abs(ad - float(fd)) / abs(float(fd))
        print(f"direction {k}: adjoint {ad:.10e} fd {float(fd):.10e} rel {rel:.2e}")
        assert rel < 1e-5


@pytest.mark.parametrize("precision", ["fp64", "fp32", "fp16"])
def test_run_between_equals_the_in_place_run(precision):
    """dg_run_between (steps from one device state into another, the handle's own
    state untouched unless named) against dg_run in place: identical states."""
    eng = _engine("stretched", precision)
    eng.set_stream(torch.cuda.current_stream().cuda_stream)
    eng.set_state(seeded_state(eng.nx, eng.ny, eng.nz, seed=24))
    dt = {"fp64": torch.float64, "fp32": torch.float32, "fp16": torch.float16}[precision]
    src = torch.empty(eng.soa_len, dtype=dt, device="cuda")
    eng.get_state_device(src.data_ptr())
    keep = src.clone()
    dst = torch.full_like(src, float("nan"))
    cells = lambda t: da.to_dump_order(eng, t)  # noqa: E731  (the x pitch padding is never written)
    eng.run_between(5, 4, src.data_ptr(), dst.data_ptr())
    own = torch.empty_like(src)
    eng.get_state_device(own.data_ptr())
    torch.cuda.synchronize()
    assert torch.equal(src, keep) and torch.equal(own, keep)   # neither the source nor the handle's state moved
    eng.run(5, 4)
    eng.get_state_device(own.data_ptr())
    torch.cuda.synchronize()
    assert torch.equal(cells(dst), cells(own))
    eng.run_between(9, 3, dst.data_ptr(), None)                   # into the handle's own state
    eng.run_between(9, 3, dst.data_ptr(), dst.data_ptr())         # in place in dst
    eng.get_state_device(own.data_ptr())
    torch.cuda.synchronize()
    assert torch.equal(cells(dst), cells(own))
    with pytest.raises(pydugks.DugksError):
        eng.run_between(1, 1, src.data_ptr(), eng.device_ptr(pydugks.DG_BUF_FB))
