"""Gradient with respect to a spatially varying body-force field (an
extension: the reference has a per-cell force only in stage (a) and uses the
ambient force on the faces; with a field the face force is the mean of the
two cells).

Per step: <(S(f, phi+e d) - S(f, phi-e d)) / 2e, lam> == <d, dJ/dphi> for
random d, lam, and the state transpose identity with the field set, FP64.
Through the binomial-checkpointed run (dugks_autograd.DugksObjectiveRun):
gradient of the time-averaged wall shear stress with respect to the field and
to the initial state against central differences (relative <= 1e-5), and
independence of the gradient from the number of stored states.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

import pydugks  # noqa: E402
import dugks_autograd as da  # noqa: E402
from _cases import CASES  # noqa: E402
from seeded import seeded_state, uniform_sym  # noqa: E402

FIELD_CASES = [("walls", 2), ("periodic", 0), ("stretched", 2), ("walls", 1)]


def _engine(case, precision="fp64"):
    kw = dict(CASES[case])
    kw["precision"] = precision
    return pydugks.Engine(pydugks.make_config(**kw))


def _field(eng, seed, scale=2e-5):
    return uniform_sym(seed, eng.nx * eng.ny * eng.nz, 3).reshape(eng.nz, eng.ny, eng.nx) * scale


def _richardson(fn, e):
    """O(e^4) central difference of fn at 0."""
    c = lambda h: (fn(h) - fn(-h)) / (2 * h)  # noqa: E731
    return (4 * c(e / 2) - c(e)) / 3


@pytest.mark.parametrize("case,axis", FIELD_CASES)
def test_field_adjoint_is_the_transpose_of_the_step(case, axis):
    eng = _engine(case)
    f = seeded_state(eng.nx, eng.ny, eng.nz, seed=31)
    phi = _field(eng, 4)
    dphi_dir = _field(eng, 5, scale=1.0)
    lam = uniform_sym(6, f.size, 2).reshape(f.shape)

    def lam_dot_step(h):
        eng.set_force_field(axis, phi + h * dphi_dir)
        eng.set_state(f)
        eng.run(2, 1)
        return float(np.sum(eng.get_state() * lam))

    lhs = _richardson(lam_dot_step, 1e-4)
    eng.set_force_field(axis, phi)
    eng.field_grad(reset=True)
    ft = da.from_dump_order(eng, torch.from_numpy(f).cuda())
    lt = da.from_dump_order(eng, torch.from_numpy(lam).cuda())
    out = torch.zeros_like(lt)
    eng.set_stream(torch.cuda.current_stream().cuda_stream)
    eng.adjoint_step(2, ft.data_ptr(), lt.data_ptr(), out.data_ptr())
    torch.cuda.synchronize()
    g = eng.field_grad(reset=True)
    rhs = float(np.sum(g * dphi_dir))
    rel = abs(lhs - rhs) / abs(rhs)
    print(f"{case} axis {axis}: <dS/dphi d, lam> = {lhs:.12e}, <d, dJ/dphi> = {rhs:.12e}, rel {rel:.2e}")
    assert rel < 1e-7

    # state transpose identity with the field set
    d = uniform_sym(7, f.size, 1).reshape(f.shape) * 1e-2 * f

    def lam_dot_state(h):
        eng.set_state(f + h * d)
        eng.run(2, 1)
        return float(np.sum(eng.get_state() * lam))

    lhs = _richardson(lam_dot_state, 1e-4)
    rhs = float(np.sum(d * da.to_dump_order(eng, out).cpu().numpy()))
    rel = abs(lhs - rhs) / abs(rhs)
    print(f"{case} axis {axis}: state transpose rel {rel:.2e}")
    assert rel < 1e-7


def _channel(precision="fp64"):
    kw = dict(CASES["stretched"])
    kw["precision"] = precision
    eng = pydugks.Engine(pydugks.make_config(**kw))
    f0 = seeded_state(eng.nx, eng.ny, eng.nz, seed=41)
    return eng, torch.from_numpy(f0).cuda()


def test_wall_shear_gradient_matches_finite_differences():
    eng, f0d = _channel()
    obj = da.WallShear(eng, axis=2)
    nsteps = 24
    phi0 = torch.from_numpy(_field(eng, 8)).cuda()

    def J(phi, f0=f0d, snaps=5):
        t0 = da.from_dump_order(eng, f0)
        _, j = da.run_objective(t0, phi, eng, 1, nsteps, obj, snaps=snaps, axis=2)
        return j

    phi = phi0.clone().requires_grad_(True)
    f0 = f0d.clone().requires_grad_(True)
    Jv = J(phi, f0)
    gphi, gf0 = torch.autograd.grad(Jv, [phi, f0])
    for k in range(2):
        d = torch.from_numpy(_field(eng, 50 + k, scale=1.0)).cuda()
        with torch.no_grad():
            fd = _richardson(lambda h: float(J(phi0 + h * d)), 1e-4)
        ad = float((gphi * d).sum())
        rel = abs(ad - fd) / abs(fd)
        print(f"field direction {k}: adjoint {ad:.10e} fd {fd:.10e} rel {rel:.2e}")
        assert rel < 1e-5
    d = torch.from_numpy(uniform_sym(60, f0d.numel(), 0).reshape(f0d.shape)).cuda() * 1e-2 * f0d
    with torch.no_grad():
        fd = _richardson(lambda h: float(J(phi0, f0d + h * d)), 1e-3)
    ad = float((gf0 * d).sum())
    rel = abs(ad - fd) / abs(fd)
    print(f"initial-state direction: adjoint {ad:.10e} fd {fd:.10e} rel {rel:.2e}")
    assert rel < 1e-5


def test_gradient_does_not_depend_on_the_checkpoint_count():
    eng, f0d = _channel()
    obj = da.WallShear(eng, axis=2)
    phi0 = torch.from_numpy(_field(eng, 9)).cuda()
    grads = []
    for snaps in (0, 3, 40):
        phi = phi0.clone().requires_grad_(True)
        t0 = da.from_dump_order(eng, f0d).requires_grad_(True)
        fN, j = da.run_objective(t0, phi, eng, 1, 17, obj, snaps=snaps, axis=2)
        loss = j + 1e-3 * da.kinetic_energy(eng, fN)
        grads.append(torch.autograd.grad(loss, [phi, t0]))
    for g in grads[1:]:
        assert torch.equal(g[0], grads[0][0])
        assert torch.equal(g[1], grads[0][1])


def test_wall_shear_fast_source_equals_autograd_source():
    eng, f0d = _channel()
    obj = da.WallShear(eng, axis=2)
    plain = lambda s, p: obj(s, p)  # noqa: E731  (no `accumulate`: torch autograd path)

    class PerStep:  # `accumulate` per state, without the prepared constant source
        __call__ = staticmethod(obj.__call__)
        accumulate = staticmethod(obj.accumulate)

    phi0 = torch.from_numpy(_field(eng, 10)).cuda()
    out = []
    for o in (obj, PerStep(), plain):
        phi = phi0.clone().requires_grad_(True)
        t0 = da.from_dump_order(eng, f0d).requires_grad_(True)
        _, j = da.run_objective(t0, phi, eng, 1, 9, o, snaps=4, axis=2)
        out.append(torch.autograd.grad(j, [phi, t0]))
    for got in out[:2]:
        for a, b in zip(got, out[2]):
            assert float((a - b).abs().max()) <= 1e-12 * float(b.abs().max())


@pytest.mark.parametrize("case,axis", [("walls", 2), ("periodic", 0), ("stretched", 2), ("aniso", None)])
def test_fp32_adjoint_matches_fp64(case, axis):
    """The FP32 adjoint (TMA-staged face kernel) against the FP64 one on the same state and field."""
    outs = []
    for prec in ("fp64", "fp32"):
        eng = _engine(case, prec)
        f = seeded_state(eng.nx, eng.ny, eng.nz, seed=33)
        lam = uniform_sym(8, f.size, 3).reshape(f.shape)
        if axis is not None:
            eng.set_force_field(axis, _field(eng, 11))
            eng.field_grad(reset=True)
        dt = torch.float64 if prec == "fp64" else torch.float32
        ft = da.from_dump_order(eng, torch.from_numpy(f).cuda().to(dt))
        lt = da.from_dump_order(eng, torch.from_numpy(lam).cuda().to(dt))
        out = torch.zeros_like(lt)
        eng.set_stream(torch.cuda.current_stream().cuda_stream)
        eng.adjoint_step(2, ft.data_ptr(), lt.data_ptr(), out.data_ptr())
        torch.cuda.synchronize()
        g = eng.field_grad(reset=True) if axis is not None else None
        outs.append((da.to_dump_order(eng, out).double().cpu().numpy(), g))
        eng.close()
    (a64, g64), (a32, g32) = outs
    rel = float(np.max(np.abs(a32 - a64)) / np.max(np.abs(a64)))
    print(f"{case}: fp32 vs fp64 adjoint rel {rel:.2e}")
    assert rel < 1e-5
    if axis is not None:
        relg = float(np.max(np.abs(g32 - g64)) / np.max(np.abs(g64)))
        print(f"{case}: fp32 vs fp64 field gradient rel {relg:.2e}")
        assert relg < 1e-4
