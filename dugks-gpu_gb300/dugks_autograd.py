"""PyTorch verification harness for the hand-written adjoint.

`DugksRun.apply(f0, engine, istep0, nsteps, every)` advances a state tensor
(the engine's SoA layout, 19*pop_stride elements on the engine's GPU) by
`nsteps` DUGKS steps through the C ABI; its backward runs the hand-written
adjoint kernels (dg_adjoint_step) with two-level checkpointing: the forward
keeps a copy of the state every `every` steps, the backward recomputes each
segment forward once and walks it back with the adjoint.  Memory is
(nsteps/every + every) states, compute one extra forward step per step.

No CPU or autograd-traced implementation of the step exists here: torch only
holds the buffers and chains the objective; the step and its adjoint are the
engine's kernels.
"""
import torch

import pydugks

_TORCH_DTYPE = {0: torch.float64, 1: torch.float32}


def state_dtype(eng):
    if eng.info.precision not in _TORCH_DTYPE:
        raise pydugks.DugksError(pydugks.DG_ERR_UNSUPPORTED, "the adjoint exists for the fp64 and fp32 forms")
    return _TORCH_DTYPE[eng.info.precision]


def empty_state(eng, device="cuda"):
    return torch.empty(eng.soa_len, dtype=state_dtype(eng), device=device)


def soa_view(eng, t):
    """(19, nz, ny, nx) view of an SoA state tensor (drops the x pitch padding)."""
    nx, ny, nz = eng.nx, eng.ny, eng.nz
    ps, pitch = eng.info.pop_stride, eng.info.pitch
    return t.view(19, ps)[:, : nz * ny * pitch].view(19, nz, ny, pitch)[..., :nx]


def from_dump_order(eng, f):
    """(nz, ny, nx, 19) dump-order tensor -> SoA state tensor."""
    out = torch.zeros(eng.soa_len, dtype=state_dtype(eng), device=f.device)
    soa_view(eng, out).copy_(f.permute(3, 0, 1, 2))
    return out


def to_dump_order(eng, t):
    return soa_view(eng, t).permute(1, 2, 3, 0)


def _sync_stream(eng):
    eng.set_stream(torch.cuda.current_stream().cuda_stream)


class DugksRun(torch.autograd.Function):
    @staticmethod
    def forward(ctx, f0, eng, istep0, nsteps, every):
        _sync_stream(eng)
        every = max(1, int(every))
        cps = [f0.detach().clone()]
        eng.set_state_device(f0.data_ptr())
        for s in range(nsteps):
            if s > 0 and s % every == 0:
                cp = empty_state(eng, f0.device)
                eng.get_state_device(cp.data_ptr())
                cps.append(cp)
            eng.step(istep0 + s)
        out = empty_state(eng, f0.device)
        eng.get_state_device(out.data_ptr())
        ctx.eng, ctx.istep0, ctx.nsteps, ctx.every, ctx.cps = eng, istep0, nsteps, every, cps
        return out

    @staticmethod
    def backward(ctx, lam_out):
        eng, istep0, nsteps, every = ctx.eng, ctx.istep0, ctx.nsteps, ctx.every
        _sync_stream(eng)
        lam = lam_out.detach().contiguous().clone()
        nseg = (nsteps + every - 1) // every
        for seg in reversed(range(nseg)):
            s0, s1 = seg * every, min(nsteps, (seg + 1) * every)
            eng.set_state_device(ctx.cps[seg].data_ptr())
            states = []
            for s in range(s0, s1):
                cur = empty_state(eng, lam.device)
                eng.get_state_device(cur.data_ptr())
                states.append(cur)
                if s + 1 < s1:
                    eng.step(istep0 + s)
            for s in reversed(range(s0, s1)):
                eng.adjoint_step(istep0 + s, states[s - s0].data_ptr(), lam.data_ptr(), lam.data_ptr())
            del states
        ctx.cps = None
        return lam, None, None, None, None


def run(f0, eng, istep0, nsteps, every=100):
    return DugksRun.apply(f0, eng, istep0, nsteps, every)


# --- D3Q19 helpers for objectives and controls (torch, differentiable) ---
_C = [[0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0],
      [0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1],
      [0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1]]
_W = [1 / 3] + [1 / 18] * 6 + [1 / 36] * 12


def lattice(dtype, device):
    c = torch.tensor(_C, dtype=dtype, device=device)  # (3, 19)
    w = torch.tensor(_W, dtype=dtype, device=device)
    return c, w


def feq(rho, u):
    """rho (...), u (3, ...) -> (19, ...) second-order equilibrium."""
    c, w = lattice(u.dtype, u.device)
    eu = 3.0 * torch.einsum("ap,a...->p...", c, u)
    uu = 3.0 * (u * u).sum(0)
    shape = (19,) + (1,) * rho.dim()
    return w.view(shape) * rho * (1.0 + eu + 0.5 * (eu * eu - uu))


def macro(f19):
    """f (19, ...) -> rho (...), u (3, ...)."""
    c, _ = lattice(f19.dtype, f19.device)
    rho = f19.sum(0)
    j = torch.einsum("ap,p...->a...", c, f19)
    return rho, j / rho


def kinetic_energy(eng, t, shift=None):
    """0.5 * sum rho |u|^2 over the grid; u = j/rho (+ shift, e.g. hdt*F)."""
    rho, u = macro(soa_view(eng, t))
    if shift is not None:
        u = u + torch.as_tensor(shift, dtype=u.dtype, device=u.device).view(3, 1, 1, 1)
    return 0.5 * (rho * (u * u).sum(0)).sum()
