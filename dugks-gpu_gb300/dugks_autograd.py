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
import revolve

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


class _DeviceBuffer:
    """A CUDA array interface over a raw device pointer (no ownership, no copy)."""

    def __init__(self, ptr, n, typestr):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": typestr, "data": (int(ptr), False),
                                         "strides": None, "version": 3}


def engine_state(eng):
    """Tensor view of the engine's own state buffer (DG_BUF_F, SoA layout): it
    follows the state as steps run on the engine's stream; no copy."""
    dt = state_dtype(eng)
    buf = _DeviceBuffer(eng.device_ptr(pydugks.DG_BUF_F), eng.soa_len, "<f8" if dt == torch.float64 else "<f4")
    return torch.as_tensor(buf, device="cuda")


def _sync_stream(eng):
    eng.set_stream(torch.cuda.current_stream().cuda_stream)


class ActionTimer:
    """GPU time per kind of action of a checkpointed reversal (CUDA events on the
    current stream).  Assign an instance to `dugks_autograd.PROFILE` to have
    DugksObjectiveRun record into it; `summary()` synchronises once and gives
    {kind: (count, milliseconds)}."""

    def __init__(self):
        self.events = {}

    def wrap(self, kind, fn, *a):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        out = fn(*a)
        e1.record()
        self.events.setdefault(kind, []).append((e0, e1))
        return out

    def summary(self):
        torch.cuda.synchronize()
        return {k: (len(v), sum(a.elapsed_time(b) for a, b in v)) for k, v in self.events.items()}


PROFILE = None


def _timed(kind, fn, *a):
    return PROFILE.wrap(kind, fn, *a) if PROFILE is not None else fn(*a)


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
        # one buffer of `every` states, refilled per segment by the engine (recomputation and
        # the reversed adjoint steps each run as one call)
        states = torch.empty((min(every, nsteps), eng.soa_len), dtype=lam.dtype, device=lam.device)
        stride = states.stride(0) * states.element_size()
        for seg in reversed(range(nseg)):
            s0, s1 = seg * every, min(nsteps, (seg + 1) * every)
            eng.set_state_device(ctx.cps[seg].data_ptr())
            eng.run_store(istep0 + s0, s1 - s0, states.data_ptr(), stride)
            eng.adjoint_run(istep0 + s0, s1 - s0, states.data_ptr(), stride, lam.data_ptr())
        del states
        ctx.cps = None
        return lam, None, None, None, None


def run(f0, eng, istep0, nsteps, every=100):
    return DugksRun.apply(f0, eng, istep0, nsteps, every)


class _StatePool:
    """Slots for the checkpointed states of one schedule, allocated at once:
    hundreds of separate allocations of a few hundred MB each can cost
    seconds on a fresh device.  `for_engine` keeps one pool per engine and
    reuses it while the slot count and layout match (the memory stays
    allocated while the engine object lives)."""

    def __init__(self, eng, nslots, device):
        self.buf = torch.empty((nslots, eng.soa_len), dtype=state_dtype(eng), device=device)
        self.reset()

    def reset(self):
        self.free = list(range(self.buf.shape[0] - 1, -1, -1))
        self.slot = {}

    @staticmethod
    def for_engine(eng, nslots, device):
        pool = getattr(eng, "_dg_state_pool", None)
        if (pool is None or pool.buf.shape != (nslots, eng.soa_len) or pool.buf.dtype != state_dtype(eng)
                or pool.buf.device != torch.device(device)):
            eng._dg_state_pool = None  # release the old pool before allocating the new one
            pool = _StatePool(eng, nslots, device)
            eng._dg_state_pool = pool
        pool.reset()
        return pool

    def store(self, key):
        """The slot that holds state `key` from now on (its old slot if it has one)."""
        if key not in self.slot:
            if not self.free:
                raise RuntimeError("checkpoint pool exhausted")
            self.slot[key] = self.free.pop()
        return self.buf[self.slot[key]]

    def __getitem__(self, key):
        return self.buf[self.slot[key]]

    def release(self, key):
        i = self.slot.pop(key, None)
        if i is not None:
            self.free.append(i)


class DugksObjectiveRun(torch.autograd.Function):
    """(f0, phi) -> (f_n, J), J = (1/n) sum_{k=1..n} objective(f_k, phi).

    phi (nz, ny, nx) is the engine's body-force field along `axis`
    (dg_set_force_field).  The backward reverses the n steps with the binomial
    checkpointing schedule of revolve.py using `snaps` stored states besides
    f0; the state-side gradient runs the hand-written adjoint kernels
    (dg_adjoint_step), which also accumulate dJ/dphi of every step
    (dg_field_grad).  The objective's own gradients (the source added to the
    adjoint at each state and its direct dependence on phi) come from torch
    autograd on `objective`, or from `objective.accumulate(lam, state, phi,
    weight)` when the objective provides it (returns d/dphi of weight * g).
    """

    @staticmethod
    def forward(ctx, f0, phi, eng, istep0, nsteps, snaps, objective, axis):
        _sync_stream(eng)
        eng.set_force_field(axis, phi.detach().double().cpu().numpy())
        acts = revolve.actions(nsteps, snaps)
        end, last = revolve.spine(acts)
        stored = _StatePool.for_engine(eng, snaps + 1, f0.device)  # f0 and at most `snaps` more
        stored.store(0).copy_(f0.detach())
        eng.set_state_device(f0.data_ptr())
        J = torch.zeros((), dtype=torch.float64, device=f0.device)
        phi_d = phi.detach()
        state = engine_state(eng)
        # objectives with `prepare(phi)` give a per-state evaluator for the fixed control
        value = objective.prepare(phi_d) if hasattr(objective, "prepare") else (lambda s: objective(s, phi_d))

        def advance(a, b):
            for k in range(a, b):
                _timed("forward step", eng.step, istep0 + k)
                with torch.no_grad():
                    _timed("forward objective", lambda: J.add_(value(state).double()))

        k = 0
        for a in acts[:end]:
            if a[0] == "advance":
                advance(a[1], a[2])
                k = a[2]
            else:
                _timed("forward store", eng.get_state_device, stored.store(a[1]).data_ptr())
        advance(k, nsteps)
        out = empty_state(eng, f0.device)
        eng.get_state_device(out.data_ptr())
        ctx.eng, ctx.istep0, ctx.nsteps, ctx.objective, ctx.axis = eng, istep0, nsteps, objective, axis
        ctx.acts, ctx.end, ctx.last, ctx.stored = acts, end, last, stored
        ctx.save_for_backward(phi)
        return out, J / nsteps

    @staticmethod
    def backward(ctx, lam_out, gJ):
        eng, istep0, n, objective = ctx.eng, ctx.istep0, ctx.nsteps, ctx.objective
        (phi,) = ctx.saved_tensors
        _sync_stream(eng)
        dev = lam_out.device if lam_out is not None else phi.device
        w = (gJ.double() / n) if gJ is not None else torch.zeros((), dtype=torch.float64, device=dev)
        eng.set_force_field(ctx.axis, phi.detach().double().cpu().numpy())
        eng.field_grad(reset=True)
        stored = ctx.stored
        if lam_out is None:
            lam = torch.zeros_like(stored[0])
        else:
            lam = lam_out.detach().contiguous().clone()
        dphi_direct = torch.zeros(phi.shape, dtype=torch.float64, device=phi.device)
        cur = engine_state(eng)  # the engine's current state (read by the adjoint and the sources)
        # objectives with `prepare_adjoint(phi, w)` give a per-state source for the fixed control
        # (a few kernels per step) and the direct phi-gradient summed over all steps at the end
        fast = objective.prepare_adjoint(phi.detach(), w) if hasattr(objective, "prepare_adjoint") else None

        def source(state):
            nonlocal dphi_direct
            if fast is not None:
                _timed("adjoint source", fast[0], lam, state)
                return
            acc = getattr(objective, "accumulate", None)
            if acc is not None:
                dphi_direct += acc(lam, state, phi.detach(), w).double()
                return
            with torch.enable_grad():
                s = state.detach().clone().requires_grad_(True)
                p = phi.detach().requires_grad_(True)
                g = objective(s, p).double() * w
                gs, gp = torch.autograd.grad(g, [s, p], allow_unused=True)
            if gs is not None:
                lam.add_(gs.to(lam.dtype))
            if gp is not None:
                dphi_direct += gp.double()

        # The current state lives either in the engine's own buffer (`cur`) or in a
        # stored slot: advances step out of place from a slot (dg_run_between), an
        # advance followed by a store writes its last state straight into the new
        # slot, and a restore only points at the slot -- no state copies.
        where = [stored[ctx.last]]  # tensor holding the current state
        own = cur.data_ptr()

        def same(x, y):
            return x is not None and y is not None and x.data_ptr() == y.data_ptr()

        def advance_to(a, b, dst):
            src = None if where[0].data_ptr() == own else where[0].data_ptr()
            _timed("recompute", eng.run_between, istep0 + a, b - a, src, None if dst.data_ptr() == own else dst.data_ptr())
            where[0] = dst

        # source at the final state f_n
        if n > ctx.last:
            advance_to(ctx.last, n, cur)
        source(where[0])
        # resume the schedule from the last state of the forward sweep
        where[0] = stored[ctx.last]
        acts = ctx.acts[ctx.end:]
        for i, a in enumerate(acts):
            kind = a[0]
            if kind == "advance":
                nxt = acts[i + 1] if i + 1 < len(acts) else None
                if nxt is not None and nxt[0] == "store" and nxt[1] == a[2]:
                    advance_to(a[1], a[2], stored.store(a[2]))
                else:
                    advance_to(a[1], a[2], cur)
            elif kind == "store":
                slot = stored.store(a[1])
                if not same(where[0], slot):  # a store not written by the advance before it
                    _timed("store", slot.copy_, where[0])
                    where[0] = slot
            elif kind == "restore":
                where[0] = stored[a[1]]
            elif kind == "release":
                if same(where[0], stored[a[1]]):
                    where[0] = None
                stored.release(a[1])
            else:  # adjoint of step k at the current state k
                k = a[1]
                st = where[0]
                _timed("adjoint step", eng.adjoint_step, istep0 + k, st.data_ptr(), lam.data_ptr(), lam.data_ptr())
                if k >= 1:
                    source(st)
        if fast is not None:
            dphi_direct += fast[1]()
        dphi = torch.from_numpy(eng.field_grad(reset=True)).to(phi.device) + dphi_direct
        ctx.stored = None
        return lam, dphi.to(phi.dtype), None, None, None, None, None, None


def run_objective(f0, phi, eng, istep0, nsteps, objective, snaps=64, axis=2):
    """f_n, J = DugksObjectiveRun (see its docstring)."""
    return DugksObjectiveRun.apply(f0, phi, eng, istep0, nsteps, snaps, objective, axis)


class WallShear:
    """Mean wall shear stress of a channel with walls on the two x faces.

    tau = rho nu u_s / d at the first cell of each wall (no-slip wall, d the
    distance of the cell centre from the wall), u_s the velocity along
    `axis` including the half-step force shift hdt*F that the reference's
    output velocity carries, F = ambient + phi; averaged over both walls.
    With rho u_s = j_s + hdt rho F_s the objective is linear in the state
    for fixed phi; `accumulate` adds its gradient to the wall planes of the
    adjoint directly.
    """

    def __init__(self, eng, axis=2):
        self.eng, self.axis = eng, axis
        info = eng.info
        xc, _ = eng.mesh()
        xw = eng.info.xwidth
        self.d0, self.d1 = float(xc[1]), float(xw - xc[eng.nx])
        self.nu = float(info.visc)
        self.hdt = 0.5 * float(info.dt)
        self.F = float(info.ambient[axis])
        self.area = 2.0 * eng.ny * eng.nz
        c, _ = lattice(torch.float64, "cpu")
        self.cs = c[axis]

    def _planes(self, t):
        v = soa_view(self.eng, t)
        return v[..., 0], v[..., self.eng.nx - 1]   # (19, nz, ny) each

    def prepare(self, phi):
        """Evaluator of the objective for a fixed field phi: the objective is a
        weighted sum over the two wall planes, weights (nu/d)(c_s + hdt F_s)/area
        formed once; each evaluation is one gather and one FP64 reduction."""
        nx = self.eng.nx
        dev = phi.device
        cs = self.cs.to(torch.float64).to(dev).view(19, 1, 1, 1)
        ph = phi[:, :, [0, nx - 1]].double()                                  # (nz, ny, 2)
        wd = torch.tensor([self.nu / self.d0, self.nu / self.d1], dtype=torch.float64, device=dev)
        W = (cs + self.hdt * (self.F + ph).unsqueeze(0)) * wd / self.area      # (19, nz, ny, 2)
        idx = torch.tensor([0, nx - 1], device=dev)

        def value(state):
            planes = soa_view(self.eng, state).index_select(3, idx)          # (19, nz, ny, 2)
            return (planes.double() * W).sum()

        return value

    def __call__(self, state, phi):
        lo, hi = self._planes(state)
        cs = self.cs.to(state.dtype).to(state.device).view(19, 1, 1)
        tot = 0.0
        for pl, d, ii in ((lo, self.d0, 0), (hi, self.d1, self.eng.nx - 1)):
            rho = pl.sum(0)
            js = (cs * pl).sum(0)
            Fs = self.F + phi[:, :, ii].to(state.dtype)
            tot = tot + (self.nu / d) * (js + self.hdt * rho * Fs).sum()
        return tot / self.area

    def prepare_adjoint(self, phi, w):
        """(add, finish) for the reversal with phi and the weight w fixed: the
        source this objective adds to the adjoint at every state is constant,
        (w nu / (d area)) (c_s + hdt F_s) on the two wall planes, so it is formed
        once and `add(lam, state)` adds it with one kernel; the direct phi
        gradient, (w nu hdt / (d area)) rho at the wall cells of every state, is
        summed per state into one FP64 buffer and `finish()` scales it once."""
        nx = self.eng.nx
        dev = phi.device
        dt = state_dtype(self.eng)
        idx = torch.tensor([0, nx - 1], device=dev)
        cs = self.cs.to(torch.float64).to(dev).view(19, 1, 1, 1)
        k = torch.stack([w * (self.nu / self.d0) / self.area, w * (self.nu / self.d1) / self.area]).to(dev)
        Fs = (self.F + phi[:, :, [0, nx - 1]].double()).unsqueeze(0)            # (1, nz, ny, 2)
        S = (k * (cs + self.hdt * Fs)).to(dt)                                   # (19, nz, ny, 2)
        rho_sum = torch.zeros((self.eng.nz, self.eng.ny, 2), dtype=torch.float64, device=dev)

        def add(lam, state):
            soa_view(self.eng, lam).index_add_(3, idx, S)
            rho_sum.add_(soa_view(self.eng, state).index_select(3, idx).sum(0, dtype=torch.float64))

        def finish():
            dphi = torch.zeros(phi.shape, dtype=torch.float64, device=dev)
            dphi[:, :, [0, nx - 1]] = k * self.hdt * rho_sum
            return dphi

        return add, finish

    def accumulate(self, lam, state, phi, w):
        lo_l, hi_l = self._planes(lam)
        lo_s, hi_s = self._planes(state)
        cs = self.cs.to(lam.dtype).to(lam.device).view(19, 1, 1)
        dphi = torch.zeros(phi.shape, dtype=torch.float64, device=phi.device)
        for pl, pst, d, ii in ((lo_l, lo_s, self.d0, 0), (hi_l, hi_s, self.d1, self.eng.nx - 1)):
            k = w * (self.nu / d) / self.area
            Fs = (self.F + phi[:, :, ii].double())
            # d/df_p (j_s + hdt rho F_s) = c_sp + hdt F_s
            pl.add_((k * (cs.double() + self.hdt * Fs.unsqueeze(0))).to(lam.dtype))
            dphi[:, :, ii] += k * self.hdt * pst.double().sum(0)
        return dphi


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
