#!/usr/bin/env python3
"""Adjoint verification on the 3-D Taylor-Green vortex.

64^3 periodic, D3Q19, u0 = 0.05, Re = u0 L / nu = 1600 with L = 64/(2 pi),
CFL 0.5.  Objective: total kinetic energy 0.5 sum rho |u|^2 after `--steps`
steps; control: the initial velocity field u0(x) (3 x 64^3), entering through
f0 = feq(rho0, u0) with the tg_eq density rho0 held fixed.  The gradient comes
from the hand-written adjoint (dugks_autograd.DugksRun, checkpoints every
`--every` steps, one recomputation per step) and is checked by central
differences (eps = 1e-6) along `--dirs` seeded random directions
(splitmix64 seeds 0..dirs-1).  Also reports the cost of the adjoint pass
(including recomputation) relative to the forward pass, and of one adjoint
step alone relative to one forward step.

  python dugks-gpu_gb300/verify_adjoint.py --precision fp64 --steps 2000 --every 100 --dirs 16

With --precision fp32 the FP32 adjoint gradient is checked against the FP64
problem: central differences of the FP64 forward (an FP32 forward cannot
resolve a 1e-6 perturbation) and the FP64 adjoint gradient (relative
max-norm difference).
"""
import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import pydugks  # noqa: E402


def uniform_sym(seed, n):
    """splitmix64(seed, index) -> n values in [-1, 1)."""
    M = (1 << 64) - 1
    with np.errstate(over="ignore"):
        z = np.arange(n, dtype=np.uint64) * np.uint64(64) + np.uint64((seed * 0xD1B54A32D192ED03) & M)
        z = z + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(11)).astype(np.float64) * (2.0 / 9007199254740992.0) - 1.0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=64)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--every", type=int, default=100)
    ap.add_argument("--dirs", type=int, default=16)
    ap.add_argument("--eps", type=float, default=1e-6)
    ap.add_argument("--precision", default="fp64", choices=("fp64", "fp32"))
    args = ap.parse_args()

    import torch
    import dugks_autograd as da

    n = args.n
    # tg_eq with the amplitude u0 = 0.05 in the velocity and the density term (key tg_u0)
    cfg = pydugks.taylor_green_config(n=n, u0=0.05, re=1600.0, precision=args.precision)
    eng = pydugks.Engine(cfg)
    f0 = eng.get_state()
    dt = torch.float64 if args.precision == "fp64" else torch.float32
    rho0, u_tg = da.macro(torch.from_numpy(f0).permute(3, 0, 1, 2).cuda())
    u_init = u_tg.to(dt)
    rho0 = rho0.to(dt)

    def J(u, every=args.every):
        f = da.feq(rho0, u).permute(1, 2, 3, 0)
        t0 = da.from_dump_order(eng, f)
        fN = da.run(t0, eng, 1, args.steps, every)
        return da.kinetic_energy(eng, fN)

    # forward alone (timing), after one untimed run (first-use costs of the engine and torch)
    with torch.no_grad():
        J(u_init, every=args.steps + 1)
    torch.cuda.synchronize()
    t = time.perf_counter()
    with torch.no_grad():
        J(u_init, every=args.steps + 1)
    torch.cuda.synchronize()
    t_fwd = time.perf_counter() - t

    # one untimed gradient (first use of the adjoint kernels and buffers), then the timed one
    u = u_init.clone().requires_grad_(True)
    torch.autograd.grad(J(u), u)
    torch.cuda.synchronize()
    t = time.perf_counter()
    Ju = J(u)
    torch.cuda.synchronize()
    t_fwd_ckpt = time.perf_counter() - t
    t = time.perf_counter()
    (g,) = torch.autograd.grad(Ju, u)
    torch.cuda.synchronize()
    t_adj = time.perf_counter() - t

    # the adjoint step alone: `every` steps reversed from states recorded beforehand, against
    # the forward step of the timed forward run
    with torch.no_grad():
        f_init = da.from_dump_order(eng, da.feq(rho0, u_init).permute(1, 2, 3, 0))
        states = torch.empty((args.every, eng.soa_len), dtype=f_init.dtype, device="cuda")
        stride = states.stride(0) * states.element_size()
        eng.set_state_device(f_init.data_ptr())
        eng.run_store(1, args.every, states.data_ptr(), stride)
        lam_t = torch.ones(eng.soa_len, dtype=f_init.dtype, device="cuda")
        eng.adjoint_run(1, args.every, states.data_ptr(), stride, lam_t.data_ptr())  # warm-up
        torch.cuda.synchronize()
        t = time.perf_counter()
        eng.adjoint_run(1, args.every, states.data_ptr(), stride, lam_t.data_ptr())
        torch.cuda.synchronize()
        t_adj_step = (time.perf_counter() - t) / args.every
        del states

    Jfd, extra = J, {}
    if args.precision == "fp32":
        eng64 = pydugks.Engine(cfg.replace("precision=fp32", "precision=fp64"))
        rho64, u64 = da.macro(torch.from_numpy(eng64.get_state()).permute(3, 0, 1, 2).cuda())

        def Jfd(uu, every=args.every):
            f = da.feq(rho64, uu.double()).permute(1, 2, 3, 0)
            fN = da.run(da.from_dump_order(eng64, f), eng64, 1, args.steps, every)
            return da.kinetic_energy(eng64, fN)

        uu = u64.clone().requires_grad_(True)
        (g64,) = torch.autograd.grad(Jfd(uu), uu)
        extra = {"fd_source": "fp64 forward",
                 "grad_rel_vs_fp64_adjoint": float((g.double() - g64).abs().max() / g64.abs().max())}
        u_init = u64

    rels = []
    for k in range(args.dirs):
        d = torch.from_numpy(uniform_sym(k, u.numel()).reshape(u.shape)).to(device="cuda", dtype=u_init.dtype)
        with torch.no_grad():
            fd = float((Jfd(u_init + args.eps * d) - Jfd(u_init - args.eps * d)) / (2 * args.eps))
        ad = float((g.to(d.dtype) * d).sum())
        rels.append(abs(ad - fd) / abs(fd))
    cells = n ** 3
    out = {"workload": f"Taylor-Green vortex {n}^3 periodic, u0=0.05, Re=1600, {args.precision}",
           "steps": args.steps, "checkpoint_every": args.every, "J": float(Ju.detach()),
           "fd_rel_err_max": max(rels), "fd_rel_err_median": float(np.median(rels)), "dirs": args.dirs,
           "eps": args.eps,
           "forward_s": t_fwd, "forward_with_checkpoints_s": t_fwd_ckpt, "adjoint_s": t_adj,
           "adjoint_over_forward": t_adj / t_fwd,
           "adjoint_step_ms": 1e3 * t_adj_step, "forward_step_ms": 1e3 * t_fwd / args.steps,
           "adjoint_step_over_forward_step": t_adj_step / (t_fwd / args.steps),
           "forward_mlups": cells * args.steps / t_fwd / 1e6,
           "adjoint_mlups": cells * args.steps / t_adj / 1e6,
           "checkpoint_states": args.steps // args.every + args.every,
           "checkpoint_bytes": (args.steps // args.every + args.every) * eng.soa_len * (8 if args.precision == "fp64" else 4)}
    out.update(extra)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
