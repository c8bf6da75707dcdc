#!/usr/bin/env python3
"""Adjoint of the time-averaged wall shear stress through the turbulent
channel with respect to a spatially varying streamwise body-force field.

Workload: Re_tau = 180 channel, 192 (streamwise) x 128 (wall-normal, tanh) x
96 (spanwise) cells, in the engine's orientation nx = 128 (walls on the x
faces), ny = 96, nz = 192 with the force along z.  FP32 forward with FP64
objective accumulation, `--steps` steps from the seeded perturbed laminar
start (case=channel_turb, seed 0), control phi = per-cell z force field
(FP32, zero), objective J = (1/n) sum_k tau_w(f_k) (dugks_autograd.WallShear),
gradient dJ/dphi through dugks_autograd.DugksObjectiveRun with the binomial
checkpointing schedule; the stored states are sized to <= `--snap-gb` GB.

Reports, side by side: the FP32 forward step (plain, and with the control
field set: the step the gradient differentiates), the FP16-deviation (mixed)
forward step, the adjoint step (dg_adjoint_step alone) and the whole
gradient (forward sweep + recomputation + adjoint) per step, and, with
`--fd-steps`, an FP64 check of the gradient against central differences on
the same grid over a shorter horizon.

  python dugks-gpu_gb300/adjoint_channel.py --steps 4000
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
import revolve  # noqa: E402


def _events_ms(torch, fn, reps):
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    fn()
    torch.cuda.synchronize()
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    e1.synchronize()
    return e0.elapsed_time(e1) / reps


def forward_ms(torch, prec, args, field=False):
    cfg, _ = pydugks.channel_config(nx=args.nx, ny=args.ny, nz=args.nz, precision=prec, seed=0)
    eng = pydugks.Engine(cfg)
    eng.set_stream(torch.cuda.current_stream().cuda_stream)
    if field:  # the step the gradient differentiates: with the (zero) control field set
        eng.set_force_field(2, np.zeros((eng.nz, eng.ny, eng.nx)))
    step = [1]

    def one():
        eng.step(step[0])
        step[0] += 1

    ms = _events_ms(torch, one, args.time_reps)
    eng.close()
    return ms


def gradient_run(torch, da, args):
    cfg, meta = pydugks.channel_config(nx=args.nx, ny=args.ny, nz=args.nz, precision="fp32", seed=0)
    eng = pydugks.Engine(cfg)
    eng.set_stream(torch.cuda.current_stream().cuda_stream)
    state_bytes = eng.soa_len * 4
    snaps = min(args.steps, int(args.snap_gb * 1e9 // state_bytes) - 4)
    obj = da.WallShear(eng, axis=2)
    f0 = torch.empty(eng.soa_len, dtype=torch.float32, device="cuda")
    eng.get_state_device(f0.data_ptr())
    phi = torch.zeros((eng.nz, eng.ny, eng.nx), dtype=torch.float32, device="cuda", requires_grad=True)

    # adjoint step alone (kernels of dg_adjoint_step), at the initial state
    eng.set_force_field(2, np.zeros((eng.nz, eng.ny, eng.nx)))
    lam = torch.zeros_like(f0)
    adj_ms = _events_ms(torch, lambda: eng.adjoint_step(1, f0.data_ptr(), lam.data_ptr(), lam.data_ptr()),
                        args.time_reps)
    eng.field_grad(reset=True)

    acts = revolve.actions(args.steps, snaps)
    end, _ = revolve.spine(acts)
    total_adv, peak = revolve.simulate(args.steps, snaps)
    spine_adv = sum(a[2] - a[1] for a in acts[:end] if a[0] == "advance")
    # an untimed two-step gradient first: allocates the engine's checkpoint pool (tens of GB,
    # whose first allocation on a device can take seconds), reused by the timed run
    _, Jw = da.run_objective(f0, phi, eng, 1, 2, obj, snaps=snaps, axis=2)
    torch.autograd.grad(Jw, [phi])
    eng.field_grad(reset=True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    _, J = da.run_objective(f0, phi, eng, 1, args.steps, obj, snaps=snaps, axis=2)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    (g,) = torch.autograd.grad(J, [phi])
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    # the same gradient once more with every action bracketed by CUDA events: GPU time per kind
    eng.field_grad(reset=True)
    da.PROFILE = da.ActionTimer()
    _, Jp = da.run_objective(f0, phi, eng, 1, args.steps, obj, snaps=snaps, axis=2)
    torch.autograd.grad(Jp, [phi])
    breakdown = {k: {"count": c, "gpu_ms": round(ms, 1)} for k, (c, ms) in da.PROFILE.summary().items()}
    da.PROFILE = None
    gd = g.double()
    res = dict(J=float(J.detach()), tau_w_laminar=meta["utau"] ** 2, snaps=snaps, snap_gb=round(peak * state_bytes / 1e9, 2),
               recomputed_steps=total_adv - spine_adv,
               forward_sweep_s=round(t1 - t0, 3), backward_s=round(t2 - t1, 3),
               gpu_ms_by_action=breakdown,
               adjoint_ms_per_step_harness=(t2 - t1) * 1e3 / args.steps,
               grad_l2=float(gd.norm()), grad_max=float(gd.abs().max()),
               grad_sum=float(gd.sum()), grad_mean_wall_cells=float(gd[:, :, [0, -1]].mean()),
               grad_mean_centre=float(gd[:, :, eng.nx // 2 - 1: eng.nx // 2 + 1].mean()))
    eng.close()
    return res, adj_ms


def fd_check(torch, da, args):
    """FP64 adjoint vs central differences on the same grid, --fd-steps steps."""
    cfg, meta = pydugks.channel_config(nx=args.nx, ny=args.ny, nz=args.nz, precision="fp64", seed=0)
    eng = pydugks.Engine(cfg)
    eng.set_stream(torch.cuda.current_stream().cuda_stream)
    obj = da.WallShear(eng, axis=2)
    f0 = torch.empty(eng.soa_len, dtype=torch.float64, device="cuda")
    eng.get_state_device(f0.data_ptr())
    n = args.fd_steps
    phi0 = torch.zeros((eng.nz, eng.ny, eng.nx), dtype=torch.float64, device="cuda")
    phi = phi0.clone().requires_grad_(True)
    _, J = da.run_objective(f0, phi, eng, 1, n, obj, snaps=16, axis=2)
    (g,) = torch.autograd.grad(J, [phi])
    rng = np.random.default_rng(5)
    out = []
    for k in range(args.fd_dirs):
        # directions scaled to the driving force, steps eps * F
        d = torch.from_numpy(rng.uniform(-1, 1, size=phi0.shape)).cuda() * meta["F"]

        def Jd(h):
            with torch.no_grad():
                _, j = da.run_objective(f0, phi0 + h * d, eng, 1, n, obj, snaps=0, axis=2)
            return float(j)

        e = args.fd_eps
        c = lambda h: (Jd(h) - Jd(-h)) / (2 * h)  # noqa: E731
        fd = (4 * c(e / 2) - c(e)) / 3
        ad = float((g * d).sum())
        out.append(dict(adjoint=ad, fd=fd, rel=abs(ad - fd) / abs(fd)))
    eng.close()
    return out


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--nx", type=int, default=128)
    ap.add_argument("--ny", type=int, default=96)
    ap.add_argument("--nz", type=int, default=192)
    ap.add_argument("--steps", type=int, default=4000)
    ap.add_argument("--snap-gb", type=float, default=100.0)
    ap.add_argument("--time-reps", type=int, default=100)
    ap.add_argument("--fd-steps", type=int, default=0)
    ap.add_argument("--fd-dirs", type=int, default=2)
    ap.add_argument("--fd-eps", type=float, default=1e-3)
    args = ap.parse_args()
    import torch
    import dugks_autograd as da

    fwd32 = forward_ms(torch, "fp32", args)
    fwd32f = forward_ms(torch, "fp32", args, field=True)
    fwd16 = forward_ms(torch, "fp16", args)
    grad, adj_ms = gradient_run(torch, da, args)
    n = args.nx * args.ny * args.nz
    res = dict(workload=f"Re_tau=180 channel {args.nz}x{args.nx}x{args.ny} (streamwise x wall-normal tanh x spanwise)",
               steps=args.steps, cells=n,
               forward_fp32_ms=fwd32, forward_fp32_field_ms=fwd32f, forward_fp16_ms=fwd16, adjoint_step_ms=adj_ms,
               forward_fp32_mlups=n / fwd32 / 1e3, forward_fp16_mlups=n / fwd16 / 1e3,
               # the adjoint (of the step with the control field) against that step, and against the plain step
               adjoint_over_forward=adj_ms / fwd32f, adjoint_over_plain_forward=adj_ms / fwd32,
               gradient_ms_per_step=grad["adjoint_ms_per_step_harness"] + grad["forward_sweep_s"] * 1e3 / args.steps,
               **grad)
    # the adjoint cost per step: the whole gradient (forward sweep, recomputation, adjoint) per step
    # and the reversal alone, each over the forward step it differentiates
    res["gradient_over_forward_step"] = res["gradient_ms_per_step"] / fwd32f
    res["reversal_over_forward_step"] = res["adjoint_ms_per_step_harness"] / fwd32f
    if args.fd_steps:
        res["fd_fp64"] = fd_check(torch, da, args)
    print(json.dumps(res))


if __name__ == "__main__":
    main()
