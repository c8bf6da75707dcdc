#!/usr/bin/env python3
"""Accuracy and speed of the mixed-precision forms against FP64.

Runs the turbulent channel (Re_tau = 180, tanh wall-normal mesh, seeded
synthetic start, the benchmark workload) in FP64, FP32, FP16-deviation and
BF16-deviation storage from the same initial state, accumulates time-averaged
profiles in FP64 on the device (dg_stats_accumulate) every `--every` steps
after `--burn` steps, and reports per form:

  U+        mean streamwise velocity / u_tau     (rel. L2 error vs FP64)
  uw+       Reynolds shear stress <u'w'> / u_tau^2 (error / max |FP64|)
  urms+     streamwise rms / u_tau               (rel. L2 error vs FP64)
  MLUPS     step throughput of the form (device-resident, CUDA events)
  mass      relative drift of the volume-weighted mass

The form `fp64p` is FP64 from the same start with every value multiplied by
(1 + eps r), r uniform in [-1, 1) (seeded, eps = --pert): its errors against
FP64 are the sampling floor of a chaotic flow, the difference that any change
of rounding makes to finite-time averages once the trajectories have
decorrelated; errors of the reduced forms at that level are not precision
errors.  `bf16n` and `fp16n` are the 16-bit forms with round-to-nearest
storage (the default is stochastic rounding), `fp16s` the FP16 form with
stochastic rounding named explicitly.  With --start every form starts from the
given state (a developed turbulent state from channel_spinup.py) instead of
the seeded laminar start.

Reference orientation: x wall-normal, y spanwise, z streamwise.

  python dugks-gpu_gb300/verify_mixed.py --steps 5000 --every 10 --burn 1000
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


def run_form(form, args):
    import torch
    prec = {"fp64p": "fp64", "bf16n": "bf16", "fp16n": "fp16", "fp16s": "fp16"}.get(form, form)
    extra = {"bf16n": {"rounding": "nearest"}, "fp16n": {"rounding": "nearest"},
             "fp16s": {"rounding": "stochastic"}}.get(form, {})
    cfg, meta = pydugks.channel_config(nx=args.nx, ny=args.ny, nz=args.nz, precision=prec, **extra)
    eng = pydugks.Engine(cfg)
    eng.set_stream(torch.cuda.current_stream().cuda_stream)
    if args.start:
        eng.set_state(np.load(args.start, mmap_mode="r"))
    if form == "fp64p":
        f = eng.get_state()
        r = np.random.default_rng(args.seed).uniform(-1.0, 1.0, f.shape)
        eng.set_state(f * (1.0 + args.pert * r))
    _, dxx = eng.mesh()
    w = dxx[1:-1]
    m0 = float((eng.get_state().sum(axis=-1) * w).sum())
    n = args.nx * args.ny * args.nz
    step = 1
    t_dev = 0.0
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    while step <= args.steps:
        chunk = args.every if step > args.burn else min(args.every, args.burn - step + 1)
        chunk = min(chunk, args.steps - step + 1)
        e0.record()
        eng.run(step, chunk)
        e1.record()
        e1.synchronize()
        t_dev += e0.elapsed_time(e1)
        step += chunk
        if step - 1 >= args.burn:
            eng.stats_accumulate()
    prof, count = eng.stats_accumulated()
    m1 = float((eng.get_state().sum(axis=-1) * w).sum())
    eng.close()
    return dict(prof=prof, count=count, mlups=n * args.steps / (t_dev / 1e3) / 1e6, mass_drift=(m1 - m0) / m0,
                utau=meta["utau"])


def errors(p, ref, utau):
    Up, Ur = p[:, 2] / utau, ref[:, 2] / utau
    uwp, uwr = p[:, 3] / utau ** 2, ref[:, 3] / utau ** 2
    rp, rr = np.sqrt(np.maximum(p[:, 8], 0)) / utau, np.sqrt(np.maximum(ref[:, 8], 0)) / utau
    return {
        "U+": float(np.linalg.norm(Up - Ur) / np.linalg.norm(Ur)),
        "uw+": float(np.max(np.abs(uwp - uwr)) / max(np.max(np.abs(uwr)), 1e-300)),
        "urms+": float(np.linalg.norm(rp - rr) / max(np.linalg.norm(rr), 1e-300)),
        "U+_centre_fp64": float(Ur[len(Ur) // 2]),
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--nx", type=int, default=128)
    ap.add_argument("--ny", type=int, default=128)
    ap.add_argument("--nz", type=int, default=256)
    ap.add_argument("--steps", type=int, default=5000)
    ap.add_argument("--every", type=int, default=10)
    ap.add_argument("--burn", type=int, default=1000)
    ap.add_argument("--forms", default="fp64,fp32,fp16,bf16")
    ap.add_argument("--pert", type=float, default=1e-12, help="relative perturbation of the fp64p start")
    ap.add_argument("--seed", type=int, default=1, help="seed of the fp64p perturbation")
    ap.add_argument("--start", default="", help="start every form from this state (dump order, float64 .npy, "
                    "e.g. a turbulent state from channel_spinup.py) instead of the seeded start")
    ap.add_argument("--save", default="", help="write the time-averaged profiles of every form to this .npz")
    ap.add_argument("--ref", default="", help="take the FP64 (and fp64p) results from a --save file of the "
                    "same workload instead of running them")
    args = ap.parse_args()
    forms = args.forms.split(",")
    t0 = time.time()
    res = {}
    if args.ref:
        z = np.load(args.ref)
        for p in ("fp64", "fp64p"):
            if p in z.files:
                get = lambda key, d: float(z[key]) if key in z.files else d  # noqa: E731
                res[p] = dict(prof=z[p], count=int(get(p + "_count", 0)), mlups=get(p + "_mlups", float("nan")),
                              mass_drift=get(p + "_mass", float("nan")), utau=float(z["utau"]))
        forms = [p for p in ("fp64", "fp64p") if p in res] + [p for p in forms if p not in res]
    for p in forms:
        if p not in res:
            res[p] = run_form(p, args)
    ref = res["fp64"]
    out = {"workload": f"channel Re_tau=180 {args.nz}x{args.nx}x{args.ny} (stream x wall x span), tanh mesh",
           "start": args.start or "seeded perturbed laminar start",
           "steps": args.steps, "burn": args.burn, "every": args.every, "samples": ref["count"],
           "wall_s": time.time() - t0, "forms": {}}
    if "fp64p" in forms:
        out["pert"] = args.pert
    for p in forms:
        r = res[p]
        d = {"mlups": r["mlups"], "mass_drift": r["mass_drift"], "speedup_vs_fp64": r["mlups"] / ref["mlups"]}
        if p != "fp64":
            d.update(errors(r["prof"], ref["prof"], ref["utau"]))
        out["forms"][p] = d
    if args.save:
        arrs = {}
        for p in forms:
            arrs[p] = np.asarray(res[p]["prof"])
            arrs[p + "_count"] = res[p]["count"]
            arrs[p + "_mlups"] = res[p]["mlups"]
            arrs[p + "_mass"] = res[p]["mass_drift"]
        np.savez(args.save, utau=ref["utau"], **arrs)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
