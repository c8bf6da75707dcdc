#!/usr/bin/env python3
"""Spin-up of the Re_tau = 180 channel to a turbulent state.

Runs the benchmark channel (tanh wall-normal mesh, seeded perturbed laminar
start) in one form with the reference's own turbulence trigger, the
perturbation body force of src/dugks.cu:1086-1126 (perturb=1), for
`--perturb-steps` steps, then without it, and prints a trajectory of the
instantaneous plane-averaged statistics every `--chunk` steps:

  Uc+     centreline mean velocity / u_tau
  uw+     max |<u'w'>| / u_tau^2        (about 0.7 in a developed Re_tau=180 channel)
  urms+   max sqrt(<u'u'>) / u_tau      (about 2.6)

The final state is saved (dump order, float64, .npy) for
verify_mixed.py --start, which branches every precision form from it.

  python dugks-gpu_gb300/channel_spinup.py --steps 400000 --perturb-steps 150000 --out start.npy
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


def snapshot(eng, utau):
    _, prof = eng.stats_values()          # per x: u v w <uw>' <uv>' <vw>' <u'u'> <v'v'> <w'w'>
    w = prof[:, 2] / utau                 # streamwise = z
    uw = prof[:, 3] / utau ** 2
    urms = np.sqrt(np.maximum(prof[:, 8], 0)) / utau
    return {"Uc+": float(w[len(w) // 2]), "uw+": float(np.max(np.abs(uw))), "urms+": float(np.max(urms))}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--nx", type=int, default=128)
    ap.add_argument("--ny", type=int, default=128)
    ap.add_argument("--nz", type=int, default=256)
    ap.add_argument("--precision", default="fp32")
    ap.add_argument("--steps", type=int, default=400000)
    ap.add_argument("--perturb-steps", type=int, default=150000)
    ap.add_argument("--chunk", type=int, default=20000)
    ap.add_argument("--out", default="")
    args = ap.parse_args()
    import torch
    t0 = time.time()
    cfg, meta = pydugks.channel_config(nx=args.nx, ny=args.ny, nz=args.nz, precision=args.precision)
    utau = meta["utau"]
    eng = pydugks.Engine(cfg.replace("perturb=0", "perturb=1"))
    eng.set_stream(torch.cuda.current_stream().cuda_stream)
    traj = []
    step = 1
    while step <= args.steps:
        if step > args.perturb_steps and eng.info.perturb:
            f = eng.get_state()
            eng.close()
            eng = pydugks.Engine(cfg)
            eng.set_stream(torch.cuda.current_stream().cuda_stream)
            eng.set_state(f)
        stop = args.perturb_steps + 1 if step <= args.perturb_steps else args.steps + 1
        n = min(args.chunk, stop - step)
        eng.run(step, n)
        eng.sync()
        step += n
        rec = {"step": step - 1, "perturb": int(eng.info.perturb), **snapshot(eng, utau)}
        traj.append(rec)
        print(json.dumps(rec), flush=True)
    if args.out:
        np.save(args.out, eng.get_state())
    print(json.dumps({"workload": f"channel Re_tau=180 {args.nz}x{args.nx}x{args.ny}, {args.precision}",
                      "steps": args.steps, "perturb_steps": args.perturb_steps, "wall_s": time.time() - t0,
                      "final": traj[-1]}))


if __name__ == "__main__":
    main()
