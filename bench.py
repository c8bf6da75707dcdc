#!/usr/bin/env python3
"""DUGKS D3Q19 step throughput (MLUPS) on GB300.

Workload: turbulent channel at Re_tau = 180, 256 (streamwise) x 128 (wall-
normal, tanh-stretched, first cell centre at y+ = 0.5) x 128 (spanwise)
cells, in the reference orientation (walls on the x faces, streamwise z:
nx=128, ny=128, nz=256).  Seeded synthetic initial state (laminar profile +
perturbations + near-wall streaks); the reference's Zenodo restart dumps are
not available.  A step is one full DUGKS step (stage (a) f-bar-plus, ghost
formation, reconstruction, face fluxes, update) over the whole grid.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--precision fp64|fp32|fp16|bf16]
  python bench.py --impl reference ...   # the step on the host cores (CPU port of the reference)

Prints one JSON line (rank 0).  Under torchrun (N>1) every rank advances its
own replica (the step does not shard across GPUs here): weak scaling, no
data-path collective.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "dugks-gpu_gb300"))

CLOCK_FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=("ours", "reference"))
    ap.add_argument("--precision", default="fp64", choices=("fp64", "fp32", "fp16", "bf16"))
    ap.add_argument("--grid", default="128,128,256", help="nx,ny,nz in the reference orientation")
    ap.add_argument("--no-extras", action="store_true", help="skip the CPU baseline, other forms and reference-GPU legs")
    return ap.parse_args()


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def workload(args, precision):
    import workloads
    nx, ny, nz = (int(v) for v in args.grid.split(","))
    cfg, meta = workloads.channel_config(nx=nx, ny=ny, nz=nz, precision=precision)
    return cfg, meta, (nx, ny, nz)


def bench_config(args, meta, grid, world):
    """The `config` object of the JSON line, the same for both arms."""
    n = grid[0] * grid[1] * grid[2]
    return {"workload": describe(grid, args.precision), "grid_nx_ny_nz": list(grid), "mesh": "tanh",
            "re_tau": 180, "nu": meta["nu"], "alpha": meta["alpha"], "parallelism": f"replicas x{world}",
            "l2": "inputs larger than L2 (f and f-bar-plus resident, %d MB each)"
                  % (n * 19 * {"fp64": 8, "fp32": 4}.get(args.precision, 2) // 2**20),
            "structure": "two-pass (stage a kernel, flux+update kernel)"}


def oracle_setup(cfg_text):
    """The oracle and the initial state of a workload, from the config text alone
    (the oracle's own restatement of the mesh, coefficients and the seeded start;
    nothing of the engine library is loaded)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    orc = pyoracle.Oracle.from_config(cfg_text)
    return orc, pyoracle.to_ghosted(orc.initial_state())


def describe(grid, precision):
    nx, ny, nz = grid
    return (f"DUGKS D3Q19 turbulent channel Re_tau=180, {nz}(streamwise) x {nx}(wall-normal, tanh-stretched) x "
            f"{ny}(spanwise), {precision}")


class ClockSampler:
    def __init__(self, gpu_index):
        self.proc = None
        self.path = None
        self.gpu = gpu_index

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={CLOCK_FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), float(parts[3]), parts[5:9]))
            except ValueError:
                continue
        os.unlink(self.path)
        if not rows:
            return None
        sm = sorted(r[0] for r in rows)
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        reasons = sorted({names[i] for r in rows for i, v in enumerate(r[3]) if v.lower().startswith("active")})
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": max(r[1] for r in rows),
                "power_w_max": max(r[2] for r in rows), "samples": len(rows), "reasons": reasons}


def measured_peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def launches_per_step(precision, periodic_x):
    """Kernel launches of one step: stage (a), the flux kernel and, in FP64 and
    the 16-bit forms with periodic x, the separate ghost pass of f-bar-plus."""
    if precision == "fp32" or (precision in ("fp16", "bf16") and not periodic_x):
        return 2
    return 3


def ncu_traffic(precision, grid):
    """DRAM bytes per flux launch from the committed ncu capture of the same
    grid and form (profiles/traffic.json, written from an ncu capture; ncu
    cannot run inside this process), with the capture it comes from; None when
    no capture of this grid exists."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        d = json.load(open(p))
    except Exception:
        return None, None
    e = d.get("flux", {}).get(precision)
    if not e or list(e.get("grid_nx_ny_nz", [])) != list(grid):
        return None, None
    return e["dram_bytes"], {"source": "profiles/traffic.json (committed ncu capture, not measured in this run)",
                             "kernel": e["kernel"], "command": d.get("command")}


def fp64_inst_per_cell(kernel):
    """FP64 thread instructions per cell of `kernel` from the committed ncu capture."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        return json.load(open(p))["fp64_inst_per_cell"][kernel]
    except Exception:
        return None


def fp64_pipe_peak(stream):
    """FP64 FMA thread instructions per second, measured now (dugks-gpu_gb300/libdg_peak.so)."""
    import ctypes
    L = ctypes.CDLL(os.path.join(ROOT, "dugks-gpu_gb300", "libdg_peak.so"))
    L.dg_probe_fp64_fma_rate.restype = ctypes.c_int
    L.dg_probe_fp64_fma_rate.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
    rate = ctypes.c_double(0.0)
    rc = L.dg_probe_fp64_fma_rate(ctypes.c_void_p(stream), 20, ctypes.byref(rate))
    if rc != 0:
        raise RuntimeError(f"FP64 probe failed with CUDA error {rc}")
    return rate.value


def combine_ranks(world, n_cells, steps, ms_local, dist=None, device="cpu"):
    """Whole-job MLUPS of `world` replicas: every rank advanced n_cells for
    `steps` steps; the job time is the maximum over ranks."""
    ms = float(ms_local)
    if dist is not None and world > 1:
        import torch
        t = torch.tensor([ms], device=device, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    return world * n_cells * steps / (ms / 1e3) / 1e6, ms


def time_steps(eng, istep0, k):
    import torch
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    ms_a, ms_b = eng.run_profiled(istep0, k)
    e1.record()
    e1.synchronize()
    return e0.elapsed_time(e1), ms_a, ms_b


def run_form(args, precision, k, w):
    """Device-resident timing of one form; returns (MLUPS, ms/step, ms_a, ms_b)."""
    import pydugks
    import torch
    cfg, _, grid = workload(args, precision)
    with pydugks.Engine(cfg) as eng:
        eng.set_stream(torch.cuda.current_stream().cuda_stream)
        eng.run(1, w)
        eng.sync()
        ms, ms_a, ms_b = time_steps(eng, w + 1, k)
        eng.sync()  # raises on a kernel-reported error (e.g. a timed-out TMA wait)
        n = grid[0] * grid[1] * grid[2]
        return n * k / (ms / 1e3) / 1e6, ms / k, ms_a / k, ms_b / k


def cpu_baseline(args, budget_s=12.0):
    """The oracle (CPU port of the reference step, OpenMP over all host cores) on
    the same workload; a bounded number of full-grid steps."""
    cfg, _, grid = workload(args, "fp64")
    orc, g = oracle_setup(cfg)
    import pyoracle
    threads = pyoracle.max_threads()
    t = time.perf_counter()
    orc.run(g, 1, 1, threads)
    t1 = time.perf_counter() - t
    steps = max(1, min(50, int(budget_s / max(t1, 1e-3))))
    t = time.perf_counter()
    orc.run(g, 2, steps, threads)
    dt = time.perf_counter() - t
    n = grid[0] * grid[1] * grid[2]
    return {"value": n * steps / dt / 1e6, "unit": "MLUPS", "cores": threads, "kind": "port",
            "sample": f"{steps} full-grid FP64 steps of the same workload (after 1 untimed step), "
                      f"oracle/dugks_oracle.c with OpenMP"}


def other_configs(k=200, w=3, cpu_budget_s=3.0):
    """MLUPS of the other single-GPU workloads (they fit in L2, so MLUPS only):
    the laminar channel (32 x 64 x 32, walls at the wall-normal faces; in the
    reference orientation 64 wall-normal x 32 x 32) and the Taylor-Green vortex
    (64^3 periodic, u0 = 0.05 in the velocity and the density term, Re = 1600),
    FP64 and FP32 on the GPU and the oracle (FP64, OpenMP) on the host cores for
    a bounded number of steps."""
    import pydugks
    import torch
    import workloads
    cases = {"laminar channel 32x64x32": workloads.laminar_config,
             "Taylor-Green 64^3 u0=0.05 Re=1600": workloads.taylor_green_config}
    out = {}
    for name, make in cases.items():
        res = {}
        for prec in ("fp64", "fp32"):
            with pydugks.Engine(make(precision=prec)) as eng:
                eng.set_stream(torch.cuda.current_stream().cuda_stream)
                eng.run(1, w)
                eng.sync()
                ms = time_steps(eng, w + 1, k)[0]
                eng.sync()
                res[prec + "_mlups"] = eng.nx * eng.ny * eng.nz * k / (ms / 1e3) / 1e6
        orc, g = oracle_setup(make(precision="fp64"))
        import pyoracle
        n = orc.cfg.nx * orc.cfg.ny * orc.cfg.nz
        threads = pyoracle.max_threads()
        t = time.perf_counter()
        orc.run(g, 1, 1, threads)
        steps = max(1, min(400, int(cpu_budget_s / max(time.perf_counter() - t, 1e-4))))
        t = time.perf_counter()
        orc.run(g, 2, steps, threads)
        res["cpu_port_mlups"] = n * steps / (time.perf_counter() - t) / 1e6
        res["cpu_port_sample"] = f"{steps} steps, {threads} threads"
        out[name] = res
    return out


def reference_gpu(args, k=10):
    """The reference's own CUDA-C kernels (oracle/_ref cubins, FP64 and its
    PREC4 FP32 build) on the uniform-mesh variant of the same grid (the
    reference has no stretched mesh), parameters parsed from the same
    config.txt text as the reference would (std::stof)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import numpy as np
    import pyoracle
    if not pyoracle.ref_cubins_present():
        return None
    cfg, _, (nx, ny, nz) = workload(args, "fp64")
    kv = dict(l.split("=", 1) for l in cfg.splitlines() if "=" in l)
    st = lambda key: float(np.float32(float(kv[key])))  # noqa: E731
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from seeded import seeded_state  # noqa: E402
    out = {}
    for prec, name in ((0, "fp64"), (1, "fp32")):
        f = pyoracle.to_ghosted(seeded_state(nx, ny, nz, seed=0, umax=0.05, eps=0.001))
        common = dict(periods=(0, 1, 1), prec=prec)
        args_ = (f, nx, ny, nz, st("CFL"), st("xwidth"), st("ywidth"), st("zwidth"), st("visc"),
                 (st("ambient_fx"), st("ambient_fy"), st("ambient_fz")))
        pyoracle.ref_run(*args_, istep0=1, nsteps=2, **common)
        ms = pyoracle.ref_run(*args_, istep0=3, nsteps=k, **common)
        out[name] = {"value": nx * ny * nz / (ms / 1e3) / 1e6, "unit": "MLUPS", "ms_per_step": ms, "steps": k}
    out["what"] = ("reference src/dugks.cu kernels (unmodified, nvcc sm_103a; FP32 = its PREC4 build), "
                   "uniform-mesh variant of the grid, CUDA events around dugks_step's launches")
    return out


def main_reference(args):
    """The reference arm: the reference step on the host cores.  The reference has
    no CPU implementation of its step, so this is the oracle's restatement of it
    (oracle/dugks_oracle.c, OpenMP over every host core), on the same workload
    and config as the GPU arm; its mesh, coefficients and seeded initial state
    come from the oracle's own restatement too, so the engine library is never
    loaded by this arm."""
    world, rank, _ = dist_env()
    if rank != 0:
        return
    cfg, meta, grid = workload(args, "fp64")
    orc, g = oracle_setup(cfg)
    import pyoracle
    threads = pyoracle.max_threads()
    orc.run(g, 1, args.warmup, threads)
    t = time.perf_counter()
    orc.run(g, args.warmup + 1, args.steps, threads)
    dt = time.perf_counter() - t
    n = grid[0] * grid[1] * grid[2]
    value = n * args.steps / dt / 1e6
    line = {"impl": "reference", "metric": "MLUPS", "value": value, "unit": "MLUPS", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": bench_config(args, meta, grid, world),
            "cpu_baseline": {"value": value, "unit": "MLUPS", "cores": threads, "kind": "port",
                             "sample": f"{args.steps} full-grid FP64 steps after {args.warmup} warm-up steps; "
                                       "the reference has no CPU path, so this is the oracle's restatement of "
                                       "its step (oracle/dugks_oracle.c, OpenMP)"},
            "e2e": {"value": value, "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if not args.no_extras:
        try:
            line["reference_gpu"] = reference_gpu(args)
        except Exception as e:
            line["reference_gpu"] = f"error: {e}"
    print(json.dumps(line), flush=True)


def main():
    args = parse_args()
    if args.impl == "reference":
        return main_reference(args)
    import torch
    import pydugks
    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    cfg, meta, grid = workload(args, args.precision)
    n = grid[0] * grid[1] * grid[2]
    K, W = args.steps, max(3, args.warmup)

    eng = pydugks.Engine(cfg)
    eng.set_stream(torch.cuda.current_stream().cuda_stream)
    eng.run(1, W)
    eng.sync()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    ms, ms_a, ms_b = time_steps(eng, W + 1, K)
    clocks = sampler.stop()
    eng.sync()  # raises on a kernel-reported error (a timed-out TMA wait) instead of printing a number
    value, ms = combine_ranks(world, n, K, ms, dist, device="cuda")

    # end to end through the C ABI with host buffers: upload the state from
    # pinned host memory, K steps each followed by a host read of the step's
    # conserved moments, download the final state
    state_bytes = n * 19 * 8
    h_in = torch.empty(n * 19, dtype=torch.float64, pin_memory=True).numpy()
    h_out = torch.empty(n * 19, dtype=torch.float64, pin_memory=True).numpy()
    h_in[:] = eng.get_state().ravel()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    eng.set_state(h_in)
    for s in range(K):
        eng.step(W + K + 1 + s)
        eng.moments()
    eng._check(pydugks.lib().dg_get_state(eng._h, h_out.ctypes.data_as(pydugks._D)))
    eng.sync()
    e2e_s = time.perf_counter() - t0
    e2e = {"value": n * K / e2e_s / 1e6, "unit": "MLUPS",
           "h2d_bytes_per_step": state_bytes / K,
           "d2h_bytes_per_step": state_bytes / K + 608 * 4 * 8,
           "what": "dg_set_state(pinned host) + K x (dg_step + dg_moments host read) + dg_get_state(pinned host)"}
    eng.close()

    info_bytes = {"fp64": 8, "fp32": 4, "fp16": 2, "bf16": 2}[args.precision]
    flux_bytes = 57 * info_bytes * n
    achieved = flux_bytes / (ms_b / K / 1e3) / 1e9
    peak, peak_kind = measured_peak_hbm()
    traffic, traffic_src = ncu_traffic(args.precision, grid)
    roof = {"bound": "hbm", "kernel": "flux_kernel", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "traffic": traffic, "traffic_from": traffic_src,
            "peak_source": peak_kind, "alg_bytes_per_cell": 57 * info_bytes,
            "kernel_ms": {"fbar_kernel": ms_a / K, "flux_kernel": ms_b / K},
            "step_alg_bytes_per_cell": 95 * info_bytes,
            "step_frac": 95 * info_bytes * n * K / (ms / 1e3) / 1e9 / peak}
    if args.precision == "fp64":
        # the FP64 step is bound by FP64 instruction issue: its compute roofline
        per_cell = fp64_inst_per_cell("flux_kernel")
        dp_peak = fp64_pipe_peak(torch.cuda.current_stream().cuda_stream)
        comp = {"bound": "fp64 pipe", "kernel": "flux_kernel", "unit": "T FP64 inst/s", "peak": dp_peak / 1e12,
                "peak_source": "measured in this run: FP64 FMA chains on every SM (libdg_peak.so)",
                "fp64_inst_per_cell": per_cell}
        if per_cell:
            comp["achieved"] = per_cell * n / (ms_b / K / 1e3) / 1e12
            comp["frac"] = comp["achieved"] / comp["peak"]
        roof["compute"] = comp

    extras = {}
    if rank == 0 and world == 1 and not args.no_extras:
        forms = {}
        for p in ("fp64", "fp32", "fp16", "bf16"):
            if p == args.precision:
                forms[p] = value
                continue
            try:
                forms[p] = run_form(args, p, K, W)[0]
            except Exception as e:  # report, do not hide
                forms[p] = f"error: {e}"
        extras["forms_mlups"] = forms
        try:
            extras["cpu_baseline"] = cpu_baseline(args)
        except Exception as e:
            extras["cpu_baseline"] = {"error": str(e)}
        try:
            extras["other_configs"] = other_configs()
        except Exception as e:
            extras["other_configs"] = {"error": str(e)}

    if rank == 0:
        line = {"metric": "MLUPS", "value": value, "unit": "MLUPS", "n_gpus": world, "steps": K, "warmup": W,
                "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": {"fp64": "f64", "fp32": "f32", "fp16": "f16-storage/f32", "bf16": "bf16-storage/f32"}[args.precision],
                "data": "synthetic",
                "config": bench_config(args, meta, grid, world),
                "e2e": e2e, "gpu_launches": launches_per_step(args.precision, periodic_x=False) * K, "roofline": roof, "clocks": clocks}
        line.update(extras)
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
