"""Parity at the benchmark workloads' own sizes: every form of the step on the
full grids against the oracle, which is set up from the config text alone
(mesh, time step, coefficients and initial state restated from the reference
and from the seeded-start definition; nothing taken from the engine).

  channel Re_tau=180, 256 x 128 (tanh) x 128      FP64, FP32, FP16, BF16
  channel 192 x 128 (tanh) x 96                     FP32
  Taylor-Green 64^3, u0 = 0.05, Re = 1600           FP64, FP32
  laminar channel 32 x 64 (walls) x 32              FP64

Tolerances (max |a-b| / max |b| over f-tilde): FP64 1e-12 (the bound of the
reference comparison); FP32 2e-5 (as for the reference's PREC4 build); the
16-bit forms 3 storage quanta of the largest deviation from the rest
equilibrium, as in tests/test_gpu_mixed.py.  The oracle takes about a third of
a second per step of the 4.2 M-cell channel on 16 host cores, so the channel
runs a few steps and the smaller grids more.
"""
import numpy as np
import pytest

import pydugks
import pyoracle
import workloads
from seeded import rel_err

pytestmark = pytest.mark.gpu

QUANT = {"fp16": 2.0 ** -11, "bf16": 2.0 ** -8}
W = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)


def _parity(cfg, nsteps, oracle_dtype=np.float64):
    """(engine state, oracle state, engine initial state) after nsteps from each side's own start."""
    orc = pyoracle.Oracle.from_config(cfg, dtype=oracle_dtype)
    with pydugks.Engine(cfg) as eng:
        f0 = eng.get_state()
        eng.run(1, nsteps)
        eng.sync()
        got = eng.get_state()
    g = pyoracle.to_ghosted(orc.initial_state(), dtype=oracle_dtype)
    orc.run(g, 1, nsteps)
    return got, pyoracle.interior(g).astype(np.float64), f0


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-12), ("fp32", 2e-5)])
def test_channel_re_tau_180_full_grid(prec, tol):
    cfg = workloads.channel_config(precision=prec)[0]
    got, want, _ = _parity(cfg, 3, np.float64 if prec == "fp64" else np.float32)
    err = rel_err(got, want)
    print(f"channel 256x128x128 tanh {prec}, 3 steps: rel err {err:.3e}")
    assert err <= tol


@pytest.mark.parametrize("prec", ["fp16", "bf16"])
def test_channel_re_tau_180_full_grid_16bit(prec):
    cfg = workloads.channel_config(precision=prec)[0]
    got, want, f0 = _parity(cfg, 3)
    err = rel_err(got, want)
    bound = 3.0 * QUANT[prec] * max(1e-3, float(np.max(np.abs(f0 - W) / W)))
    print(f"channel 256x128x128 tanh {prec}, 3 steps: rel err {err:.3e} (bound {bound:.3e})")
    assert err <= bound


def test_channel_192x128x96_fp32():
    cfg = workloads.channel_config(nx=128, ny=96, nz=192, precision="fp32")[0]
    got, want, _ = _parity(cfg, 4, np.float32)
    err = rel_err(got, want)
    print(f"channel 192x128x96 tanh fp32, 4 steps: rel err {err:.3e}")
    assert err <= 2e-5


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-12), ("fp32", 2e-5)])
def test_taylor_green_64(prec, tol):
    cfg = workloads.taylor_green_config(precision=prec)
    got, want, _ = _parity(cfg, 40, np.float64 if prec == "fp64" else np.float32)
    err = rel_err(got, want)
    print(f"Taylor-Green 64^3 u0=0.05 {prec}, 40 steps: rel err {err:.3e}")
    assert err <= tol


def test_laminar_channel():
    cfg = workloads.laminar_config()
    got, want, _ = _parity(cfg, 200)
    err = rel_err(got, want)
    print(f"laminar channel 64x32x32 fp64, 200 steps: rel err {err:.3e}")
    assert err <= 1e-12
