"""The legacy-name libraries (include/dugks_legacy.h: init_dugks, dugks_step,
upload_macro, copy_vel, copy_ddf and the h_rho, h_ux, h_uy, h_uz, h_f
globals of src/dugks.h:1-9) driven the way src/main.cu:16-43 drives them, by
tests/legacy_main.cpp compiled here against them.

Checked: the dumps are byte-identical to those of the handle API's own driver
(dugks_gb300) on the same config.txt and within 1e-12 (FP64) / 2e-5 (PREC4)
of the oracle; the macro arrays equal dg_copy_vel's; a restart from a dump
(restart=1, nrestart) continues bit-identically.  The reference's own
src/main.cu linked against these libraries is checked on the CPU
(tests/test_legacy_link.py): only a host of the build machine's kind can run
that binary.
"""
import os
import subprocess

import numpy as np
import pytest

import pydugks
import pyoracle
from seeded import rel_err

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "dugks-gpu_gb300")
DRIVER = os.path.join(PKG, "dugks_gb300")
NX, NY, NZ = 32, 8, 6


def _config(**over):
    kw = dict(case="channel", nx=NX, ny=NY, nz=NZ, xwidth=NX, ywidth=NY, zwidth=NZ, periods_x=0, CFL=0.7,
              visc=0.166, ambient_fz=3.2421875e-5, istep0=1, nsteps=20, noutput2=10, ndump=10)
    kw.update(over)
    return pydugks.make_config(**kw)


def _build(tmp_path, prec4):
    exe = tmp_path / ("legacy_main_prec4" if prec4 else "legacy_main")
    lib = "dugks_legacy_prec4" if prec4 else "dugks_legacy"
    cmd = ["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), "-o", str(exe),
           os.path.join(ROOT, "tests", "legacy_main.cpp"), "-L", PKG, f"-l{lib}", f"-Wl,-rpath,{PKG}"]
    if prec4:
        cmd.insert(1, "-DPREC4")
    subprocess.run(cmd, check=True)
    return str(exe)


def _run_legacy(exe, wd, cfg, istep0=1, nsteps=20):
    os.makedirs(wd, exist_ok=True)
    with open(os.path.join(wd, "config.txt"), "w") as fh:
        fh.write(cfg)
    r = subprocess.run([exe, str(NX), str(NY), str(NZ), str(istep0), str(nsteps), "10", "10"], cwd=wd,
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr


def _run_driver(wd, cfg):
    os.makedirs(wd, exist_ok=True)
    with open(os.path.join(wd, "config.txt"), "w") as fh:
        fh.write(cfg)
    r = subprocess.run([DRIVER, "config.txt", "--quiet"], cwd=wd, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr


def _oracle_after(cfg, nsteps, dtype):
    orc = pyoracle.Oracle.from_config(cfg, dtype=dtype)
    g = pyoracle.to_ghosted(orc.initial_state(), dtype=dtype)
    orc.run(g, 1, nsteps)
    return pyoracle.interior(g).astype(np.float64)


def test_legacy_driver_equals_the_engine_driver_and_the_oracle(tmp_path):
    exe = _build(tmp_path, prec4=False)
    cfg = _config()
    _run_legacy(exe, str(tmp_path / "legacy"), cfg)
    _run_driver(str(tmp_path / "driver"), cfg)
    for step in (10, 20):
        a = (tmp_path / "legacy" / f"ddf{step:08d}.dat").read_bytes()
        b = (tmp_path / "driver" / f"ddf{step:08d}.dat").read_bytes()
        assert len(a) == NX * NY * NZ * 19 * 8 and a == b, step
    got = np.fromfile(tmp_path / "legacy" / "ddf00000020.dat", dtype=np.float64).reshape(NZ, NY, NX, 19)
    err = rel_err(got, _oracle_after(cfg, 20, np.float64))
    print(f"legacy FP64 driver vs oracle after 20 steps: {err:.2e}")
    assert err <= 1e-12
    # macro arrays at step 10 equal dg_copy_vel after the same steps
    mac = np.fromfile(tmp_path / "legacy" / "macro00000010.dat", dtype=np.float64).reshape(4, NZ + 2, NY + 2, NX + 2)
    with pydugks.Engine(cfg) as eng:
        eng.run(1, 10)
        want = eng.copy_vel()
    for a, b in zip(mac, want):
        assert np.array_equal(a, b)


def test_legacy_restart_continues_bit_identically(tmp_path):
    exe = _build(tmp_path, prec4=False)
    wd = str(tmp_path / "run")
    _run_legacy(exe, wd, _config())
    full = (tmp_path / "run" / "ddf00000020.dat").read_bytes()
    os.remove(os.path.join(wd, "ddf00000020.dat"))
    _run_legacy(exe, wd, _config(restart=1, nrestart=10, istep0=11, nsteps=10), istep0=11, nsteps=10)
    assert (tmp_path / "run" / "ddf00000020.dat").read_bytes() == full


def test_legacy_prec4_equals_the_fp32_engine_and_the_fp32_oracle(tmp_path):
    exe = _build(tmp_path, prec4=True)
    cfg = _config()
    _run_legacy(exe, str(tmp_path / "legacy"), cfg)
    _run_driver(str(tmp_path / "driver"), cfg + "precision=fp32\n")
    a = (tmp_path / "legacy" / "ddf00000020.dat").read_bytes()
    b = (tmp_path / "driver" / "ddf00000020.dat").read_bytes()
    assert len(a) == NX * NY * NZ * 19 * 4 and a == b
    got = np.frombuffer(a, dtype=np.float32).reshape(NZ, NY, NX, 19)
    err = rel_err(got, _oracle_after(cfg, 20, np.float32))
    print(f"legacy PREC4 driver vs FP32 oracle after 20 steps: {err:.2e}")
    assert err <= 2e-5
