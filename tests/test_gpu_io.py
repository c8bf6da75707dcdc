"""Dump / restart, statistics files and the host driver (src/output.cu:22-89,
223-334, src/main.cu:14-56) through the C ABI and the dugks_gb300 binary.

- a dump holds the state in dump order (interior cells, 19 populations
  fastest, double for FP64 and float for FP32 as the reference's PREC4 build);
- restarting from it continues the run bit for bit (FP64);
- dg_output_2d appends one diag.dat line and one profiles-2.dat block with the
  values of dg_stats_values, and writes the three Tecplot slices;
- the host driver's loop produces the same dump as the ABI loop.
"""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

import pydugks  # noqa: E402
from _cases import CASES  # noqa: E402
from seeded import seeded_state  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
DRIVER = os.path.join(HERE, "..", "dugks-gpu_gb300", "dugks_gb300")


def _cfg(case="walls", **over):
    kw = dict(CASES[case])
    kw.update(over)
    return pydugks.make_config(**kw)


@pytest.mark.parametrize("prec,dtype", [("fp64", np.float64), ("fp32", np.float32)])
def test_dump_holds_the_state_in_dump_order(tmp_path, prec, dtype):
    eng = pydugks.Engine(_cfg(precision=prec), workdir=str(tmp_path))
    f0 = seeded_state(eng.nx, eng.ny, eng.nz, seed=5)
    eng.set_state(f0)
    eng.run(1, 3)
    eng.dump(3)
    want = eng.get_state()
    raw = np.fromfile(tmp_path / "ddf00000003.dat", dtype=dtype)
    assert raw.size == eng.nx * eng.ny * eng.nz * 19
    got = raw.reshape(eng.nz, eng.ny, eng.nx, 19).astype(np.float64)
    if prec == "fp64":
        assert np.array_equal(got, want)
    else:
        assert np.array_equal(got, want.astype(np.float32).astype(np.float64))
    eng.close()


@pytest.mark.parametrize("case", ["walls", "stretched"])
def test_restart_continues_bit_for_bit(tmp_path, case):
    f0 = seeded_state(*[CASES[case][k] for k in ("nx", "ny", "nz")], seed=6)
    # straight run of 10 steps
    a = pydugks.Engine(_cfg(case), workdir=str(tmp_path))
    a.set_state(f0)
    a.run(1, 10)
    want = a.get_state()
    a.close()
    # 5 steps, dump, restart from the dump, 5 more
    b = pydugks.Engine(_cfg(case), workdir=str(tmp_path))
    b.set_state(f0)
    b.run(1, 5)
    b.dump(5)
    b.close()
    c = pydugks.Engine(_cfg(case, restart=1, nrestart=5, istep0=6), workdir=str(tmp_path))
    assert c.info.istep0 == 6
    c.run(6, 5)
    got = c.get_state()
    c.close()
    assert np.array_equal(got, want)


def test_output_2d_writes_the_statistics_files(tmp_path):
    eng = pydugks.Engine(_cfg("walls"), workdir=str(tmp_path))
    eng.set_state(seeded_state(eng.nx, eng.ny, eng.nz, seed=7))
    eng.run(1, 4)
    eng.output_2d(4)
    diag, prof = eng.stats_values()
    lines = (tmp_path / "diag.dat").read_text().splitlines()
    assert len(lines) == 1
    cols = lines[0].split()
    assert int(cols[0]) == 4 and len(cols) == 13
    np.testing.assert_allclose([float(c) for c in cols[1:]], diag[:12], rtol=1e-7, atol=1e-12)
    block = (tmp_path / "profiles-2.dat").read_text().splitlines()
    assert int(block[0]) == 4 and len(block) == 1 + eng.nx
    rows = np.array([[float(c) for c in l.split()] for l in block[1:]])
    np.testing.assert_allclose(rows, np.asarray(prof).reshape(eng.nx, 9), rtol=1e-7, atol=1e-12)
    for tag, n in (("s2X", eng.ny * eng.nz), ("s2Y", eng.nx * eng.nz), ("s2Z", eng.nx * eng.ny)):
        text = (tmp_path / f"{tag}00000004.tec").read_text().splitlines()
        assert text[1].startswith("VARIABLES") and len(text) == 3 + n
        assert all(len(l.split()) == 7 for l in text[3:])
    eng.close()


def test_host_driver_matches_the_abi_loop(tmp_path):
    if not os.path.exists(DRIVER):
        pytest.skip("host driver not built")
    cfg = _cfg("walls", nsteps=6, noutput2=3, ndump=6, istep0=1)
    (tmp_path / "drv").mkdir()
    (tmp_path / "abi").mkdir()
    (tmp_path / "drv" / "config.txt").write_text(cfg)
    r = subprocess.run([DRIVER, "config.txt", "--quiet"], cwd=tmp_path / "drv", capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    assert "Main loop time" in r.stdout
    eng = pydugks.Engine(cfg, workdir=str(tmp_path / "abi"))
    for istep in range(1, 7):
        eng.step(istep)
        if istep == 1 or istep % 3 == 0:
            eng.output_2d(istep)
        if istep % 6 == 0:
            eng.dump(istep)
    eng.close()
    a = (tmp_path / "drv" / "ddf00000006.dat").read_bytes()
    b = (tmp_path / "abi" / "ddf00000006.dat").read_bytes()
    assert a == b
    assert (tmp_path / "drv" / "diag.dat").read_text() == (tmp_path / "abi" / "diag.dat").read_text()
    assert len((tmp_path / "drv" / "diag.dat").read_text().splitlines()) == 3  # steps 1, 3, 6


def test_host_driver_writes_the_profiles_fixture_the_reference_script_read(tmp_path):
    """The host driver on tests/golden/laminar_profiles_config.txt writes profiles-2.dat
    byte for byte as tests/golden/laminar_profiles-2.dat, the file that the reference's
    own ProcessProfiles.py was run on (tests/test_postprocessing.py)."""
    if not os.path.exists(DRIVER):
        pytest.skip("host driver not built")
    golden = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    with open(os.path.join(golden, "laminar_profiles_config.txt")) as fh:
        (tmp_path / "config.txt").write_text(fh.read())
    r = subprocess.run([DRIVER, "config.txt", "--quiet"], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    with open(os.path.join(golden, "laminar_profiles-2.dat"), "rb") as fh:
        assert (tmp_path / "profiles-2.dat").read_bytes() == fh.read()
