"""The legacy-name libraries on the CPU: they export the reference's names
(src/dugks.h:1-9) with its C++ linkage, and the reference's own unmodified
src/main.cu, numerics.cu, parallel.cu, cuda.cu, checks.cu, output.cu and
lbm_d3q19.cu link against them in place of src/dugks.cu
(oracle/_ref/ref_main_legacy*, built by oracle/build_ref.sh where the
reference sources are mounted).  The binary is not run here: without a GPU
the reference's src/cuda.cu:26-32 loops over an uninitialised device count.
The legacy libraries' behaviour is checked on the GPU
(tests/test_gpu_legacy.py)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "dugks-gpu_gb300")
REF = os.path.join(ROOT, "oracle", "_ref")

FUNCS = ["_Z10init_dugksv", "_Z10dugks_stepi", "_Z12upload_macrov", "_Z8copy_velv", "_Z8copy_ddfv"]
GLOBALS = ["h_rho", "h_ux", "h_uy", "h_uz", "h_f"]


def _symbols(path, *flags):
    r = subprocess.run(["nm", "-D", *flags, path], capture_output=True, text=True, check=True)
    return {line.split()[-1]: line.split()[-2] for line in r.stdout.splitlines() if line.strip()}


@pytest.mark.parametrize("lib", ["libdugks_legacy.so", "libdugks_legacy_prec4.so"])
def test_legacy_library_exports_the_reference_names(lib):
    if shutil.which("nm") is None:
        pytest.skip("nm not available")
    syms = _symbols(os.path.join(PKG, lib), "--defined-only")
    for name in FUNCS:
        assert syms.get(name) == "T", name
    for name in GLOBALS:
        assert syms.get(name) in ("B", "D"), name


@pytest.mark.parametrize("exe,objs", [("ref_main_legacy", "legacy_f64"), ("ref_main_legacy_prec4", "legacy_prec4")])
def test_reference_main_links_unchanged_against_the_legacy_library(exe, objs):
    path = os.path.join(REF, exe)
    if not os.path.exists(path):
        pytest.skip("the reference's driver is built only where its sources are mounted")
    if shutil.which("nm") is None or shutil.which("readelf") is None:
        pytest.skip("binutils not available")
    # the reference's objects use the names and define none of them (src/dugks.cu is not among them)
    defined, used = set(), set()
    odir = os.path.join(REF, objs)
    for o in sorted(os.listdir(odir)):
        for line in subprocess.run(["nm", os.path.join(odir, o)], capture_output=True, text=True,
                                   check=True).stdout.splitlines():
            parts = line.split()
            (used if parts[-2] == "U" else defined).add(parts[-1])
    assert {"main", "_Z4dumpiPKd" if objs == "legacy_f64" else "_Z4dumpiPKf"} <= defined
    for name in FUNCS + GLOBALS:
        assert name not in defined, name
    assert {"_Z10init_dugksv", "_Z10dugks_stepi", "h_f"} <= used   # src/main.cu:20,31,42
    # the executable needs the legacy library and leaves the functions to it
    dyn = subprocess.run(["readelf", "-d", path], capture_output=True, text=True, check=True).stdout
    lib = "libdugks_legacy_prec4.so" if "prec4" in exe else "libdugks_legacy.so"
    assert f"[{lib}]" in dyn
    undefined = subprocess.run(["nm", "-u", path], capture_output=True, text=True, check=True).stdout.split()
    for name in ("_Z10init_dugksv", "_Z10dugks_stepi", "_Z12upload_macrov", "_Z8copy_velv", "_Z8copy_ddfv"):
        assert name in undefined, name
