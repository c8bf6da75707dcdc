"""Runs the reference's own post-processing script
(examples/laminar/ProcessProfiles.py, read where the reference is mounted)
on tests/golden/laminar_profiles-2.dat -- the profiles-2.dat that this
engine's host driver writes for tests/golden/laminar_profiles_config.txt
(the laminar example grid, 2000 steps, a profile block every 500) -- and
stores the VELMEAN.dat the script writes as tests/golden/laminar_velmean.dat.
The script's own configuration module (params.py) is written here for this
file: nz = 64 profile rows, blocks at steps 1..2001 every 500, none ignored.
    python tests/golden/make_velmean_fixture.py REFERENCE_ROOT
"""
import os
import runpy
import shutil
import sys
import tempfile

if len(sys.argv) != 2:
    sys.exit("usage: python tests/golden/make_velmean_fixture.py REFERENCE_ROOT")
HERE = os.path.dirname(os.path.abspath(__file__))
script = os.path.join(sys.argv[1], "examples", "laminar", "ProcessProfiles.py")
with tempfile.TemporaryDirectory() as wd:
    shutil.copy(os.path.join(HERE, "laminar_profiles-2.dat"), os.path.join(wd, "profiles-2.dat"))
    with open(os.path.join(wd, "params.py"), "w") as fh:
        fh.write("istart=1\niend=2000\nstep=500\nignore_before=0\nnz=64\n")
    cwd = os.getcwd()
    sys.path.insert(0, wd)
    os.chdir(wd)
    try:
        runpy.run_path(script, run_name="__main__")
    finally:
        os.chdir(cwd)
    shutil.copy(os.path.join(wd, "VELMEAN.dat"), os.path.join(HERE, "laminar_velmean.dat"))
print("wrote", os.path.join(HERE, "laminar_velmean.dat"))
