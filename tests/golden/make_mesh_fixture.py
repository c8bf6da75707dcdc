"""Copies the reference's tanh mesh (src/fortran/channel/run/mesh.txt: 129 face
positions for nx=128, zsize=61.72, alpha=0.85, written by run/mesh.py) into
tests/golden/mesh_tanh_128.txt as a golden vector for the engine's mesh
generator.  Run where the reference is mounted, with its root as the argument:
    python tests/golden/make_mesh_fixture.py REFERENCE_ROOT
"""
import os
import sys

if len(sys.argv) != 2:
    sys.exit("usage: python tests/golden/make_mesh_fixture.py REFERENCE_ROOT")
ref = sys.argv[1]
src = os.path.join(ref, "src/fortran/channel/run/mesh.txt")
vals = [float(l) for l in open(src) if l.strip()]
assert len(vals) == 129
out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "mesh_tanh_128.txt")
with open(out, "w") as f:
    f.write("# face positions of the reference's tanh mesh: nx=128 zsize=61.72 alpha=0.85\n")
    for v in vals:
        f.write(repr(v) + "\n")
print("wrote", out)
