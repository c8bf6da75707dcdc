"""Parity with the reference's own CUDA-C kernels.

oracle/_ref/dugks_{f64,f32}.cubin are the reference's unmodified src/dugks.cu
compiled for sm_103a (oracle/build_ref.sh); oracle/ref_runner.cpp launches
them in dugks_step's order (src/dugks.cu:322-391).  These tests pin the CPU
oracle to the reference and check the engine against it directly.
"""
import numpy as np
import pytest

import pydugks
import pyoracle
from seeded import rel_err, seeded_state

pytestmark = pytest.mark.gpu

REF_CASES = {
    # reference orientation: walls in x, force along z (examples/laminar/config.txt)
    "walls": dict(nx=32, ny=8, nz=4, xwidth=32, ywidth=8, zwidth=4, periods_x=0, CFL=0.7, visc=0.166,
                  ambient_fz=3.2421875e-5),
    "periodic": dict(nx=16, ny=16, nz=6, xwidth=16, ywidth=16, zwidth=6, periods_x=1, CFL=0.5, visc=0.01,
                     ambient_fx=1e-5, ambient_fy=2e-5, ambient_fz=0.0),
}


def _need_ref():
    if not pyoracle.ref_cubins_present():
        pytest.skip("reference cubins (oracle/_ref) not built: run oracle/build_ref.sh where the reference is present")


def _ref_args(kw):
    return dict(nx=kw["nx"], ny=kw["ny"], nz=kw["nz"], CFL=float(np.float32(kw["CFL"])),
                xwidth=float(np.float32(kw["xwidth"])), ywidth=float(np.float32(kw["ywidth"])),
                zwidth=float(np.float32(kw["zwidth"])), visc=float(np.float32(kw["visc"])),
                F=tuple(float(np.float32(kw.get(k, 0.0))) for k in ("ambient_fx", "ambient_fy", "ambient_fz")),
                periods=(kw["periods_x"], 1, 1))


@pytest.mark.parametrize("case", sorted(REF_CASES))
@pytest.mark.parametrize("nsteps", [1, 50])
def test_oracle_and_engine_match_reference_fp64(case, nsteps):
    _need_ref()
    kw = dict(REF_CASES[case])
    f0 = seeded_state(kw["nx"], kw["ny"], kw["nz"], seed=3)
    ref = pyoracle.to_ghosted(f0)
    pyoracle.ref_run(ref, **_ref_args(kw), istep0=1, nsteps=nsteps, prec=0)
    eng = pydugks.Engine(pydugks.make_config(**kw))
    eng.set_state(f0)
    eng.run(1, nsteps)
    got = eng.get_state()
    orc = pyoracle.Oracle.from_config(pydugks.make_config(**kw))
    g = pyoracle.to_ghosted(f0)
    orc.run(g, 1, nsteps)
    e_oracle = rel_err(pyoracle.interior(g), pyoracle.interior(ref))
    e_engine = rel_err(got, pyoracle.interior(ref))
    print(f"{case} {nsteps} steps: oracle-vs-ref {e_oracle:.3e}  engine-vs-ref {e_engine:.3e}")
    assert e_oracle <= 1e-13
    assert e_engine <= 1e-12


@pytest.mark.parametrize("case", sorted(REF_CASES))
def test_engine_matches_reference_fp32(case):
    _need_ref()
    kw = dict(REF_CASES[case])
    f0 = seeded_state(kw["nx"], kw["ny"], kw["nz"], seed=4)
    ref = pyoracle.to_ghosted(f0)
    pyoracle.ref_run(ref, **_ref_args(kw), istep0=1, nsteps=20, prec=1)
    eng = pydugks.Engine(pydugks.make_config(precision="fp32", **kw))
    eng.set_state(f0)
    eng.run(1, 20)
    err = rel_err(eng.get_state(), pyoracle.interior(ref))
    print(f"{case} fp32 20 steps engine-vs-ref {err:.3e}")
    assert err <= 2e-5


def test_gradient_option_matches_reference():
    """calc_fx (the central-difference variant): oracle and engine against the reference kernel."""
    _need_ref()
    kw = dict(REF_CASES["walls"])
    f0 = seeded_state(kw["nx"], kw["ny"], kw["nz"], seed=5)
    ref = pyoracle.to_ghosted(f0)
    pyoracle.ref_run(ref, **_ref_args(kw), istep0=1, nsteps=5, prec=0, recon=1)
    cfg = pydugks.make_config(recon="gradient", **kw)
    eng = pydugks.Engine(cfg)
    orc = pyoracle.Oracle.from_config(cfg)
    g = pyoracle.to_ghosted(f0)
    orc.run(g, 1, 5)
    assert rel_err(pyoracle.interior(g), pyoracle.interior(ref)) <= 1e-13
    eng.set_state(f0)
    eng.run(1, 5)
    assert rel_err(eng.get_state(), pyoracle.interior(ref)) <= 1e-12


# Laminar channel of the benchmark configurations in the reference orientation:
# 64 (walls) x 32 x 32 cells, dx = 1, force along z, centreline velocity 0.1,
# Re_c = u_c H / nu = 100 with H = 32 (nu = 0.032), CFL 0.5, rest start f = w_p.
C1 = dict(nx=64, ny=32, nz=32, xwidth=64, ywidth=32, zwidth=32, periods_x=0, CFL=0.5, visc=0.032,
          ambient_fz=6.25e-6)


def _rest_state(nx, ny, nz):
    from seeded import W
    return np.ascontiguousarray(np.broadcast_to(W, (nz, ny, nx, 19)))


@pytest.mark.slow
def test_laminar_channel_matches_reference_over_1e4_steps():
    """FP64 engine vs the reference's kernels: <= 1e-12 relative in f-tilde after
    1, 100, 1000 and 10^4 steps (the FP64 parity bound)."""
    _need_ref()
    f0 = _rest_state(64, 32, 32)
    ref = pyoracle.to_ghosted(f0)
    eng = pydugks.Engine(pydugks.make_config(**C1))
    eng.set_state(f0)
    done = 0
    for upto in (1, 100, 1000, 10000):
        pyoracle.ref_run(ref, **_ref_args(C1), istep0=done + 1, nsteps=upto - done, prec=0)
        eng.run(done + 1, upto - done)
        done = upto
        err = rel_err(eng.get_state(), pyoracle.interior(ref))
        print(f"laminar channel, {upto} steps: engine-vs-reference {err:.3e}")
        assert err <= 1e-12


@pytest.mark.parametrize("recon", [0, 1])
def test_stretched_code_path_on_evenly_spaced_faces_matches_reference(recon, tmp_path):
    """The engine's stretched-mesh path (mesh=file: per-column weight tables, ghost
    extrapolation weights from the centres, dt from the first cell, and with
    recon=gradient the stretched gradient rule) on a mesh file with evenly spaced
    faces, against the reference's own uniform-mesh kernels."""
    _need_ref()
    kw = dict(REF_CASES["walls"])
    f0 = seeded_state(kw["nx"], kw["ny"], kw["nz"], seed=6)
    ref = pyoracle.to_ghosted(f0)
    pyoracle.ref_run(ref, **_ref_args(kw), istep0=1, nsteps=50, prec=0, recon=recon)
    with open(tmp_path / "mesh.txt", "w") as fh:
        fh.write("\n".join(repr(float(v)) for v in np.arange(kw["nx"] + 1.0)) + "\n")
    extra = {"recon": "gradient"} if recon else {}
    eng = pydugks.Engine(pydugks.make_config(mesh="file", mesh_file="mesh.txt", **extra, **kw), workdir=str(tmp_path))
    assert eng.info.mesh == 2
    eng.set_state(f0)
    eng.run(1, 50)
    err = rel_err(eng.get_state(), pyoracle.interior(ref))
    print(f"stretched path on evenly spaced faces, recon={recon}, 50 steps vs the reference: {err:.2e}")
    assert err <= 1e-12
