"""Parity of the GB300 engine (through the C ABI) with the oracle, the CPU
restatement of the reference step (src/dugks.cu:322-391 and, for the
stretched mesh, src/fortran/channel/src/dugks.cuf).

Tolerances (max |a-b| / max |b| over f-tilde):
  FP64 form: 1e-12 per step and over the run (the FP64 parity bound)
  FP32 form: 2e-5 (the reference's PREC4 build itself mixes double literals
             into float expressions, so FP32 parity is not bitwise)
"""
import numpy as np
import pytest

from _cases import CASES, make_pair, run_both
from seeded import rel_err

FP64_TOL = 1e-12
FP32_TOL = 2e-5

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("nsteps", [1, 40])
def test_fp64_matches_oracle(case, nsteps):
    eng, orc, f0 = make_pair(case, "fp64")
    got, want = run_both(eng, orc, f0, 1, nsteps)
    err = rel_err(got, want)
    print(f"{case} fp64 {nsteps} steps: rel err {err:.3e}")
    assert err <= FP64_TOL


@pytest.mark.parametrize("case", ["walls", "periodic", "stretched"])
def test_fp32_matches_oracle(case):
    eng, orc, f0 = make_pair(case, "fp32")
    got, want = run_both(eng, orc, f0, 1, 20)
    err = rel_err(got, want)
    print(f"{case} fp32 20 steps: rel err {err:.3e}")
    assert err <= FP32_TOL


@pytest.mark.parametrize("case", ["walls", "periodic", "aniso", "stretched"])
def test_gradient_reconstruction_matches_oracle(case):
    """recon=gradient: the central-difference variant of src/dugks.cu:421-649 (calc_fx); on the
    tanh-stretched mesh with the face-interpolated values and non-uniform central differences."""
    from _cases import CASES as C
    import pydugks
    import pyoracle
    from seeded import seeded_state
    kw = dict(C[case])
    kw["recon"] = "gradient"
    cfg = pydugks.make_config(**kw)
    eng = pydugks.Engine(cfg)
    orc = pyoracle.Oracle.from_config(cfg)
    f0 = seeded_state(eng.nx, eng.ny, eng.nz, seed=3)
    eng.set_state(f0)
    got, want = run_both(eng, orc, f0, 1, 20)
    err = rel_err(got, want)
    print(f"{case} gradient fp64 20 steps: rel err {err:.3e}")
    assert err <= FP64_TOL


@pytest.mark.parametrize("case", ["walls", "periodic", "stretched"])
def test_gradient_reconstruction_fp32_matches_oracle(case):
    """recon=gradient in the FP32 form (the TMA-staged flux kernel) against the FP32 oracle."""
    from _cases import CASES as C
    import numpy as np
    import pydugks
    import pyoracle
    from seeded import seeded_state
    kw = dict(C[case])
    kw["recon"] = "gradient"
    kw["precision"] = "fp32"
    cfg = pydugks.make_config(**kw)
    eng = pydugks.Engine(cfg)
    orc = pyoracle.Oracle.from_config(cfg, dtype=np.float32)
    f0 = seeded_state(eng.nx, eng.ny, eng.nz, seed=3)
    eng.set_state(f0)
    got, want = run_both(eng, orc, f0, 1, 20)
    err = rel_err(got, want)
    print(f"{case} gradient fp32 20 steps: rel err {err:.3e}")
    assert err <= FP32_TOL


@pytest.mark.parametrize("prec", ["fp16", "bf16"])
@pytest.mark.parametrize("case", ["walls", "stretched"])
def test_gradient_reconstruction_16bit_matches_oracle(case, prec):
    """recon=gradient in the 16-bit forms (face values formed from decoded values, carried as
    f - w like the interpolated ones) within 3 storage quanta of the FP64 oracle."""
    from _cases import CASES as C
    import pydugks
    import pyoracle
    from seeded import seeded_state
    kw = dict(C[case])
    kw["recon"] = "gradient"
    kw["precision"] = prec
    cfg = pydugks.make_config(**kw)
    eng = pydugks.Engine(cfg)
    orc = pyoracle.Oracle.from_config(cfg)
    eng.set_state(seeded_state(eng.nx, eng.ny, eng.nz, seed=3))
    f0 = eng.get_state()
    got, want = run_both(eng, orc, f0, 1, 10)
    err = rel_err(got, want)
    w = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)
    tol = 3.0 * {"fp16": 2.0 ** -11, "bf16": 2.0 ** -8}[prec] * max(1e-3, float(np.max(np.abs(f0 - w) / w)))
    print(f"{case} gradient {prec} 10 steps: rel err {err:.3e} (bound {tol:.3e})")
    assert err <= tol


@pytest.mark.parametrize("shape,periodic_x", [((33, 5, 4), 0), ((65, 3, 2), 0), ((20, 1, 3), 0), ((20, 4, 1), 1),
                                              ((9, 1, 1), 0)])
def test_edge_shapes_match_oracle(shape, periodic_x):
    """Shapes at the edges of the tilings: nx = 1 (mod 32) between walls, a single row
    or plane (both ghost rows or planes of f-bar-plus are images of it)."""
    import pydugks
    import pyoracle
    from seeded import seeded_state
    nx, ny, nz = shape
    cfg = pydugks.make_config(nx=nx, ny=ny, nz=nz, xwidth=nx, ywidth=ny, zwidth=nz, periods_x=periodic_x,
                              CFL=0.5, visc=0.02, ambient_fx=1e-5 if periodic_x else 0.0, ambient_fz=1e-5)
    eng = pydugks.Engine(cfg)
    orc = pyoracle.Oracle.from_config(cfg)
    f0 = seeded_state(nx, ny, nz, seed=9)
    eng.set_state(f0)
    got, want = run_both(eng, orc, f0, 1, 10)
    err = rel_err(got, want)
    print(f"{shape} periodic_x={periodic_x}: rel err {err:.3e}")
    assert err <= FP64_TOL


@pytest.mark.parametrize("prec", ["fp32", "fp16", "bf16"])
@pytest.mark.parametrize("shape,periodic_x", [((33, 5, 4), 0), ((65, 3, 2), 0), ((20, 1, 3), 0), ((20, 4, 1), 1),
                                              ((9, 1, 1), 0), ((40, 9, 3), 0)])
def test_edge_shapes_float_forms(shape, periodic_x, prec):
    """The same shapes in the FP32 form (stage (a) writes the ghost layer) and the 16-bit forms
    (between walls stage (a) writes the y / z images and the flux kernel forms the wall ghost
    columns in shared memory, in the first tile and in the tile holding column nx).  FP32 within
    2e-5 of the FP32 oracle; 16-bit within 3 storage quanta of the largest deviation from the
    rest equilibrium of the FP64 oracle (as tests/test_gpu_mixed.py)."""
    import pydugks
    import pyoracle
    from seeded import seeded_state
    nx, ny, nz = shape
    cfg = pydugks.make_config(nx=nx, ny=ny, nz=nz, xwidth=nx, ywidth=ny, zwidth=nz, periods_x=periodic_x,
                              CFL=0.5, visc=0.02, ambient_fx=1e-5 if periodic_x else 0.0, ambient_fz=1e-5,
                              precision=prec)
    eng = pydugks.Engine(cfg)
    orc = pyoracle.Oracle.from_config(cfg, dtype=np.float32 if prec == "fp32" else np.float64)
    f0 = seeded_state(nx, ny, nz, seed=9)
    eng.set_state(f0)
    f0 = eng.get_state()  # the stored start (16-bit: rounded)
    got, want = run_both(eng, orc, f0, 1, 10)
    err = rel_err(got, want)
    if prec == "fp32":
        tol = FP32_TOL
    else:
        w = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)
        tol = 3.0 * {"fp16": 2.0 ** -11, "bf16": 2.0 ** -8}[prec] * max(1e-3, float(np.max(np.abs(f0 - w) / w)))
    print(f"{shape} periodic_x={periodic_x} {prec}: rel err {err:.3e} (bound {tol:.3e})")
    assert err <= tol


def test_step_is_deterministic():
    eng, _, f0 = make_pair("walls", "fp64")
    eng.run(1, 5)
    a = eng.get_state()
    eng.set_state(f0)
    eng.run(1, 5)
    assert np.array_equal(a, eng.get_state())


def test_stats_match_oracle():
    eng, orc, f0 = make_pair("walls", "fp64")
    got, _ = run_both(eng, orc, f0, 1, 10)
    g = np.zeros(orc.shape)
    g[1:-1, 1:-1, 1:-1] = got
    diag_o, prof_o = orc.stats(g)
    diag_e, prof_e = eng.stats_values()
    assert rel_err(diag_e, diag_o) <= 1e-13
    # plane averages and second moments; covariances cancel to ~1e-17 absolute
    assert np.max(np.abs(prof_e - prof_o)) <= 1e-13 * max(1.0, np.max(np.abs(prof_o)))


def test_macro_matches_oracle():
    eng, orc, f0 = make_pair("periodic", "fp64")
    got, _ = run_both(eng, orc, f0, 1, 3)
    g = np.zeros(orc.shape)
    g[1:-1, 1:-1, 1:-1] = got
    want = orc.macro(g)
    have = eng.copy_vel()
    for a, b in zip(have, want):
        assert rel_err(a[1:-1, 1:-1, 1:-1], b[1:-1, 1:-1, 1:-1]) <= 1e-14


def test_mass_conserved_periodic_and_walls():
    for case in ("periodic", "walls"):
        eng, _, _ = make_pair(case, "fp64")
        m0 = eng.moments()[0]
        eng.run(1, 50)
        m1 = eng.moments()[0]
        assert abs(m1 - m0) / m0 < 1e-12, case


def test_volume_weighted_mass_conserved_stretched():
    # on the stretched mesh the finite-volume update conserves sum(rho_i * dxx_i)
    eng, _, _ = make_pair("stretched", "fp64")
    _, dxx = eng.mesh()
    w = dxx[1:-1]
    m0 = (eng.get_state().sum(axis=-1) * w).sum()
    eng.run(1, 50)
    m1 = (eng.get_state().sum(axis=-1) * w).sum()
    assert abs(m1 - m0) / m0 < 1e-12


@pytest.mark.parametrize("prec", ["fp64", "fp32", "fp16"])
def test_graph_replayed_run_equals_single_steps(prec):
    """dg_run replays captured step graphs (8 steps per launch) when the step's parameters do not
    change; the result must equal the same steps launched one by one, and a force field set between
    runs must reach the replayed steps."""
    import numpy as np
    from _cases import CASES as C
    import pydugks
    from seeded import seeded_state
    kw = dict(C["walls"])
    kw["precision"] = prec
    f0 = seeded_state(kw["nx"], kw["ny"], kw["nz"], seed=14)
    phi = np.full((kw["nz"], kw["ny"], kw["nx"]), 3e-6)
    a = pydugks.Engine(pydugks.make_config(**kw))
    b = pydugks.Engine(pydugks.make_config(**kw))
    a.set_state(f0)
    b.set_state(f0)
    a.run(1, 37)
    for s in range(1, 38):
        b.step(s)
    assert np.array_equal(a.get_state(), b.get_state())
    a.set_force_field(2, phi)
    b.set_force_field(2, phi)
    a.run(38, 21)
    for s in range(38, 59):
        b.step(s)
    assert np.array_equal(a.get_state(), b.get_state())


def test_adjoint_refuses_the_gradient_reconstruction():
    """The hand-written adjoint transposes the trilinear reconstruction only."""
    import ctypes
    import pydugks
    from _cases import CASES as C
    kw = dict(C["walls"])
    kw["recon"] = "gradient"
    import torch
    eng = pydugks.Engine(pydugks.make_config(**kw))
    lam = torch.zeros(2, eng.soa_len, dtype=torch.float64, device="cuda")
    rc = pydugks.lib().dg_adjoint_step(eng._h, 1, ctypes.c_void_p(eng.device_ptr(pydugks.DG_BUF_F)),
                                       ctypes.c_void_p(lam[0].data_ptr()), ctypes.c_void_p(lam[1].data_ptr()))
    assert rc == pydugks.DG_ERR_UNSUPPORTED
