"""Large grids: the tile, chunk and index arithmetic of the step kernels at
production sizes (ragged tiles in every direction, more than one CTA wave).

The FP32, FP16 and FP64 forms start from the same seeded state of a
258 x 197 x 131 channel (6.7 M cells, no size a multiple of a tile), must
conserve mass and agree after 3 steps within the FP32 / 16-bit storage
tolerances; the FP64 step must agree with the oracle on a 4-plane slab of the
same x-y size (the oracle is too slow for the full grid).
"""
import pytest

pytestmark = pytest.mark.gpu

import pydugks  # noqa: E402
from seeded import seeded_state, rel_err  # noqa: E402

NX, NY, NZ = 258, 197, 131


def _config(prec, nz=NZ):
    return pydugks.make_config(nx=NX, ny=NY, nz=nz, xwidth=NX, ywidth=NY, zwidth=nz, periods_x=0, CFL=0.5,
                               visc=0.02, ambient_fz=1e-5, precision=prec)


def _engine(prec, nz=NZ):
    return pydugks.Engine(_config(prec, nz))


def test_forms_agree_on_a_large_ragged_grid():
    f0 = seeded_state(NX, NY, NZ, seed=12, umax=0.05, eps=0.002)
    out = {}
    for prec in ("fp64", "fp32", "fp16"):
        eng = _engine(prec)
        eng.set_state(f0)
        m0 = eng.moments()[0]
        eng.run(1, 3)
        out[prec] = eng.get_state()
        m1 = eng.moments()[0]
        print(f"{prec}: mass drift {abs(m1 - m0) / m0:.2e}")
        assert abs(m1 - m0) / m0 < (1e-12 if prec == "fp64" else 1e-5)
        eng.close()
    e32 = rel_err(out["fp32"], out["fp64"])
    e16 = rel_err(out["fp16"], out["fp64"])
    print(f"fp32 vs fp64 {e32:.2e}, fp16 vs fp64 {e16:.2e}")
    assert e32 < 2e-5
    assert e16 < 2e-3


def test_fp64_large_slab_matches_oracle():
    import pyoracle
    nz = 4
    eng = _engine("fp64", nz=nz)
    orc = pyoracle.Oracle.from_config(_config("fp64", nz))
    f0 = seeded_state(NX, NY, nz, seed=13)
    eng.set_state(f0)
    eng.run(1, 2)
    got = eng.get_state()
    g = pyoracle.to_ghosted(f0)
    orc.run(g, 1, 2, 0)
    err = rel_err(got, pyoracle.interior(g))
    print(f"258x197x4 fp64 vs oracle, 2 steps: {err:.2e}")
    assert err <= 1e-12
