"""The oracle's tangent-linear model (libtangent.so: the oracle's restatement
of the reference step run on dual numbers) on the CPU: its value part is the
FP64 oracle bit for bit, and its derivative part is the directional derivative
of the step -- checked against Richardson-extrapolated central differences of
the FP64 oracle (O(eps^4) truncation), <= 1e-7 relative, for every boundary
configuration and both reconstructions."""
import numpy as np
import pytest

import pydugks
import pyoracle
from _cases import CASES
from seeded import seeded_state, uniform_sym

NSTEPS = 3


def _setup(case, recon=0):
    kw = dict(CASES[case])
    if recon:
        kw["recon"] = "gradient"
    orc = pyoracle.Oracle.from_config(pydugks.make_config(**kw))
    f = pyoracle.to_ghosted(seeded_state(orc.cfg.nx, orc.cfg.ny, orc.cfg.nz, seed=31))
    d = pyoracle.to_ghosted(uniform_sym(8, f[1:-1, 1:-1, 1:-1].size, 3).reshape(f[1:-1, 1:-1, 1:-1].shape)
                            * 1e-2 * f[1:-1, 1:-1, 1:-1])
    return orc, f, d


@pytest.mark.parametrize("case,recon", [(c, 0) for c in sorted(CASES)] + [("walls", 1), ("periodic", 1),
                                                                          ("stretched", 1)])
def test_tangent_is_the_derivative_of_the_oracle_step(case, recon):
    orc, f, d = _setup(case, recon)
    fv, dv = f.copy(), d.copy()
    orc.tangent_run(fv, dv, 1, NSTEPS)
    ref = f.copy()
    orc.run(ref, 1, NSTEPS)
    assert np.array_equal(pyoracle.interior(fv), pyoracle.interior(ref))

    def cdiff(eps):
        a, b = f + eps * d, f - eps * d
        orc.run(a, 1, NSTEPS)
        orc.run(b, 1, NSTEPS)
        return pyoracle.interior((a - b) / (2 * eps))

    e = 1e-4
    fd = (4 * cdiff(e / 2) - cdiff(e)) / 3
    tan = pyoracle.interior(dv)
    rel = float(np.max(np.abs(tan - fd)) / np.max(np.abs(fd)))
    print(f"{case} recon={recon}: tangent vs extrapolated central difference {rel:.2e}")
    assert rel <= 1e-7


def test_tangent_is_linear_in_the_direction():
    orc, f, d = _setup("stretched")
    outs = []
    for scale in (1.0, -2.5):
        fv, dv = f.copy(), scale * d
        orc.tangent_run(fv, dv, 1, NSTEPS)
        outs.append(pyoracle.interior(dv) / scale)
    assert np.max(np.abs(outs[0] - outs[1])) <= 1e-13 * np.max(np.abs(outs[0]))
