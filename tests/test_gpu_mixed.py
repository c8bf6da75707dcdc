"""The 16-bit storage forms (FP16 / BF16 deviations from the rest equilibrium,
FP32 arithmetic) against the FP64 oracle.

Bounds: after 10 steps from a seeded state the max-norm error relative to the
oracle stays within 3 storage quanta of the largest deviation from the rest
equilibrium (quantum 2^-11 for FP16, 2^-8 for BF16; measured 0.1-0.8 quanta)
with either rounding of either form; the total mass drifts by less than a
tenth of a quantum over 200 steps; runs are deterministic (stochastic
rounding included, its seed is the step number).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from _cases import make_pair, run_both  # noqa: E402
from seeded import rel_err  # noqa: E402

QUANT = {"fp16": 2.0 ** -11, "bf16": 2.0 ** -8}


def _maxdev(f0):
    w = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)
    return float(np.max(np.abs(f0 - w) / w))


@pytest.mark.parametrize("prec,rounding", [("fp16", "stochastic"), ("fp16", "nearest"), ("bf16", "stochastic"),
                                           ("bf16", "nearest")])
@pytest.mark.parametrize("case", ["walls", "periodic", "stretched"])
def test_16bit_forms_stay_within_the_storage_quantum(case, prec, rounding):
    n = 10
    eng, orc, f0 = make_pair(case, precision=prec, rounding=rounding)
    # the state was just quantised by set_state: compare against the oracle run from the same stored values
    fq = eng.get_state()
    eng.set_state(fq)
    got, ref = run_both(eng, orc, fq, 1, n)
    err = rel_err(got, ref)
    bound = 3.0 * QUANT[prec] * max(1e-3, _maxdev(f0))
    print(f"{case} {prec} {rounding}: rel err {err:.3e} after {n} steps, bound {bound:.3e}")
    assert err <= bound


@pytest.mark.parametrize("prec", ["fp16", "bf16"])
def test_16bit_mass_drift(prec):
    eng, _, f0 = make_pair("periodic", precision=prec)
    m0 = eng.moments()[0]
    eng.run(1, 200)
    m1 = eng.moments()[0]
    drift = abs(m1 - m0) / abs(m0)
    print(f"{prec}: mass drift {drift:.3e} over 200 steps")
    assert drift < 0.1 * QUANT[prec] * max(1e-3, _maxdev(f0))


@pytest.mark.parametrize("prec", ["bf16", "fp16"])
def test_16bit_runs_are_deterministic_and_rounding_modes_differ(prec):
    outs = []
    for rounding in ("stochastic", "stochastic", "nearest"):
        eng, _, _ = make_pair("walls", precision=prec, rounding=rounding)
        eng.run(1, 15)
        outs.append(eng.get_state())
        eng.close()
    assert np.array_equal(outs[0], outs[1])
    assert not np.array_equal(outs[0], outs[2])
