"""Compatibility of the statistics files with the reference's post-processing.

tests/golden/laminar_profiles-2.dat is the profiles-2.dat this engine's host
driver writes for tests/golden/laminar_profiles_config.txt (checked byte for
byte on the GPU by tests/test_gpu_io.py); tests/golden/laminar_velmean.dat is
what the reference's own examples/laminar/ProcessProfiles.py wrote when run
unchanged on it (tests/golden/make_velmean_fixture.py).  Here, on the CPU: the
script read every block of the file (its mean profile is the symmetrised time
mean of the file's streamwise column) and the result is the laminar channel's
start-up profile (positive, symmetric, largest at the centre)."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
NX = 64


def _blocks():
    lines = open(os.path.join(GOLDEN, "laminar_profiles-2.dat")).read().splitlines()
    blocks = []
    while lines:
        head, rows, lines = lines[0], lines[1:NX + 1], lines[NX + 1:]
        blocks.append((int(head), np.array([[float(v) for v in r.split()] for r in rows])))
    return blocks


def test_profiles_file_has_the_reference_layout():
    blocks = _blocks()
    assert [b[0] for b in blocks] == [1, 500, 1000, 1500, 2000]
    for step, rows in blocks:
        assert rows.shape == (NX, 9)


def test_reference_script_consumed_every_block():
    vel = np.loadtxt(os.path.join(GOLDEN, "laminar_velmean.dat"))
    assert vel.shape == (NX, 6)
    assert np.array_equal(vel[:, 0], np.arange(1, NX + 1))
    uz = np.mean([rows[:, 2] for _, rows in _blocks()], axis=0)
    want = 0.5 * (uz + uz[::-1])
    assert np.max(np.abs(vel[:, 1] - want)) <= 1e-12 * np.max(np.abs(want))


def test_mean_profile_is_the_laminar_start_up_shape():
    vel = np.loadtxt(os.path.join(GOLDEN, "laminar_velmean.dat"))[:, 1]
    assert np.all(vel > 0)
    assert np.allclose(vel, vel[::-1], rtol=1e-12, atol=0)
    assert np.argmax(vel) in (NX // 2 - 1, NX // 2)
    assert np.all(np.diff(vel[: NX // 2]) >= 0)
