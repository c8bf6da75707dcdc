"""Binomial checkpointing schedules (host logic of the adjoint harness)."""
import pytest

import revolve


@pytest.mark.parametrize("n", [1, 2, 3, 7, 10, 33, 100, 257])
@pytest.mark.parametrize("free", [0, 1, 2, 5, 20])
def test_schedule_reverses_every_step_within_the_slots(n, free):
    if free == 0 and n > 60:
        pytest.skip("quadratic without slots")
    advanced, peak = revolve.simulate(n, free)
    assert peak <= free
    t = revolve.repetitions(n, free + 1)
    # each step is advanced at most t times (Griewank's bound)
    assert advanced <= t * n


def test_binomial_counts():
    assert revolve.beta(1, 3) == 4          # initial state only: t + 1 steps
    assert revolve.beta(5, 1) == 6          # every state stored
    assert revolve.beta(3, 2) == 10
    assert revolve.repetitions(4000, 101) == 2
    assert revolve.repetitions(1, 1) == 0


def test_spine_ends_at_the_state_the_reversal_resumes_from():
    for n, free in [(10, 1), (10, 3), (100, 5), (4000, 100)]:
        acts = revolve.actions(n, free)
        end, state = revolve.spine(acts)
        assert all(a[0] in ("advance", "store") for a in acts[:end])
        cur = 0
        for a in acts[:end]:
            if a[0] == "advance":
                cur = a[2]
        assert cur == state
        assert acts[end][0] in ("advance", "adjoint")
        if acts[end][0] == "advance":
            assert acts[end][1] == state
        else:
            assert acts[end][1] == state == n - 1


def test_channel_adjoint_budget():
    # 4000 steps with 100 stored states: about one recomputed step per step
    acts = revolve.actions(4000, 100)
    end, _ = revolve.spine(acts)
    spine_steps = sum(a[2] - a[1] for a in acts[:end] if a[0] == "advance")
    total, peak = revolve.simulate(4000, 100)
    assert peak == 100
    assert (total - spine_steps) / 4000 < 1.05


def test_checkpoint_pool_holds_every_schedule():
    """The harness's state pool (snaps + 1 slots) runs every schedule without
    running out, and a restored slot holds what was stored there."""
    torch = pytest.importorskip("torch")
    import types
    import dugks_autograd as da
    eng = types.SimpleNamespace(soa_len=3, info=types.SimpleNamespace(precision=next(iter(da._TORCH_DTYPE))))
    for n, free in [(10, 1), (33, 2), (100, 5), (257, 20)]:
        pool = da._StatePool(eng, free + 1, "cpu")
        pool.store(0).fill_(0)
        for a in revolve.actions(n, free):
            if a[0] == "store":
                pool.store(a[1]).fill_(a[1])
            elif a[0] == "restore":
                assert float(pool[a[1]][0]) == a[1]
            elif a[0] == "release":
                pool.release(a[1])
        assert len(pool.free) + len(pool.slot) == free + 1
