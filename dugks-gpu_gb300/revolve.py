"""Binomial checkpointing ("revolve") schedules for reversing a run of time steps.

The adjoint of n steps needs the forward states 0..n-1 in reverse order.
With s stored states (the initial one included) and every step advanced at
most t times during the reversal, at most beta(s, t) = C(s + t, t) steps can
be reversed (Griewank, Optimization Methods and Software 1 (1992) 35-54;
Griewank and Walther, ACM TOMS 26 (2000) 19-45, "Algorithm 799: revolve").
The schedule below meets that bound: a segment [a, b) whose state a is held
is split at m = a + min(n - 1, beta(s, t - 1)) with t the smallest
repetition count that covers n = b - a steps; the state m is stored, the
right part [m, b) is reversed with one slot less, the slot is released, and
the left part [a, m) is reversed from state a again.

`actions(n, free)` lists the actions for `free` slots besides the one
holding state 0:
    ("advance", a, b)   run the steps a .. b-1 from the current state a
    ("store", m)        keep a copy of the current state (state m)
    ("restore", m)      make the stored state m current
    ("release", m)      drop the copy of state m
    ("adjoint", k)      the current state is state k: apply the adjoint of step k
The leading advance/store actions up to the last store before the first
adjoint form the forward sweep (`spine`): a caller may perform them while it
computes the forward result, and later resume the schedule from the last
state that sweep stored.
"""
from math import comb


def beta(s, t):
    """Steps reversible with s stored states and t advances per step."""
    return comb(s + t, t)


def repetitions(n, s):
    """Smallest t with beta(s, t) >= n (s >= 1)."""
    if s < 1:
        raise ValueError("at least the initial state must be stored")
    t = 0
    while beta(s, t) < n:
        t += 1
    return t


def actions(n, free):
    """Action list reversing steps 0..n-1 with `free` slots beyond state 0."""
    if n < 0 or free < 0:
        raise ValueError("n and free must be non-negative")
    out = []
    # explicit stack: entries are ("rev", a, b, free) tasks or finished actions
    stack = [("rev", 0, n, free)] if n > 0 else []
    while stack:
        task = stack.pop()
        if task[0] != "rev":
            out.append(task)
            continue
        _, a, b, fr = task
        n_seg = b - a
        if n_seg == 1:
            out.append(("adjoint", a))
            continue
        if fr == 0:
            # no slot left: advance from state a for every step, last step first
            for j in range(b - 1, a - 1, -1):
                if j != b - 1:
                    out.append(("restore", a))
                if j > a:
                    out.append(("advance", a, j))
                out.append(("adjoint", j))
            continue
        t = repetitions(n_seg, fr + 1)
        m = a + min(n_seg - 1, beta(fr + 1, t - 1))
        out.append(("advance", a, m))
        out.append(("store", m))
        # pushed in reverse order of execution
        stack.append(("rev", a, m, fr))
        stack.append(("restore", a))
        stack.append(("release", m))
        stack.append(("rev", m, b, fr - 1))
    return out


def spine(acts):
    """(end, state): acts[:end] is the forward sweep, which ends with a store of
    `state` (state 0 when it stores nothing); the reversal resumes at
    acts[end] from that state."""
    end, state = 0, 0
    for i, a in enumerate(acts):
        if a[0] == "store":
            end, state = i + 1, a[1]
        elif a[0] != "advance":
            break
    return end, state


def simulate(n, free):
    """Dry run: checks the schedule and returns (advanced steps, peak slots)."""
    acts = actions(n, free)
    cur = 0
    held = {0}
    peak = 0
    advanced = 0
    expect = n - 1
    for a in acts:
        kind = a[0]
        if kind == "advance":
            if a[1] != cur or a[2] <= a[1]:
                raise AssertionError(f"advance {a} from state {cur}")
            advanced += a[2] - a[1]
            cur = a[2]
        elif kind == "store":
            if a[1] != cur or a[1] in held:
                raise AssertionError(f"store {a} at state {cur}")
            held.add(a[1])
            peak = max(peak, len(held) - 1)
        elif kind == "restore":
            if a[1] not in held:
                raise AssertionError(f"restore of a state not held: {a}")
            cur = a[1]
        elif kind == "release":
            held.discard(a[1])
        elif kind == "adjoint":
            if a[1] != cur or a[1] != expect:
                raise AssertionError(f"adjoint {a} at state {cur}, expected step {expect}")
            expect -= 1
        else:
            raise AssertionError(f"unknown action {a}")
    if expect != -1:
        raise AssertionError(f"schedule reversed steps down to {expect + 1} only")
    return advanced, peak
