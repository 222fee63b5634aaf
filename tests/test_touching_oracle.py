"""The oracle's run_until_touching (integrate.cpp:221-415) against a replay of
the same trajectory step by step with the event logic restated in Python."""
import numpy as np
import pytest

from oracle.oracle import Oracle
from phafd_gb300 import workloads as W


def scene(d):
    cfg = dict(W.CONFIGS["32cube_64beads"])
    cfg.update(nchains=1, chain_len=24, dt=2e-3, field_noise="off", bead_temp=0.0)
    W.apply(d, cfg)
    d.setup()
    return d


def distances(nsteps):
    o = scene(Oracle())
    out = []
    for _ in range(nsteps):
        o.run(1)
        x = o.atoms_get()[0]
        out.append(float(np.sqrt(((x[-1] - x[0]) ** 2).sum())))
    return np.array(out)


def replay(d, touch, cont, delay):
    """integrate.cpp:350-395 on the per-step distances (steps 1, 2, ...)."""
    if not cont:
        delay = 0
    since, brk, ev = delay, 0, []
    for s, dist in enumerate(d, start=1):
        if dist < touch:
            if since >= delay:
                ev.append((0, s))
            since, brk = 0, 1
        else:
            if brk and since == delay:
                ev.append((1, s - delay))
            since += 1
        if not cont and brk:
            return s, ev
    return len(d), ev


def touch_between(d, q):
    """A touch point between two sampled distances, away from both."""
    v = np.sort(d)
    i = int(q * (len(v) - 1))
    return 0.5 * (v[i] + v[i + 1])


@pytest.mark.parametrize("cont,delay,q", [(False, 0, 0.3), (True, 0, 0.5), (True, 3, 0.5), (True, 10, 0.2)])
def test_oracle_events_match_replay(cont, delay, q):
    n = 60
    d = distances(n)
    touch = touch_between(d, q)
    done, ev = scene(Oracle()).run_until_touching(n, touch, cont, delay)
    assert (done, ev) == replay(d, touch, cont, delay)


def test_never_and_always_touching():
    o = scene(Oracle())
    assert o.run_until_touching(10, 0.0, False, 0) == (10, [])
    o = scene(Oracle())
    assert o.run_until_touching(10, 1e9, False, 0) == (1, [(0, 1)])
