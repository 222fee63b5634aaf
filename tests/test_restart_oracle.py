"""Restart continuity on the oracle: a run stopped at step 10 and restarted
from its phi, wrapped bead positions and image flags (what the grid and atom
dumps hold) with timestep 10 continues the uninterrupted trajectory.  The
field and bead noise are keyed by (seed, step), so the only difference is the
summation order of the rebuilt neighbor lists."""
import numpy as np

from oracle.oracle import Oracle
from phafd_gb300 import workloads as W

CFG = dict(W.CONFIGS["32cube_64beads"], dt=5e-4, field_noise="philox", bead_temp=1.0)


def make(chains, phi=None, images=None, step=0):
    o = Oracle()
    W.apply(o, CFG, chains=chains)
    if phi is not None:
        o.grid_set("phi", phi)
    if images is not None:
        o.atoms_set_images(images)
    o.set_timestep(step)
    o.setup()
    return o


def test_restart_continues_the_trajectory():
    chains = W.random_walk_chains(CFG["nchains"], CFG["chain_len"], CFG["origin"], CFG["L"], CFG["chain_seed"])
    a = make(chains)
    a.run(10)
    phi10 = a.grid_get("phi").copy()
    x10, _, _, im10 = a.atoms_get()
    a.run(10)
    b = make((x10.copy(),) + tuple(chains[1:]), phi10, im10.copy(), 10)
    b.run(10)
    pa, pb = a.grid_get("phi"), b.grid_get("phi")
    assert np.linalg.norm(pb - pa) < 1e-12 * np.linalg.norm(pa)
    uxa, uxb = a.atoms_get()[1], b.atoms_get()[1]
    assert np.abs(uxb - uxa).max() < 1e-12 * np.abs(uxa).max()
    # without the step offset the noise repeats steps 1-10 and the runs part
    c = make((x10.copy(),) + tuple(chains[1:]), phi10, im10.copy(), 0)
    c.run(10)
    assert np.linalg.norm(c.grid_get("phi") - pa) > 1e-3 * np.linalg.norm(pa)


def test_reference_noise_resumes_with_its_generator_state():
    """The reference's mt19937 field noise continues exactly when its state
    is saved with the restart (the reference itself re-seeds on a restart)."""
    cfg = dict(CFG, field_noise="reference")
    chains = W.random_walk_chains(cfg["nchains"], cfg["chain_len"], cfg["origin"], cfg["L"], cfg["chain_seed"])

    def make(phi=None, images=None, step=0, state=None, ch=chains):
        o = Oracle()
        W.apply(o, cfg, chains=ch)
        if phi is not None:
            o.grid_set("phi", phi)
        if images is not None:
            o.atoms_set_images(images)
        if state is not None:
            o.set_noise_state(state)
        o.set_timestep(step)
        o.setup()
        return o

    a = make()
    a.run(10)
    phi10, state = a.grid_get("phi").copy(), a.noise_state()
    x10, _, _, im10 = a.atoms_get()
    a.run(10)
    rest = (x10.copy(),) + tuple(chains[1:])
    b = make(phi10, im10.copy(), 10, state, rest)
    b.run(10)
    pa = a.grid_get("phi")
    assert np.linalg.norm(b.grid_get("phi") - pa) < 1e-12 * np.linalg.norm(pa)
    c = make(phi10, im10.copy(), 10, None, rest)  # re-seeded: the stream restarts
    c.run(10)
    assert np.linalg.norm(c.grid_get("phi") - pa) > 1e-3 * np.linalg.norm(pa)


def test_noise_state_round_trip_and_errors():
    o = Oracle()
    W.apply(o, dict(CFG, field_noise="reference"))
    s = o.noise_state()
    assert len(s) > 6000 and s.split()[0].isdigit()
    o.set_noise_state(s)
    assert o.noise_state() == s
    from oracle.oracle import OracleError
    import pytest
    with pytest.raises(OracleError, match="malformed"):
        o.set_noise_state("1 2 3")
