"""Writes tests/golden/oracle_cases.npz: regression fixtures produced by the
FP64 oracle (oracle/) on small seeded cases.  The reference ships no test
vectors and cannot be built here, so these fixtures pin the oracle to its
own earlier outputs (and give the GPU tests data that does not depend on the
oracle's code at test time); they are not outputs of the reference.

    python tests/golden/make_golden.py

Cases: one FFT (r2c of a 6 x 10 x 8 seeded real array, the reference's
[ky][kz][kx] layout) and one 10-step run of a 16^3 grid with a 12-bead chain
(Philox field and bead noise, FP64), stored with its inputs."""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as OR  # noqa: E402
from oracle.oracle import Oracle  # noqa: E402
from phafd_gb300 import workloads as W  # noqa: E402

STEP_CFG = dict(W.CONFIGS["32cube_64beads"], n=16, L=16.0, origin=-8.0, nchains=1, chain_len=12,
                field_noise="philox", bead_temp=1.0, dt=5e-4)
STEPS = 10


def step_case(driver, phi0, chains):
    W.apply(driver, STEP_CFG, chains=chains, phi=phi0)
    driver.setup()
    driver.run(STEPS)
    x, ux, f, im = driver.atoms_get()
    return driver.grid_get("phi"), x, ux, f, im


def main():
    rng = np.random.default_rng(2024)
    fft_in = rng.standard_normal((6, 10, 8))
    fft_out = OR.fft_r2c(fft_in)
    chains = W.random_walk_chains(STEP_CFG["nchains"], STEP_CFG["chain_len"], STEP_CFG["origin"],
                                  STEP_CFG["L"], STEP_CFG["chain_seed"])
    n = STEP_CFG["n"]
    phi0 = STEP_CFG["phi0"] + STEP_CFG["amp"] * (rng.random((n, n, n)) - 0.5)
    phi, x, ux, f, im = step_case(Oracle(), phi0, chains)
    np.savez_compressed(os.path.join(HERE, "oracle_cases.npz"), fft_in=fft_in, fft_out=fft_out, phi0=phi0,
                        x0=chains[0], tags=chains[1], mol=chains[2], types=chains[3], phi=phi, x=x, ux=ux, f=f,
                        images=im)


if __name__ == "__main__":
    main()
