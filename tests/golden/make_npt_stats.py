"""Record the reference algorithm's own NpT chain for
tests/test_gpu_npt.py: N = 500 spheres (5^3 FCC start at rho = 0.573) at
beta P = 2.28, dr_max 0.25, ln V steps up to dv_max = 0.01 (sweep_npt and
vol_move, src/npt.c:177-196, src/moves.c:83-153), eight independent chains
of the CPU oracle (oracle/hsmc_oracle.c, pinned to the reference build by
tests/test_oracle.py), each 5000 sweeps of equilibration then 40,000 sweeps
with the density sampled every 10.  The volume of a 500-sphere box
decorrelates over about 10^2 sweeps at this step, so each chain's mean is
one independent sample and the chain-to-chain scatter is the error.

    python tests/golden/make_npt_stats.py     # a few minutes on 8 cores
"""
from __future__ import annotations

import multiprocessing as mp
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

P, RHO0, CELLS, DR, DV = 2.28, 0.573, 5, 0.25, 0.01
EQUIL, SAMPLES, EVERY = 5000, 4000, 10
CHAINS = 8


def chain(seed):
    from oracle.oracle import OracleSim

    o = OracleSim(rho=RHO0, n_cells=CELLS, seed=seed, dr_max=DR, press=P, dv_max=DV, neigh_dr=1.3)
    o.sweeps_npt(EQUIL)
    o.reset_counters()
    d = np.zeros(SAMPLES)
    for k in range(SAMPLES):
        o.sweeps_npt(EVERY)
        d[k] = o.box()["rho"]
    c = o.counters()
    return d.mean(), float(c[4]) / max(float(c[3]), 1.0)


def main():
    with mp.get_context("spawn").Pool(CHAINS) as pool:
        res = pool.map(chain, [700 + k for k in range(CHAINS)])
    out = os.path.join(HERE, "npt_oracle_stats.npz")
    np.savez_compressed(out, pressure=P, rho0=RHO0, cells=CELLS, dr_max=DR, dv_max=DV, equil=EQUIL,
                        samples=SAMPLES, every=EVERY, rho_mean=np.array([r[0] for r in res]),
                        vol_acc=np.array([r[1] for r in res]))
    print("wrote", out, [round(r[0], 5) for r in res], [round(r[1], 3) for r in res])


if __name__ == "__main__":
    main()
