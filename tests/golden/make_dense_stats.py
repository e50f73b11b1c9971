"""Record the reference algorithm's own chain at the dense replica states
for tests/test_gpu_batch_stats.py: N = 2048 spheres (8^3 FCC start) at
rho = 0.75 and 0.85, dr_max 0.15, the virial contact histogram (5 bins of
0.01 on [1, 1.05), pressv_compute_hist, src/compute_press.c:123-165) every
20 sweeps after 2000 sweeps from the lattice, 8 independent chains per
density of the CPU oracle (random-particle moves with MT19937 draws,
oracle/hsmc_oracle.c, pinned to the reference build by tests/test_oracle.py).

    python tests/golden/make_dense_stats.py      # a few minutes on 8 cores

The gate compares the straight-line contact fit of these chains
(python/hsmc_pressure.py:11-41) with the batched GPU replicas' at the same
states, which shows whether a departure from Carnahan-Starling comes from
the chain or from the fit.
"""
from __future__ import annotations

import multiprocessing as mp
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

RHOS = (0.75, 0.85)
CELLS, DR = 8, 0.15
EQUIL, SAMPLES, EVERY = 2000, 500, 20
NB, BIN = 5, 0.01
CHAINS = 8


def chain(args):
    rho, seed = args
    from oracle.oracle import OracleSim

    o = OracleSim(rho=rho, n_cells=CELLS, seed=seed, dr_max=DR, neigh_dr=1.05, neigh_max_part=10)
    o.sweeps_nvt(EQUIL)
    pv = np.zeros(NB)
    for _ in range(SAMPLES):
        o.sweeps_nvt(EVERY)
        pv += o.pressv_counts(BIN)[0][:NB]
    return pv


def main():
    jobs = [(rho, 500 + 10 * k + j) for k, rho in enumerate(RHOS) for j in range(CHAINS)]
    with mp.get_context("spawn").Pool(8) as pool:
        res = pool.map(chain, jobs)
    pv = np.array(res).reshape(len(RHOS), CHAINS, NB)
    out = os.path.join(HERE, "dense_oracle_stats.npz")
    np.savez_compressed(out, rhos=np.array(RHOS), cells=CELLS, dr_max=DR, equil=EQUIL, samples=SAMPLES,
                        every=EVERY, bin=BIN, pv=pv)
    print("wrote", out, pv.sum(axis=1))


if __name__ == "__main__":
    main()
