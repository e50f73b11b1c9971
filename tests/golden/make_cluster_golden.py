"""Generate tests/golden/cluster_vectors.npz from the HSMC reference's own
cluster-move code (cluster_move, cluster_move_part, pocket_add, pocket_del of
src/cluster_nvt.c, compiled unmodified into oracle/_ref/libhsmc_ref.so by
oracle/Makefile).  Run where the reference sources are available:

    python tests/golden/make_cluster_golden.py

Each case starts from the reference's lattice, runs local sweeps, then
  - cluster moves with the reference's own draws (Mersenne twister): the
    cluster sizes and the final configuration;
  - cluster moves from given pivots, axes and seed particles (the pocket
    order still from the generator): sizes and configuration.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.oracle import RefSim, build_oracle  # noqa: E402

# (name, rho, n_cells, lattice type, neigh_dr, seed, dr_max, local sweeps, cluster moves)
CASES = [
    ("rho040_n3", 0.40, 3, 2, 1.05, 5, 0.30, 20, 40),
    ("rho030_sc6", 0.30, 6, 1, 1.10, 9, 0.40, 10, 40),
    ("rho070_n4", 0.70, 4, 2, 1.05, 3, 0.20, 20, 8),
]


def main() -> None:
    build_oracle(with_reference=True)
    rng = np.random.default_rng(20261204)
    out = {}
    for (name, rho, n, lt, nd, seed, dr, sweeps, moves) in CASES:
        r = RefSim(rho=rho, n_cells=n, lattice_type=lt, neigh_dr=nd, seed=seed, dr_max=dr)
        r.sweeps_nvt(sweeps)
        out[f"{name}/start"] = r.get_config()
        out[f"{name}/sizes"] = r.cluster_moves(moves)
        out[f"{name}/config"] = r.get_config()
        L = np.array([r.box()["lx"], r.box()["ly"], r.box()["lz"]])
        piv = rng.uniform(0.0, 1.0, size=(6, 3)) * L
        axes = rng.integers(0, 3, size=6).astype(np.int32)
        seeds = rng.integers(0, r.n, size=6).astype(np.int32)
        out[f"{name}/at_pivot"] = piv
        out[f"{name}/at_axis"] = axes
        out[f"{name}/at_seed"] = seeds
        out[f"{name}/at_sizes"] = np.array(
            [r.cluster_move_at(piv[k], axes[k], seeds[k]) for k in range(6)], dtype=np.int32)
        out[f"{name}/at_config"] = r.get_config()
    np.savez_compressed(os.path.join(HERE, "cluster_vectors.npz"), **out)
    print("wrote", os.path.join(HERE, "cluster_vectors.npz"), len(out), "arrays")


if __name__ == "__main__":
    main()
