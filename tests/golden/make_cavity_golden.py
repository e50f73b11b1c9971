"""Generate tests/golden/cavity_vectors.npz from the HSMC reference's own
cavity-sampling code (cavity_set_distance, cavity_sweep_nvt, cavity_part_move,
cavity_check_move and the analytic cavity function of src/analytic.c,
compiled unmodified into oracle/_ref/libhsmc_ref.so by oracle/Makefile).  Run
where the reference sources are available:

    python tests/golden/make_cavity_golden.py

Recorded per case: the umbrella potential psi(x) = cavity_interaction(x) on a
grid, the start after cavity_set_distance, the configuration and move
counters after cavity sweeps with the reference's generator, and cavity
trials with given uniforms (the offset form (2r + 1) / 2^33 the device uses)
with their acceptances and the final configuration.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.oracle import RefSim, build_oracle  # noqa: E402

# (name, rho, n_cells, seed, dr_max, p_cav, maxdr, mindr, sweeps)
CASES = [
    ("rho080_n3", 0.80, 3, 4, 0.10, 0.10, 1.2, 0.0, 30),
    ("rho050_n4", 0.50, 4, 6, 0.30, 0.30, 1.1, 0.6, 20),
]


def main() -> None:
    build_oracle(with_reference=True)
    rng = np.random.default_rng(20261205)
    out = {}
    x = np.linspace(0.0, 1.5, 151)
    out["psi_x"] = x
    for (name, rho, n, seed, dr, pcav, maxdr, mindr, sweeps) in CASES:
        r = RefSim(rho=rho, n_cells=n, seed=seed, dr_max=dr)
        r.cavity_setup(pcav, maxdr, mindr)
        out[f"{name}/psi"] = r.cavity_psi_ref(x)
        out[f"{name}/start"] = r.get_config()
        r.cavity_sweeps(sweeps)
        out[f"{name}/config"] = r.get_config()
        out[f"{name}/counters"] = r.counters()
        # trials with given uniforms; a wide range keeps every trial at the
        # Metropolis test, so each one draws its acceptance uniform
        r2 = RefSim(rho=rho, n_cells=n, seed=seed, dr_max=dr)
        r2.cavity_setup(pcav, 3.0, 0.0)
        r2.set_config(out[f"{name}/config"])
        k = 400
        which = rng.integers(0, 2, size=k).astype(np.int32)
        raw = rng.integers(0, 2**32, size=3 * k, dtype=np.uint64).astype(np.uint32)
        uacc = rng.integers(0, 2**32, size=k, dtype=np.uint64).astype(np.uint32)
        out[f"{name}/rp_which"] = which
        out[f"{name}/rp_raw"] = raw
        out[f"{name}/rp_uacc"] = uacc
        out[f"{name}/rp_acc"] = r2.cavity_replay(which, raw, uacc, np.ones(k, dtype=np.int32))
        out[f"{name}/rp_config"] = r2.get_config()
    np.savez_compressed(os.path.join(HERE, "cavity_vectors.npz"), **out)
    print("wrote", os.path.join(HERE, "cavity_vectors.npz"), len(out), "arrays")


if __name__ == "__main__":
    main()
