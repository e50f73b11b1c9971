"""Generate the golden fixtures in this directory from the HSMC reference's own
code (oracle/_ref/libhsmc_ref.so, compiled from the reference sources by
oracle/Makefile).  Run where the reference sources are available:

    python tests/golden/make_golden.py

The fixtures pin the CPU restatement (oracle/hsmc_oracle.c) on machines that
do not have the reference: trajectories, move counters and every observable's
fill loop on small seeded systems.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.oracle import RefSim, build_oracle  # noqa: E402

# (name, rho, n_cells, lattice type, neigh_dr, seed, dr_max, pressure, dv_max)
CASES = [
    ("nvt_rho050_n5", 0.50, 5, 2, 1.05, 1, 0.10, 0.0, 0.001),
    ("nvt_rho085_n5", 0.85, 5, 2, 1.05, 7, 0.12, 0.0, 0.001),
    ("nvt_rho030_sc6", 0.30, 6, 1, 1.10, 0, 0.30, 0.0, 0.001),
    ("npt_p11_n4", 0.90, 4, 2, 1.20, 11, 0.10, 11.0, 0.002),
]


def main() -> None:
    build_oracle(with_reference=True)
    rng = np.random.default_rng(20261203)
    out = {}
    for (name, rho, n, lt, nd, seed, dr, p, dv) in CASES:
        r = RefSim(rho=rho, n_cells=n, lattice_type=lt, neigh_dr=nd, seed=seed, dr_max=dr, press=p, dv_max=dv)
        out[f"{name}/lattice"] = r.get_config()
        if p > 0:
            r.sweeps_npt(12)
        else:
            r.sweeps_nvt(25)
        out[f"{name}/config"] = r.get_config()
        out[f"{name}/counters"] = r.counters()
        out[f"{name}/box"] = np.array(list(r.box().values()))
        hist, rmax = r.rdf_counts(0.01, 5.0)
        out[f"{name}/rdf"] = hist
        out[f"{name}/rdf_rmax"] = np.array([rmax])
        pv, _ = r.pressv_counts(0.01)
        out[f"{name}/pressv"] = pv
        out[f"{name}/presst"] = r.presst_counts(0.0001, 0.002)
        raw = rng.integers(0, 2**32 - 1, size=3 * 2000, dtype=np.uint32)
        out[f"{name}/widom_raw"] = raw
        out[f"{name}/widom_ok"] = np.array([r.widom(raw)])
        mean, per, rc = r.ql(6, 1.5)
        out[f"{name}/ql_mean"] = np.array([mean])
        out[f"{name}/ql_per"] = per
        out[f"{name}/ql_rc"] = np.array([rc])
        ids = rng.integers(0, r.n, size=300).astype(np.int32)
        mraw = rng.integers(0, 2**32 - 1, size=3 * 300, dtype=np.uint32)
        out[f"{name}/replay_ids"] = ids
        out[f"{name}/replay_raw"] = mraw
        out[f"{name}/replay_acc"] = r.replay_moves(ids, mraw)
        out[f"{name}/replay_config"] = r.get_config()
        oraw = rng.integers(0, 2**32, size=3 * 300, dtype=np.uint64).astype(np.uint32)
        out[f"{name}/offset_raw"] = oraw
        out[f"{name}/offset_acc"] = r.replay_moves_offsets(ids, oraw)
        out[f"{name}/offset_config"] = r.get_config()
    out["mt/seed4357_first16"] = RefSim.rng_raw(4357, 16)
    out["mt/seed0_first16"] = RefSim.rng_raw(0, 16)
    out["mt/seed5489_10000"] = RefSim.rng_raw(5489, 10000)[-16:]
    out["mt/uniform_int_seed3_range1000"] = RefSim.rng_uniform_int(3, 1000, 64)
    np.savez_compressed(os.path.join(HERE, "ref_vectors.npz"), **out)
    print("wrote", os.path.join(HERE, "ref_vectors.npz"), len(out), "arrays")


if __name__ == "__main__":
    main()
