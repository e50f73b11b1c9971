"""Record the reference algorithm's own chain at the large NVT fluid state
(N = 256,000 from the 40^3 FCC lattice, rho = 0.85, dr_max 0.1635) for the
statistical gate in tests/test_gpu_statistics_large.py.

Run on a CPU machine (it takes about half an hour on eight cores):

    python tests/golden/make_c2_stats.py

Eight independent chains of the CPU oracle (the reference's random-particle
moves with MT19937 draws, oracle/hsmc_oracle.c, pinned bit for bit to the
reference build by tests/test_oracle.py), each: 1500 sweeps from the
lattice, then 20 samples 100 sweeps apart of
  - the virial contact histogram, 5 bins of 0.01 on [1, 1.05)
    (pressv_compute_hist, src/compute_press.c:123-165);
  - the global q6 with bond cutoff 1.5 (global_ql_compute,
    src/compute_order_parameter.c:82-94; computed on a copy of the
    configuration with cells of edge 1.5 so the reference's clip of the
    cutoff to the cell edge leaves 1.5);
  - 2 x 10^5 Widom insertions (widom_insertion,
    src/compute_widom_chem_pot.c:44-71);
and, every fifth sample, g(r) pair counts on [1, 5) in bins of 0.01 (ordered
pairs, the reference's 2 per pair; counted here with a periodic k-d tree,
since the reference's all-pairs loop, src/compute_rdf.c:110-128, takes
3.3e10 pair evaluations per sample at this size).

Each chain is one block of the blocking analysis: the fixture keeps per-chain
sums, so the gate compares chain-to-chain scatter with the GPU's blocks.
"""
from __future__ import annotations

import multiprocessing as mp
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

RHO, CELLS, DR = 0.85, 40, 0.1635
EQUIL, SAMPLES, EVERY, RDF_EVERY = 1500, 20, 100, 5
NB_PV, NB_RDF, BIN = 5, 400, 0.01
N_WIDOM = 200_000
CHAINS = 8


def chain(seed: int):
    from scipy.spatial import cKDTree

    from oracle.oracle import OracleSim

    o = OracleSim(rho=RHO, n_cells=CELLS, seed=seed, dr_max=DR, neigh_dr=1.05, neigh_max_part=10)
    q = OracleSim(rho=RHO, n_cells=CELLS, seed=seed, dr_max=DR, neigh_dr=1.5, neigh_max_part=40)
    L = o.box()["lx"]
    o.sweeps_nvt(EQUIL)
    o.reset_counters()
    pv = np.zeros(NB_PV)
    rdf = np.zeros(NB_RDF)
    q6 = []
    ok = 0
    n_rdf = 0
    edges = 1.0 + BIN * np.arange(NB_RDF + 1)
    for k in range(SAMPLES):
        o.sweeps_nvt(EVERY)
        pv += o.pressv_counts(BIN)[0][:NB_PV]
        conf = o.get_config()
        q.set_config(conf)
        mean, _, rc = q.ql(6, 1.5)
        assert rc == 1.5
        q6.append(mean)
        ok += o.widom_rng(N_WIDOM)
        if k % RDF_EVERY == 0:
            x = np.mod(conf[:, 1:], L)
            t = cKDTree(x, boxsize=L)
            cum = t.count_neighbors(t, edges).astype(np.float64)
            rdf += np.diff(cum)
            n_rdf += 1
    c = o.counters()
    return {"seed": seed, "pv": pv, "rdf": rdf, "n_rdf": n_rdf, "q6": float(np.mean(q6)),
            "widom_ok": ok, "widom_n": N_WIDOM * SAMPLES, "acc": float(c[1]) / float(c[0])}


def main():
    seeds = [101 + k for k in range(CHAINS)]
    with mp.get_context("spawn").Pool(CHAINS) as pool:
        res = pool.map(chain, seeds)
    out = os.path.join(HERE, "c2_oracle_stats.npz")
    np.savez_compressed(
        out, rho=RHO, cells=CELLS, dr_max=DR, equil=EQUIL, samples=SAMPLES, every=EVERY, rdf_every=RDF_EVERY,
        bin=BIN, n_widom=N_WIDOM, seeds=np.array(seeds),
        pv=np.array([r["pv"] for r in res]), rdf=np.array([r["rdf"] for r in res]),
        n_rdf=np.array([r["n_rdf"] for r in res]), q6=np.array([r["q6"] for r in res]),
        widom_ok=np.array([r["widom_ok"] for r in res]), widom_n=np.array([r["widom_n"] for r in res]),
        acc=np.array([r["acc"] for r in res]))
    for r in res:
        print(r["seed"], r["acc"], r["q6"], r["widom_ok"], r["pv"] / SAMPLES)
    print("wrote", out)


if __name__ == "__main__":
    main()
