"""Statistical parity on the reference's own CPU workload (N = 4000 from the
10x10x10 FCC lattice at rho = 0.5): the GPU chain and the reference algorithm's
chain (the CPU oracle, MT19937 draws) sample the same observables, and every
one must agree within 3 combined blocking standard errors; the pressure also
against Carnahan-Starling (src/analytic.c:112) within 3 standard errors.  Each
error is printed.

The contact value comes from a linear fit of g(r) on [1, 1.05) as the
reference's analysis does (python/hsmc_pressure.py:11-41): Z = 1 + 2 pi/3 rho g(1).
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RHO, CELLS, DR = 0.5, 10, 0.30
N = 4 * CELLS**3
EQ, PROD, EVERY = 400, 4000, 20


def blocks(x, nb=10):
    x = np.asarray(x, dtype=float)
    m = len(x) // nb
    b = x[: m * nb].reshape(nb, m).mean(axis=1)
    return b.mean(), b.std(ddof=1) / math.sqrt(nb)


def shell_norm(counts, dr, n, rho):
    r = (np.arange(len(counts)) + 0.5) * dr + 1.0
    r1, r2 = r - dr / 2, r + dr / 2
    vol = 4 * np.pi / 3 * (r2**3 - r1**3)
    return r, counts / (vol * rho * n)


def contact_z(g5, dr=0.01):
    r = (np.arange(len(g5)) + 0.5) * dr + 1.0
    b1, b0 = np.polyfit(r, g5, 1)
    return 1 + 2 * np.pi / 3 * RHO * (b0 + b1)


def sample(run_sweeps, pressv, widom, ql, rdf):
    z, mu, q6, g_peak = [], [], [], []
    run_sweeps(EQ)
    for k in range(PROD // EVERY):
        run_sweeps(EVERY)
        _, g5 = shell_norm(np.asarray(pressv(), dtype=float), 0.01, N, RHO)
        z.append(contact_z(g5))
        ok = widom(2000)
        if ok > 0:
            mu.append(-math.log(ok / 2000))
        q6.append(ql())
        if k % 5 == 0:
            _, g = shell_norm(np.asarray(rdf(), dtype=float), 0.02, N, RHO)
            g_peak.append(g[:5].mean())
    return {"Z": blocks(z), "mu": blocks(mu), "q6": blocks(q6), "g_contact": blocks(g_peak, nb=8)}


def test_observables_agree_with_reference_chain(oracle_mod, gpu_lib):
    g = gpu_lib.HardSphereSystem(rho=RHO, cells=CELLS, dr_max=DR, seed=2024)
    o = oracle_mod.OracleSim(rho=RHO, n_cells=CELLS, seed=2024, dr_max=DR, neigh_dr=1.05)
    rmax_pv = 0.01 * 5 + 1.0
    nb_rdf = int((3.0 - 1.0) / 0.02)
    rmax_rdf = 0.02 * nb_rdf + 1.0
    _, _, rc = o.ql(6, 1.5)  # the reference clips the cutoff to its cell size

    gpu = sample(g.sweep_nvt,
                 lambda: g.compute_pressv_counts(0.01, rmax_pv, 5),
                 g.widom_insertion,
                 lambda: g.global_ql(6, rc),
                 lambda: g.compute_rdf_counts(0.02, rmax_rdf, nb_rdf))
    ref = sample(o.sweeps_nvt,
                 lambda: o.pressv_counts(0.01)[0],
                 o.widom_rng,
                 lambda: o.ql(6, 1.5)[0],
                 lambda: o.rdf_counts(0.02, 3.0)[0])
    eta = np.pi * RHO / 6
    z_cs = (1 + eta + eta**2 - eta**3) / (1 - eta) ** 3
    report = []
    for key in gpu:
        (mg, eg), (mr, er) = gpu[key], ref[key]
        report.append(f"{key}: gpu {mg:.5f} +- {eg:.5f}  reference {mr:.5f} +- {er:.5f}")
        assert abs(mg - mr) <= 3.0 * math.hypot(eg, er) + 1e-12, "\n".join(report)
    mz, ez = gpu["Z"]
    report.append(f"Z vs Carnahan-Starling {z_cs:.5f}: {(mz - z_cs) / ez:+.2f} sigma ({(mz - z_cs) / z_cs:+.3%})")
    print("\n" + "\n".join(report))
    assert abs(mz - z_cs) <= 3.0 * ez, "\n".join(report)
