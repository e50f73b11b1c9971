"""NpT on the GPU: volume moves keep the configuration overlap-free and inside
the box, the box follows the reference's lattice rebuild, and the density
agrees with the reference algorithm's own NpT chain (the CPU oracle)."""
import math
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def blocked_mean(x, blocks=10):
    x = np.asarray(x, dtype=float)
    m = len(x) // blocks
    b = x[: m * blocks].reshape(blocks, m).mean(axis=1)
    return b.mean(), b.std(ddof=1) / math.sqrt(blocks)


def test_npt_invariants(gpu_lib):
    rho0, n, P = 0.5, 5, 2.28
    g = gpu_lib.HardSphereSystem(rho=rho0, cells=n, dr_max=0.2, dv_max=0.02, pressure=P, seed=5)
    c = g.sweep_npt(200)
    assert c[0] == 200 * g.n
    assert c[3] > 150 and 0 < c[4] < c[3]
    box = g.get_box()
    lx, ly, lz, vol, rho = box
    cell = math.pow(4.0 / rho, 1.0 / 3.0)
    assert lx == n * cell and ly == lx and lz == lx
    assert vol == n * n * n * (4.0 / rho)
    assert rho == g.n / vol or abs(rho - g.n / vol) < 1e-12 * rho
    conf = g.download()
    assert np.all(conf[:, 1:] >= 0.0) and np.all(conf[:, 1:] <= lx)
    ids = np.arange(g.n, dtype=np.int32)
    assert g.overlap_replay(ids, conf[:, 1:]).sum() == 0
    # observables run on the rebuilt layout after volume moves
    xi = [(k + 1) * 0.0001 for k in range(20)]
    sf = np.array([math.pow(1 - x, 1.0 / 3.0) for x in xi])
    assert g.compute_presst(sf).shape == (20,)


def cs_packing_fraction(beta_p):
    """Carnahan-Starling's packing fraction at pressure beta P sigma^3
    (src/analytic.c:112), by bisection of beta P = (6 eta / pi) Z_CS(eta)."""
    lo, hi = 1e-6, 0.7
    for _ in range(200):
        eta = 0.5 * (lo + hi)
        z = (1 + eta + eta**2 - eta**3) / (1 - eta) ** 3
        if 6 * eta / math.pi * z < beta_p:
            lo = eta
        else:
            hi = eta
    return 0.5 * (lo + hi)


def test_npt_density_matches_oracle_chain_and_carnahan_starling(gpu_lib):
    """N = 500 at beta P = 2.28 (Carnahan-Starling's pressure near eta =
    0.30), ln V steps up to 0.01: eight GPU chains against eight chains of
    the reference algorithm (tests/golden/make_npt_stats.py), each chain's
    mean density one sample (the volume of a 500-sphere box decorrelates over
    about 10^2 sweeps, far below a chain's 40,000).  The mean density must
    agree with the reference chains' within 3 combined standard errors; the
    packing fraction's distance from Carnahan-Starling's at this pressure is
    printed for both."""
    ref = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "npt_oracle_stats.npz"))
    P, rho0, n = float(ref["pressure"]), float(ref["rho0"]), int(ref["cells"])
    dr, dv = float(ref["dr_max"]), float(ref["dv_max"])
    equil, samples, every = int(ref["equil"]), int(ref["samples"]), int(ref["every"])
    means, vacc = [], []
    for k in range(8):
        g = gpu_lib.HardSphereSystem(rho=rho0, cells=n, dr_max=dr, dv_max=dv, pressure=P, seed=300 + k)
        g.sweep_npt(equil)
        g.reset_moves_counters()
        d = np.empty(samples)
        for j in range(samples):
            g.sweep_npt(every)
            d[j] = g.get_box()[4]
        c = g.get_moves_counters()
        means.append(d.mean())
        vacc.append(c[4] / max(c[3], 1))
        g.close()
    mg, eg = np.mean(means), np.std(means, ddof=1) / math.sqrt(len(means))
    mr, er = float(np.mean(ref["rho_mean"])), float(np.std(ref["rho_mean"], ddof=1) / math.sqrt(len(ref["rho_mean"])))
    s = math.hypot(eg, er)
    eta_cs = cs_packing_fraction(P)
    k6 = math.pi / 6
    print(f"\nNpT rho at beta P {P}, N={4 * n**3}: gpu {mg:.5f} +- {eg:.5f}, reference chain {mr:.5f} +- {er:.5f} "
          f"({(mg - mr) / s:+.2f} sigma); volume acceptance gpu {np.mean(vacc):.3f}, "
          f"reference {float(np.mean(ref['vol_acc'])):.3f}")
    print(f"eta: gpu {mg * k6:.5f} +- {eg * k6:.5f} ({(mg * k6 - eta_cs) / (eg * k6):+.2f} sigma from "
          f"Carnahan-Starling {eta_cs:.5f}), reference {mr * k6:.5f} +- {er * k6:.5f} "
          f"({(mr * k6 - eta_cs) / (er * k6):+.2f} sigma)")
    assert abs(mg - mr) < 3.0 * s, (mg, eg, mr, er)
