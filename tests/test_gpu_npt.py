"""NpT on the GPU: volume moves keep the configuration overlap-free and inside
the box, the box follows the reference's lattice rebuild, and the density
agrees with the reference algorithm's own NpT chain (the CPU oracle)."""
import math

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


def test_npt_density_matches_oracle_chain_and_carnahan_starling(oracle_mod, gpu_lib):
    """N = 500 at beta P = 2.28 (Carnahan-Starling's pressure near eta = 0.30),
    volume step 0.02 in ln V (about 40 % of volume moves accepted, so the
    volume decorrelates within tens of sweeps): the mean density agrees with
    the reference algorithm's own NpT chain (the oracle) and the mean packing
    fraction with Carnahan-Starling, each within 3 blocking standard errors."""
    P, rho0, n, dv = 2.28, 0.57, 5, 0.02
    g = gpu_lib.HardSphereSystem(rho=rho0, cells=n, dr_max=0.25, dv_max=dv, pressure=P, seed=17)
    g.sweep_npt(2000)
    dens = []
    for _ in range(2000):
        g.sweep_npt(5)
        dens.append(g.get_box()[4])
    c = g.get_moves_counters()
    mg, eg = blocked_mean(dens, blocks=20)
    o = oracle_mod.OracleSim(rho=rho0, n_cells=n, seed=3, dr_max=0.25, press=P, dv_max=dv, neigh_dr=1.3)
    o.sweeps_npt(2000)
    od = []
    for _ in range(2000):
        o.sweeps_npt(5)
        od.append(o.box()["rho"])
    mo, eo = blocked_mean(od, blocks=20)
    eta_cs = cs_packing_fraction(P)
    eta, e_eta = mg * math.pi / 6, eg * math.pi / 6
    print(f"\nNpT rho at beta P {P}, N=500: gpu {mg:.5f} +- {eg:.5f}, reference chain {mo:.5f} +- {eo:.5f} "
          f"({(mg - mo) / math.hypot(eg, eo):+.2f} sigma); volume acceptance {c[4] / max(c[3], 1):.3f}")
    print(f"NpT eta: gpu {eta:.5f} +- {e_eta:.5f}, Carnahan-Starling {eta_cs:.5f} "
          f"({(eta - eta_cs) / e_eta:+.2f} sigma)")
    assert abs(mg - mo) < 3.0 * math.hypot(eg, eo), (mg, eg, mo, eo)
    assert abs(eta - eta_cs) < 3.0 * e_eta, (eta, e_eta, eta_cs)
