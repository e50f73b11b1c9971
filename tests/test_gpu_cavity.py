"""Cavity sampling on the GPU against the oracle (pinned to the reference's
cavity code by tests/test_oracle_cavity.py): the device's umbrella potential,
every traced trial of whole sweeps (the other particles' checkerboard trials
and the cavity trials, replayed in order on the oracle) with identical
decisions and configurations, the invariants of a long run, and the sampled
cavity distances against the potential that biases them."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_device_psi_matches_oracle(oracle_mod, gpu_lib):
    """FP64 exp, sin, cos and log of the device against glibc: relative
    agreement to 1e-13 (the decisions use psi only through
    exp(-(psi' - psi)) compared with a uniform)."""
    for rho in (0.5, 0.8):
        g = gpu_lib.HardSphereSystem(rho=rho, cells=3, dr_max=0.1, seed=1, cavity=(0.1, 1.2, 0.0))
        x = np.concatenate([np.linspace(0.0, 1.5, 301), [1.0, 1.0 - 2**-52, 1.0 + 2**-52]])
        got = g.cavity_psi(x)
        want = oracle_mod.OracleSim.cavity_psi(rho, x)
        assert np.all(np.abs(got - want) <= 1e-13 * np.maximum(1.0, np.abs(want))), np.max(np.abs(got - want))
        inner = x < 1.0  # the cubic is evaluated with the reference's operations only
        assert np.array_equal(got[inner], want[inner])


def _replay_sweeps(oracle_mod, g, o, sweeps):
    """Run traced sweeps on the device and replay each sweep on the oracle:
    its checkerboard trials, then its cavity trials."""
    g.cavity_trace(100000)
    rec, cnt = g.sweeps_traced(sweeps)
    cav = g.cavity_trace_read()
    nc, l32, iw, _ = g.grid_info()
    base = int(rec[:, 0].min()) // 8
    n_frozen = int(np.sum(rec[:, 7] == 4))
    std = rec[rec[:, 7] != 4]
    decisions = {"std": [], "cav": []}
    for s in range(sweeps):
        sel = std[(std[:, 0] // 8) == base + s]
        sel = sel[np.lexsort((sel[:, 2], sel[:, 1], sel[:, 0]))]
        shifts = sel[:, 8:11].copy().view(np.float32)
        dec = o.replay_checkerboard(sel[:, 3].astype(np.int32), sel[:, 4:7], sel[:, 1], shifts, nc, l32, iw)
        assert not np.any(dec == 3), "a traced particle was not in its cell"
        assert np.array_equal(dec, sel[:, 7].astype(np.int32))
        cs = cav[cav[:, 0] == base + s]
        cs = cs[np.argsort(cs[:, 1])]
        cd = o.cavity_replay(cs[:, 2].astype(np.int32), cs[:, 3:6].reshape(-1), cs[:, 6])
        assert np.array_equal(cd, cs[:, 7].astype(np.int32))
        decisions["std"].append(dec)
        decisions["cav"].append(cd)
    return decisions, n_frozen, cnt


@pytest.mark.parametrize("rho,n,seed,dr,pcav,maxdr,mindr", [
    (0.80, 4, 3, 0.10, 0.10, 1.2, 0.0),
    (0.50, 5, 8, 0.30, 0.30, 1.1, 0.6),
])
def test_traced_cavity_sweeps_replay_bit_exact(oracle_mod, gpu_lib, rho, n, seed, dr, pcav, maxdr, mindr):
    g = gpu_lib.HardSphereSystem(rho=rho, cells=n, dr_max=dr, seed=seed, cavity=(pcav, maxdr, mindr))
    g.sweep_nvt(10)
    o = oracle_mod.OracleSim(rho=rho, n_cells=n, seed=1, dr_max=dr, neigh_dr=1.05, neigh_max_part=12)
    o.cavity_setup(pcav, maxdr, mindr)
    o.set_config(g.download())
    o.reset_counters()
    dec, n_frozen, cnt = _replay_sweeps(oracle_mod, g, o, 4)
    assert np.array_equal(g.download(), o.get_config())
    cav = np.concatenate(dec["cav"])
    k = max(1, round(g.n * pcav))
    assert len(cav) == 4 * k
    assert set(cav.tolist()) & {0} and set(cav.tolist()) - {0}
    assert cnt[0] == 4 * g.n + 4 * k  # every checkerboard trial plus the cavity trials
    acc = sum(int(np.sum(d == 0)) for d in dec["std"]) + int(np.sum(cav == 0))
    assert cnt[1] == acc
    assert n_frozen > 0  # trials of the passes that picked a cavity left it in place


def test_cavity_run_invariants(oracle_mod, gpu_lib):
    """No move creates an overlap.  The start places cavity 1 half a diameter
    from cavity 0 (cavity_set_distance); at rho = 0.4 that overlaps no other
    lattice site (nearest neighbours 1.52 apart), so none may appear."""
    g = gpu_lib.HardSphereSystem(rho=0.4, cells=5, dr_max=0.3, seed=21, cavity=(0.05, 0.7, 0.3))
    for _ in range(10):
        g.sweep_nvt(20)
        d = g.cavity_distance()
        assert 0.3 <= d <= 0.7
    conf = g.download()
    for i in range(2, g.n, 3):  # the other particles overlap nothing, cavities included
        assert oracle_mod.OracleSim.brute_overlap(conf, g.box, i, *conf[i, 1:]) == 0
    for w in (0, 1):  # a cavity overlaps no other particle (the other cavity aside)
        other = np.delete(conf, [0, 1], axis=0)
        other[:, 0] = np.arange(other.shape[0])
        assert oracle_mod.OracleSim.brute_overlap(other, g.box, -1, *conf[w, 1:]) == 0


def test_cavity_distances_follow_the_umbrella(gpu_lib):
    """With psi = ln y_GH as the bias, the sampled distance density is
    r^2 y(r) exp(-psi(r)): flat in r^2-scaled bins where the parametrisation
    is accurate.  ln(h(r) / r^2) may vary by less than 0.6 over 0.35 <= r
    <= 1.15 at rho = 0.5 (Grundke-Henderson is good to a few per cent of
    ln y there)."""
    rho = 0.5
    g = gpu_lib.HardSphereSystem(rho=rho, cells=4, dr_max=0.3, seed=5, cavity=(0.2, 1.2, 0.0))
    g.sweep_nvt(300)
    d = []
    for _ in range(3000):
        g.sweep_nvt(1)
        d.append(g.cavity_distance())
    d = np.array(d)
    assert d.min() >= 0.0 and d.max() <= 1.2
    edges = np.linspace(0.35, 1.15, 9)
    h, _ = np.histogram(d, bins=edges)
    r = 0.5 * (edges[1:] + edges[:-1])
    lny = np.log(h / (r * r))
    assert np.all(h > 50), h
    assert lny.max() - lny.min() < 0.6, (h, lny)
