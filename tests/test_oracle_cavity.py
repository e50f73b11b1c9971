"""Pins the oracle's cavity sampling (oracle/hsmc_oracle.c, hso_cavity_*) to
the reference's own code: the golden fixtures of tests/golden/cavity_vectors.npz
(made by tests/golden/make_cavity_golden.py) and, where the reference build
exists, a side-by-side run.  The umbrella potential, the sweeps' trajectories
and the replayed trials must be bit-identical."""
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "cavity_vectors.npz")

# as in make_cavity_golden.py
CASES = {
    "rho080_n3": dict(rho=0.80, n_cells=3, seed=4, dr_max=0.10, pcav=0.10, maxdr=1.2, mindr=0.0, sweeps=30),
    "rho050_n4": dict(rho=0.50, n_cells=4, seed=6, dr_max=0.30, pcav=0.30, maxdr=1.1, mindr=0.6, sweeps=20),
}


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


@pytest.mark.parametrize("name", list(CASES))
def test_cavity_matches_reference_fixtures(oracle_mod, golden, name):
    kw = CASES[name]
    O = oracle_mod.OracleSim
    psi = O.cavity_psi(kw["rho"], golden["psi_x"])
    assert np.array_equal(psi.view(np.uint64), golden[f"{name}/psi"].view(np.uint64))
    o = O(rho=kw["rho"], n_cells=kw["n_cells"], seed=kw["seed"], dr_max=kw["dr_max"])
    o.cavity_setup(kw["pcav"], kw["maxdr"], kw["mindr"])
    assert np.array_equal(o.get_config(), golden[f"{name}/start"])
    o.cavity_sweeps(kw["sweeps"])
    assert np.array_equal(o.get_config(), golden[f"{name}/config"])
    assert np.array_equal(o.counters(), golden[f"{name}/counters"])
    r = O(rho=kw["rho"], n_cells=kw["n_cells"], seed=kw["seed"], dr_max=kw["dr_max"])
    r.cavity_setup(kw["pcav"], 3.0, 0.0)
    r.set_config(golden[f"{name}/config"])
    dec = r.cavity_replay(golden[f"{name}/rp_which"], golden[f"{name}/rp_raw"], golden[f"{name}/rp_uacc"])
    assert np.array_equal((dec == 0).astype(np.int32), golden[f"{name}/rp_acc"])
    assert np.array_equal(r.get_config(), golden[f"{name}/rp_config"])
    assert {1, 2, 3} & set(dec.tolist()) and 0 in dec


def test_cavity_potential_shape(oracle_mod):
    """ln y is large inside the core and matches ln g_VW at contact; the
    cubic and the outer branch meet at x = 1 to within a few 1e-3."""
    x = np.array([0.0, 0.5, 1.0 - 1e-12, 1.0, 1.2])
    psi = oracle_mod.OracleSim.cavity_psi(0.8, x)
    assert psi[0] > psi[1] > psi[3] > psi[4] > 0
    assert abs(psi[2] - psi[3]) < 5e-3


def test_cavity_side_by_side(oracle_mod, ref_available):
    if not ref_available:
        pytest.skip("reference sources not present")
    kw = dict(rho=0.7, n_cells=3, seed=12, dr_max=0.2)
    o = oracle_mod.OracleSim(**kw)
    r = oracle_mod.RefSim(**kw)
    o.cavity_setup(0.2, 1.3, 0.4)
    r.cavity_setup(0.2, 1.3, 0.4)
    o.cavity_sweeps(15)
    r.cavity_sweeps(15)
    assert np.array_equal(o.get_config(), r.get_config())
    assert np.array_equal(o.counters(), r.counters())
