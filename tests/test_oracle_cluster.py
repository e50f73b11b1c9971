"""Pins the oracle's cluster moves (oracle/hsmc_oracle.c, hso_cluster_*) to
the reference's own cluster-move code: the golden fixtures of
tests/golden/cluster_vectors.npz (made by tests/golden/make_cluster_golden.py)
and, where the reference build exists, a side-by-side run.  Sizes and
configurations must be bit-identical."""
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "cluster_vectors.npz")

# as in make_cluster_golden.py
CASES = {
    "rho040_n3": dict(rho=0.40, n_cells=3, lattice_type=2, neigh_dr=1.05, seed=5, dr_max=0.30, sweeps=20, moves=40),
    "rho030_sc6": dict(rho=0.30, n_cells=6, lattice_type=1, neigh_dr=1.10, seed=9, dr_max=0.40, sweeps=10,
                       moves=40),
    "rho070_n4": dict(rho=0.70, n_cells=4, lattice_type=2, neigh_dr=1.05, seed=3, dr_max=0.20, sweeps=20, moves=8),
}


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


def _sim(oracle_mod, kw, cls=None):
    cls = cls or oracle_mod.OracleSim
    return cls(rho=kw["rho"], n_cells=kw["n_cells"], lattice_type=kw["lattice_type"], neigh_dr=kw["neigh_dr"],
               seed=kw["seed"], dr_max=kw["dr_max"])


@pytest.mark.parametrize("name", list(CASES))
def test_cluster_moves_match_reference_fixtures(oracle_mod, golden, name):
    kw = CASES[name]
    o = _sim(oracle_mod, kw)
    o.sweeps_nvt(kw["sweeps"])
    assert np.array_equal(o.get_config(), golden[f"{name}/start"])
    sizes = o.cluster_moves(kw["moves"])
    assert np.array_equal(sizes, golden[f"{name}/sizes"])
    assert np.array_equal(o.get_config(), golden[f"{name}/config"])
    got = [o.cluster_move_at(p, a, s) for p, a, s in
           zip(golden[f"{name}/at_pivot"], golden[f"{name}/at_axis"], golden[f"{name}/at_seed"])]
    assert np.array_equal(np.array(got), golden[f"{name}/at_sizes"])
    assert np.array_equal(o.get_config(), golden[f"{name}/at_config"])


def test_cluster_moves_keep_spheres_apart(oracle_mod):
    """A cluster move never creates an overlap (the rotation is an isometry
    and every overlapping particle joins the cluster)."""
    o = oracle_mod.OracleSim(rho=0.45, n_cells=4, seed=21, dr_max=0.3)
    o.sweeps_nvt(15)
    o.cluster_moves(30)
    conf = o.get_config()
    box = [o.box()["lx"]] * 3
    for i in range(0, o.n, 5):
        assert oracle_mod.OracleSim.brute_overlap(conf, box, i, *conf[i, 1:]) == 0


def test_cluster_moves_side_by_side(oracle_mod, ref_available):
    if not ref_available:
        pytest.skip("reference sources not present")
    kw = dict(rho=0.5, n_cells=3, lattice_type=2, neigh_dr=1.05, seed=44, dr_max=0.25)
    o = _sim(oracle_mod, kw)
    r = _sim(oracle_mod, kw, oracle_mod.RefSim)
    o.sweeps_nvt(12)
    r.sweeps_nvt(12)
    assert np.array_equal(o.cluster_moves(25), r.cluster_moves(25))
    assert np.array_equal(o.get_config(), r.get_config())
