"""Geometric cluster moves on the GPU against the oracle (pinned to the
reference's cluster_nvt.c by tests/test_oracle_cluster.py): cluster sizes and
every moved position bit-identical, the random stream resumable, no overlap
ever created, and the pressure of a cluster-move run on Carnahan-Starling."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# systems up to a few thousand spheres run in one block's shared memory; the
# last case (N = 6912) takes the grid-wide kernel
CASES = [(0.30, 6, 1, 0.40), (0.50, 5, 2, 0.25), (0.85, 6, 3, 0.12), (0.45, 12, 4, 0.3)]


def _pair(oracle_mod, gpu_lib, rho, n, seed, dr):
    o = oracle_mod.OracleSim(rho=rho, n_cells=n, seed=seed, dr_max=dr, neigh_dr=1.05)
    o.sweeps_nvt(15)
    g = gpu_lib.HardSphereSystem(rho=rho, cells=n, dr_max=dr, seed=seed + 1000, conf=o.get_config())
    return o, g


@pytest.mark.parametrize("rho,n,seed,dr", CASES)
def test_cluster_move_at_bit_exact(oracle_mod, gpu_lib, rho, n, seed, dr):
    o, g = _pair(oracle_mod, gpu_lib, rho, n, seed, dr)
    rng = np.random.default_rng(seed)
    L = np.array(g.box)
    sizes = []
    for _ in range(12):
        piv = rng.uniform(0.0, 1.0, 3) * L
        axis = int(rng.integers(0, 3))
        s = int(rng.integers(0, g.n))
        got = g.cluster_move_at(piv, axis, s)
        assert got == o.cluster_move_at(piv, axis, s)
        assert np.array_equal(g.download(), o.get_config())
        sizes.append(got)
    assert max(sizes) > 1


@pytest.mark.parametrize("rho,n,seed,dr", [CASES[0], CASES[1], CASES[3]])
def test_drawn_cluster_moves_replay_on_the_oracle(oracle_mod, gpu_lib, rho, n, seed, dr):
    o, g = _pair(oracle_mod, gpu_lib, rho, n, seed, dr)
    sizes, drawn = g.cluster_moves(30, drawn=True)
    L = np.array(g.box)
    assert np.all(drawn[:, :3] > 0) and np.all(drawn[:, :3] < L)
    assert set(drawn[:, 3].astype(int)) <= {0, 1, 2} and len(set(drawn[:, 3].astype(int))) > 1
    assert np.all((drawn[:, 4] >= 0) & (drawn[:, 4] < g.n))
    for k in range(30):
        assert o.cluster_move_at(drawn[k, :3], int(drawn[k, 3]), int(drawn[k, 4])) == sizes[k]
    assert np.array_equal(g.download(), o.get_config())


def test_cluster_stream_resumes(gpu_lib):
    a = gpu_lib.HardSphereSystem(rho=0.5, cells=4, dr_max=0.25, seed=9)
    a.sweep_nvt(5)
    a.cluster_moves(3)
    conf, st = a.download(), a.rng_state()
    assert st[3] == 3
    s1 = a.cluster_moves(10)
    a.sweep_nvt(2)
    b = gpu_lib.HardSphereSystem(rho=0.5, cells=4, dr_max=0.25, seed=1, conf=conf)
    b.rng_set_state(st)
    assert np.array_equal(b.cluster_moves(10), s1)
    b.sweep_nvt(2)
    assert np.array_equal(a.download(), b.download())


def test_mixed_local_and_cluster_moves_stay_overlap_free(oracle_mod, gpu_lib):
    g = gpu_lib.HardSphereSystem(rho=0.6, cells=8, dr_max=0.2, seed=17)
    for _ in range(5):
        g.sweep_nvt(4)
        sizes = g.cluster_moves(5)
        assert np.all(sizes >= 1) and np.all(sizes <= g.n)
    conf = g.download()
    for i in range(0, g.n, 11):
        assert oracle_mod.OracleSim.brute_overlap(conf, g.box, i, *conf[i, 1:]) == 0


def test_cluster_moves_refused_for_npt(gpu_lib):
    g = gpu_lib.HardSphereSystem(rho=0.5, cells=4, pressure=3.0, dv_max=0.01, seed=2)
    with pytest.raises(gpu_lib.HsmcError) as ei:
        g.cluster_moves(1)
    assert ei.value.code == 1


def test_cluster_pressure_matches_carnahan_starling(gpu_lib):
    """Packing fraction 0.25 (the reference's own comparison of cluster and
    local moves): contact pressure from cluster moves only, in 10 blocks,
    within 3 standard errors (plus the 0.5 % bias of the linear contact fit)
    of Carnahan-Starling."""
    from hsmc_gb300.batch import carnahan_starling, contact_z

    rho = 6 * 0.25 / math.pi
    g = gpu_lib.HardSphereSystem(rho=rho, cells=5, dr_max=0.4, seed=31)
    g.sweep_nvt(200)  # melt the lattice, as cluster_init_step does
    g.cluster_moves(500)
    nb, dr = 5, 0.01
    blocks, per_block, every = 10, 200, 5
    z = []
    for _ in range(blocks):
        cnt = np.zeros(nb)
        for _ in range(per_block):
            g.cluster_moves(every)
            cnt += g.compute_pressv_counts(dr, 1.0 + nb * dr, nb)
        z.append(contact_z(cnt, per_block, g.n, rho, dr))
    z = np.array(z)
    se = z.std(ddof=1) / math.sqrt(blocks)
    zcs = carnahan_starling(rho)
    assert abs(z.mean() - zcs) < 3 * se + 0.005 * zcs, (z.mean(), se, zcs)
