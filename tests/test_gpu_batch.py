"""Batched replicas: one launch per kernel for all systems; each replica must
be the chain a single context runs (replica 0 bit for bit), stay
overlap-free, and give the single-context observables on its configuration."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_replica_zero_is_the_single_system_chain(gpu_lib):
    from hsmc_gb300.batch import ReplicaBatch

    systems = [(0.80, 6, 0.15, 77), (0.50, 4, 0.30, 78), (0.92, 5, 0.08, 79)]
    b = ReplicaBatch(systems)
    c = b.sweeps(27)  # three graph launches and a remainder
    s = gpu_lib.HardSphereSystem(rho=0.80, cells=6, dr_max=0.15, seed=77)
    cs = s.sweep_nvt(27)
    assert np.array_equal(b.download(0), s.download())
    assert np.array_equal(c[0], cs)


def test_replica_with_larger_cells_is_the_single_system_chain(gpu_lib):
    """A minimum cell edge is part of the chain's definition: the replica and
    a single context given the same edge run the same chain (replica 0; the
    replica index is part of the others' random counters)."""
    from hsmc_gb300.batch import ReplicaBatch

    systems = [(0.45, 6, 0.3, 5), (0.80, 6, 0.15, 6), (0.30, 7, 0.4, 7)]
    b = ReplicaBatch(systems, min_cell_edge="auto")
    c = b.sweeps(23)
    rho, n, dr, seed = systems[0]
    s = gpu_lib.HardSphereSystem(rho=rho, cells=n, dr_max=dr, seed=seed,
                                 min_cell_edge=min(rho ** (-1.0 / 3.0), 1.4))
    cs = s.sweep_nvt(23)
    assert np.array_equal(b.download(0), s.download())
    assert np.array_equal(c[0], cs)
    for k in (1, 2):
        assert 0 < c[k, 1] < c[k, 0]


def test_uneven_replicas_stay_overlap_free(oracle_mod, gpu_lib):
    from hsmc_gb300.batch import ReplicaBatch

    rng = np.random.default_rng(3)
    systems = []
    for k in range(12):
        n = int(rng.integers(3, 8))
        rho = float(rng.uniform(0.3, 0.94))
        systems.append((rho, n, 0.1 if rho > 0.8 else 0.25, 100 + k))
    b = ReplicaBatch(systems)
    c = b.sweeps(40)
    for k, (rho, n, dr, seed) in enumerate(systems):
        assert c[k, 0] == 40 * b.n[k]
        assert 0.0 < c[k, 1] < c[k, 0]
        conf = b.download(k)
        L = b.box[k][0]
        assert np.all(conf[:, 1:] >= 0) and np.all(conf[:, 1:] <= L)
        for i in range(0, b.n[k], 7):
            assert oracle_mod.OracleSim.brute_overlap(conf, b.box[k], i, *conf[i, 1:]) == 0


def test_batched_virial_counts_match_single(gpu_lib):
    from hsmc_gb300.batch import ReplicaBatch

    systems = [(0.6, 5, 0.2, 1), (0.85, 6, 0.12, 2), (0.4, 4, 0.3, 3)]
    b = ReplicaBatch(systems)
    b.sweeps(30)
    nb, dr = 5, 0.01
    rmax = dr * nb + 1.0
    got = b.pressv_counts(dr, rmax, nb)
    for k, (rho, n, d, seed) in enumerate(systems):
        s = gpu_lib.HardSphereSystem(rho=rho, cells=n, dr_max=d, seed=seed, conf=b.download(k))
        assert np.array_equal(got[k], s.compute_pressv_counts(dr, rmax, nb))


def test_replica_pressures_follow_carnahan_starling(gpu_lib):
    """Per-replica contact pressure after equilibration, against CS within a
    loose band set by the short run (the statistical gate is on C1)."""
    from hsmc_gb300.batch import ReplicaBatch

    rhos = [0.3, 0.5, 0.7]
    b = ReplicaBatch([(r, 6, 0.3 if r < 0.6 else 0.15, 10 + i) for i, r in enumerate(rhos)])
    b.sweeps(500)
    nb, dr = 5, 0.01
    rmax = dr * nb + 1.0
    acc = np.zeros((len(rhos), nb))
    samples = 50
    for _ in range(samples):
        b.sweeps(10)
        acc += b.pressv_counts(dr, rmax, nb)
    r = (np.arange(nb) + 0.5) * dr + 1.0
    vol = 4 * np.pi / 3 * ((r + dr / 2) ** 3 - (r - dr / 2) ** 3)
    for k, rho in enumerate(rhos):
        g = acc[k] / samples / (vol * rho * b.n[k])
        b1, b0 = np.polyfit(r, g, 1)
        z = 1 + 2 * np.pi / 3 * rho * (b0 + b1)
        eta = math.pi * rho / 6
        z_cs = (1 + eta + eta**2 - eta**3) / (1 - eta) ** 3
        assert abs(z - z_cs) < 0.12 * z_cs, (rho, z, z_cs)


def _persistent_vs_flat(systems, sweeps, variants, min_cell_edge=0.0, schedule=1):
    from hsmc_gb300.batch import ReplicaBatch

    flat = ReplicaBatch(systems, min_cell_edge=min_cell_edge)
    want_c = sum(flat.sweeps(n) for n in sweeps)
    want = [flat.download(k) for k in range(len(systems))]
    flat.close()
    for cb, tile in variants:
        b = ReplicaBatch(systems, min_cell_edge=min_cell_edge)
        b.set_schedule(schedule, cb, tile)
        assert b.get_schedule() == (schedule, cb, tile)
        got_c = sum(b.sweeps(n) for n in sweeps)
        for k in range(len(systems)):
            assert np.array_equal(b.download(k), want[k]), (cb, tile, k)
        assert np.array_equal(got_c, want_c), (cb, tile)
        b.close()


def test_persistent_schedule_is_the_flat_chain(gpu_lib):
    """Every sweep of a call in one launch of thread-block clusters, one
    cluster per bundle of replicas: every replica's configuration and
    counters bit-identical to the flat launches', for several cluster sizes
    and tiles (one replica per bundle up to many), over calls of 1, 7 and 16
    sweeps."""
    rng = np.random.default_rng(11)
    systems = [(float(rng.uniform(0.3, 0.94)), int(rng.integers(3, 9)), 0.12, 300 + k) for k in range(40)]
    _persistent_vs_flat(systems, [1, 7, 16], [(1, 1), (2, 2), (4, 1), (8, 4)])


def test_persistent_schedule_mixed_cell_capacities(gpu_lib):
    """Larger cells (16 and 32 slots, 4 and 8 lanes per cell) in the same
    batch: one persistent launch per capacity, still the flat chain."""
    systems = [(0.45, 6, 0.3, 5), (0.80, 6, 0.15, 6), (0.30, 7, 0.4, 7), (0.60, 5, 0.25, 8)]
    _persistent_vs_flat(systems, [9], [(2, 1), (4, 2)], min_cell_edge="auto")


def test_grid_schedule_is_the_flat_chain(gpu_lib):
    """Every sweep of a call in one cooperative launch over the whole device
    per cell capacity, with grid barriers between the build and the passes:
    every replica's configuration and counters bit-identical to the flat
    launches', over calls of 1, 7 and 16 sweeps, and with 16- and 32-slot
    cells in the same batch."""
    rng = np.random.default_rng(12)
    systems = [(float(rng.uniform(0.3, 0.94)), int(rng.integers(3, 9)), 0.12, 500 + k) for k in range(40)]
    _persistent_vs_flat(systems, [1, 7, 16], [(4, 2)], schedule=2)
    mixed = [(0.45, 6, 0.3, 5), (0.80, 6, 0.15, 6), (0.30, 7, 0.4, 7), (0.60, 5, 0.25, 8)]
    _persistent_vs_flat(mixed, [9], [(4, 2)], min_cell_edge="auto", schedule=2)


def test_occupancy_order_is_the_flat_chain(gpu_lib):
    """The flat launches with each pass's cells over every replica listed
    fullest first (schedule 3): every replica's configuration and counters
    bit-identical to the grid-order flat launches', over calls of 1, 7 and 16
    sweeps, with 16- and 32-slot cells in the same batch, and replica 0
    against a single context with switches between the orders."""
    rng = np.random.default_rng(13)
    systems = [(float(rng.uniform(0.3, 0.94)), int(rng.integers(3, 9)), 0.12, 700 + k) for k in range(40)]
    _persistent_vs_flat(systems, [1, 7, 16], [(4, 2)], schedule=3)
    mixed = [(0.45, 6, 0.3, 5), (0.80, 6, 0.15, 6), (0.30, 7, 0.4, 7), (0.60, 5, 0.25, 8)]
    _persistent_vs_flat(mixed, [9], [(4, 2)], min_cell_edge="auto", schedule=3)
    from hsmc_gb300.batch import ReplicaBatch

    b = ReplicaBatch([(0.80, 6, 0.15, 77), (0.50, 4, 0.30, 78)])
    s = gpu_lib.HardSphereSystem(rho=0.80, cells=6, dr_max=0.15, seed=77)
    for sch, n in ((3, 11), (0, 5), (3, 8)):
        b.set_schedule(sch)
        c = b.sweeps(n)
        cs = s.sweep_nvt(n)
        assert np.array_equal(b.download(0), s.download()) and np.array_equal(c[0], cs), sch
    b.close()
    s.close()


def test_grid_schedule_replica_zero_and_observables(gpu_lib):
    """Replica 0 under the grid schedule is the single context's chain, the
    layout it leaves serves the observables, and the flat launches continue
    the same chain."""
    from hsmc_gb300.batch import ReplicaBatch

    systems = [(0.80, 6, 0.15, 77), (0.50, 4, 0.30, 78), (0.92, 5, 0.08, 79)]
    b = ReplicaBatch(systems)
    b.set_schedule(2)
    c = b.sweeps(27)
    s = gpu_lib.HardSphereSystem(rho=0.80, cells=6, dr_max=0.15, seed=77)
    cs = s.sweep_nvt(27)
    assert np.array_equal(b.download(0), s.download())
    assert np.array_equal(c[0], cs)
    nb, dr = 5, 0.01
    got = b.pressv_counts(dr, 1.0 + nb * dr, nb)
    for k, (rho, n, d, seed) in enumerate(systems):
        t = gpu_lib.HardSphereSystem(rho=rho, cells=n, dr_max=d, seed=seed, conf=b.download(k))
        assert np.array_equal(got[k], t.compute_pressv_counts(dr, 1.0 + nb * dr, nb))
        t.close()
    b.set_schedule(0)
    b.sweeps(5)
    s.sweep_nvt(5)
    assert np.array_equal(b.download(0), s.download())
    b.close()
    s.close()


def test_persistent_replica_zero_and_observables(gpu_lib):
    """Replica 0 under the persistent schedule is the single context's chain,
    and the layout it leaves behind serves the observables (virial counts
    equal a single context's on the same configuration)."""
    from hsmc_gb300.batch import ReplicaBatch

    systems = [(0.80, 6, 0.15, 77), (0.50, 4, 0.30, 78), (0.92, 5, 0.08, 79)]
    b = ReplicaBatch(systems)
    b.set_schedule(1, 2, 1)
    c = b.sweeps(27)
    s = gpu_lib.HardSphereSystem(rho=0.80, cells=6, dr_max=0.15, seed=77)
    cs = s.sweep_nvt(27)
    assert np.array_equal(b.download(0), s.download())
    assert np.array_equal(c[0], cs)
    nb, dr = 5, 0.01
    got = b.pressv_counts(dr, 1.0 + nb * dr, nb)
    for k, (rho, n, d, seed) in enumerate(systems):
        t = gpu_lib.HardSphereSystem(rho=rho, cells=n, dr_max=d, seed=seed, conf=b.download(k))
        assert np.array_equal(got[k], t.compute_pressv_counts(dr, 1.0 + nb * dr, nb))
    # switching back to the flat launches continues the same chain
    b.set_schedule(0)
    b.sweeps(5)
    s.sweep_nvt(5)
    assert np.array_equal(b.download(0), s.download())


def test_batch_autotune_keeps_the_chain(gpu_lib):
    from hsmc_gb300.batch import ReplicaBatch

    systems = [(0.7, 5, 0.2, 40 + k) for k in range(6)]
    a = ReplicaBatch(systems)
    sched = a.autotune(8)
    assert sched[0] in (0, 1, 2, 3) and sched[1] in (1, 2, 4, 8) and sched[2] in (1, 2, 4)
    assert a.get_schedule() == sched
    a.sweeps(10)
    # the same tuning sweeps, then another schedule: the same chain
    b = ReplicaBatch(systems)
    b.autotune(8)
    b.set_schedule(1 if sched[0] != 1 else 0, 2, 2)
    b.sweeps(10)
    for k in range(len(systems)):
        assert np.array_equal(a.download(k), b.download(k))
