"""GPU parity against the CPU oracle (the reference algorithm restated in C,
pinned to the reference's own code by tests/test_oracle.py).

Decisions and integer counts must be bit-identical; q_l, a floating-point
mean, must agree to 1e-12 relative.  Every call goes through the C ABI.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def fluid(oracle_mod, gpu, rho, n, seed, dr, sweeps=30, neigh_dr=1.05, lanes=0, min_edge=0.0):
    """An oracle system run from the lattice (the reference's own chain) and a
    GPU system started from the same configuration."""
    o = oracle_mod.OracleSim(rho=rho, n_cells=n, seed=seed, dr_max=dr, neigh_dr=neigh_dr,
                             neigh_max_part=10 if neigh_dr < 1.2 else 40)
    if sweeps:
        o.sweeps_nvt(sweeps)
    conf = o.get_config()
    g = gpu.HardSphereSystem(rho=rho, cells=n, dr_max=dr, seed=seed + 1000, conf=conf, lanes_per_cell=lanes,
                             min_cell_edge=min_edge)
    return o, g, conf


CASES = [(0.50, 5, 1, 0.3), (0.85, 6, 7, 0.12), (0.94, 5, 3, 0.08)]


@pytest.mark.parametrize("rho,n,seed,dr", CASES)
def test_overlap_decisions_bit_exact(oracle_mod, gpu_lib, rho, n, seed, dr):
    o, g, conf = fluid(oracle_mod, gpu_lib, rho, n, seed, dr)
    L = o.box()["lx"]
    rng = np.random.default_rng(seed)
    ids, pos = [], []
    # ordinary trial moves (part_move arithmetic) ...
    for _ in range(3000):
        i = int(rng.integers(0, o.n))
        u = rng.integers(0, 2**32 - 1, size=3, dtype=np.uint64).astype(np.float64) / 4294967295.0
        p = conf[i, 1:] + (u - 0.5) * dr
        p = np.where(p > L, p - L, np.where(p < 0.0, p + L, p))
        ids.append(i)
        pos.append(p)
    # ... and adversarial ones at |r| = 1 within a few ulps of a neighbour
    for _ in range(3000):
        i = int(rng.integers(0, o.n))
        j = int(rng.integers(0, o.n))
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        d *= 1.0 + rng.integers(-4, 5) * 2.0**-52
        p = np.mod(conf[j, 1:] + d, L)
        ids.append(i)
        pos.append(p)
    ids = np.array(ids, dtype=np.int32)
    pos = np.array(pos)
    got = g.overlap_replay(ids, pos)
    want = np.array([o.check_overlap_at(int(i), *p) for i, p in zip(ids, pos)], dtype=np.uint8)
    assert np.array_equal(got, want)
    assert 0 < want.sum() < len(want)


@pytest.mark.parametrize("lanes", [1, 2, 4, 8])
@pytest.mark.parametrize("rho,n,seed,dr,edge", [c + (0.0,) for c in CASES] +
                         [(0.70, 10, 5, 0.2, 0.0), (0.40, 8, 9, 0.3, 1.2), (0.60, 8, 11, 0.25, 1.6),
                          (1.25, 6, 13, 0.05, 0.0)])
def test_traced_sweeps_replay_bit_exact(oracle_mod, gpu_lib, rho, n, seed, dr, edge, lanes):
    """Every trial of a few sweeps replayed on the oracle; edge > 0 asks for
    larger device cells (edges 1.23 and 1.88 here: capacity 16 and 32).  The
    fcc crystal at rho = 1.25 (8 cells of edge 1.105 per axis, 1.7 spheres
    per cell) overfills the shared-memory neighbour pool of most cells, so
    their trials screen straight from global memory."""
    from oracle.philox import TAG_MOVE, draw4

    if edge > 1.41 and lanes == 1:
        # 32-slot cells with one lane each do not fit a block's shared memory
        with pytest.raises(gpu_lib.HsmcError) as ei:
            fluid(oracle_mod, gpu_lib, rho, n, seed, dr, sweeps=0, lanes=lanes, min_edge=edge)
        assert ei.value.code == 1
        return
    o, g, conf = fluid(oracle_mod, gpu_lib, rho, n, seed, dr, sweeps=10, lanes=lanes, min_edge=edge)
    if edge:
        nc, _, _, _ = g.grid_info()
        assert all(g.box[d] / nc[d] >= edge for d in range(3))
    if rho > 1.2:
        # particles in the 26 neighbour cells of each cell (unshifted grid):
        # beyond the 34 pool entries of two lanes per cell for most cells
        nc, _, _, _ = g.grid_info()
        w = np.array([g.box[d] / nc[d] for d in range(3)])
        idx = np.floor(conf[:, 1:] / w).astype(int) % np.array(nc)
        occ = np.zeros(tuple(nc))
        np.add.at(occ, tuple(idx.T), 1)
        around = sum(np.roll(occ, (dx, dy, dz), axis=(0, 1, 2))
                     for dx in (-1, 0, 1) for dy in (-1, 0, 1) for dz in (-1, 0, 1)) - occ
        assert np.mean(around > 34) > 0.5
    sweeps = 4
    rec, cnt = g.sweeps_traced(sweeps)
    assert len(rec) == o.n * sweeps
    assert cnt[0] == o.n * sweeps
    order = np.lexsort((rec[:, 2], rec[:, 1], rec[:, 0]))
    rec = rec[order]
    # the recorded draws are the Philox stream the kernel was meant to use
    r = draw4(seed + 1000, rec[:, 2], rec[:, 1], rec[:, 0].astype(np.uint64) + (np.uint64(0)), TAG_MOVE)
    assert np.array_equal(rec[:, 4], r[1]) and np.array_equal(rec[:, 5], r[2]) and np.array_equal(rec[:, 6], r[3])
    nc, l32, iw, _ = g.grid_info()
    shifts = rec[:, 8:11].copy().view(np.float32)
    o.reset_counters()
    dec = o.replay_checkerboard(rec[:, 3].astype(np.int32), rec[:, 4:7], rec[:, 1], shifts, nc, l32, iw)
    assert not np.any(dec == 3), "a traced particle was not in its cell"
    assert np.array_equal(dec, rec[:, 7].astype(np.int32))
    assert np.array_equal(o.get_config(), g.download())
    assert cnt[1] == np.sum(dec == 0)


def test_chain_independent_of_lane_mapping(gpu_lib):
    """Same seed, same trajectory whatever the number of lanes per cell."""
    finals = []
    for lanes in (1, 2, 4, 8):
        g = gpu_lib.HardSphereSystem(rho=0.8, cells=8, dr_max=0.15, seed=123, lanes_per_cell=lanes)
        g.set_schedule(0)  # the pass-barrier launches, where the lane mapping applies
        c = g.sweep_nvt(37)
        finals.append((g.download(), c.copy()))
    for conf, c in finals[1:]:
        assert np.array_equal(conf, finals[0][0]) and np.array_equal(c, finals[0][1])


@pytest.mark.parametrize("rho,n,seed,dr", CASES)
def test_rdf_and_virial_counts_bit_exact(oracle_mod, gpu_lib, rho, n, seed, dr):
    o, g, conf = fluid(oracle_mod, gpu_lib, rho, n, seed, dr)
    hist, rmax = o.rdf_counts(0.01, 5.0)
    got = g.compute_rdf_counts(0.01, rmax, len(hist))
    assert np.array_equal(got, hist.astype(np.uint64))
    assert np.array_equal(got, oracle_mod.OracleSim.brute_pair_hist(conf, [o.box()["lx"]] * 3, 0.01, rmax, len(hist)))
    pv, prmax = o.pressv_counts(0.01)
    gpv = g.compute_pressv_counts(0.01, prmax, len(pv))
    assert np.array_equal(gpv, pv.astype(np.uint64))


def test_volume_scan_near_unit_scale_factor(oracle_mod, gpu_lib):
    """A pair 2^-51 short of contact, as the rescale of an accepted volume
    move can leave one: the reference's scan reports an overlap at sf = 1
    and at sf = 1 + 2^-52 (an expansion too small to clear the deficit) and
    none once sf clears it; the device scan gives the same at every sf,
    expansions included."""
    o = oracle_mod.OracleSim(rho=0.5, n_cells=4, seed=1, dr_max=0.1)
    L = o.box()["lx"]
    s = L / 7
    y0 = z0 = 3.5 * s
    pts = [(2.0, y0, z0), (3.0 - 2.0**-51, y0, z0)]  # 1 - 2^-51 apart (both exact)
    for k in range(7):
        for j in range(7):
            for i in range(7):
                if not (j == 3 and k == 3 and i in (1, 2, 3)):
                    pts.append(((i + 0.5) * s, (j + 0.5) * s, (k + 0.5) * s))
    conf = np.zeros((o.n, 4))
    conf[:, 0] = np.arange(o.n)
    conf[:, 1:] = pts[: o.n]
    o.set_config(conf)
    g = gpu_lib.HardSphereSystem(rho=0.5, cells=4, dr_max=0.1, seed=1, conf=conf)
    sfs = [0.999, 1.0 - 2.0**-52, 1.0, 1.0 + 2.0**-52, 1.0 + 2.0**-50, 1.0 + 1e-13, 1.0 + 1e-9, 1.001]
    want = [o.scan_overlap(x) for x in sfs]
    assert want[:4] == [1, 1, 1, 1] and want[4:] == [0, 0, 0, 0], want
    assert [g.scan_overlap(x) for x in sfs] == want
    g.close()


@pytest.mark.parametrize("rho,n,seed,dr", CASES)
def test_thermo_pressure_scan_bit_exact(oracle_mod, gpu_lib, rho, n, seed, dr):
    o, g, _ = fluid(oracle_mod, gpu_lib, rho, n, seed, dr)
    xi = [(k + 1) * 0.0001 for k in range(int(0.002 / 0.0001))]
    sf = np.array([math.pow(1 - x, 1.0 / 3.0) for x in xi])
    assert np.array_equal(g.compute_presst(sf), o.presst_counts_sf(sf).astype(np.uint64))
    assert np.array_equal(o.presst_counts_sf(sf), o.presst_counts(0.0001, 0.002))
    for s in (0.99999, 0.9999, 0.999, 0.99):
        assert g.scan_overlap(s) == o.scan_overlap(s)


@pytest.mark.parametrize("rho,n,seed,dr", CASES)
def test_widom_decisions_bit_exact(oracle_mod, gpu_lib, rho, n, seed, dr):
    o, g, _ = fluid(oracle_mod, gpu_lib, rho, n, seed, dr)
    L = o.box()["lx"]
    raw = np.random.default_rng(seed).integers(0, 2**32 - 1, size=3 * 20000, dtype=np.uint32)
    pos = (raw.astype(np.float64) / 4294967295.0 * L).reshape(-1, 3)
    assert np.array_equal(g.widom_replay(pos), o.widom_decisions(raw))
    # the device's own insertion points: (2r + 1) * 2^-33 * L
    pos2 = ((2.0 * raw.astype(np.float64) + 1.0) * 2.0**-33 * L).reshape(-1, 3)
    ov = g.widom_replay(pos2)
    assert np.array_equal(ov, o.widom_points(pos2))
    # the device's random insertions count the same decisions on average
    ok = g.widom_insertion(20000)
    assert abs(ok / 20000 - (1 - ov.mean())) < 5 * np.sqrt(max(ov.mean() * (1 - ov.mean()), 1e-4) / 20000) + 1e-3


@pytest.mark.parametrize("rho,n,seed,dr", CASES)
def test_ql_matches(oracle_mod, gpu_lib, rho, n, seed, dr):
    o, g, _ = fluid(oracle_mod, gpu_lib, rho, n, seed, dr, neigh_dr=1.5)
    for l in (4, 6):
        mean, per, rc = o.ql(l, 1.5)
        gm, gper = g.global_ql(l, rc, per_particle=True)
        assert abs(gm - mean) <= 1e-12 * abs(mean)
        assert np.max(np.abs(gper - per)) <= 1e-12


def test_large_system_stays_overlap_free(oracle_mod, gpu_lib):
    """N = 256,000 at rho = 0.85 from the FCC lattice: after sweeps every
    particle passes the reference overlap test at its own position."""
    g = gpu_lib.HardSphereSystem(rho=0.85, cells=40, dr_max=0.12, seed=11)
    c = g.sweep_nvt(20)
    assert c[0] == 256000 * 20
    acc = c[1] / c[0]
    assert 0.2 < acc < 0.9
    conf = g.download()
    ids = np.arange(g.n, dtype=np.int32)
    assert g.overlap_replay(ids, conf[:, 1:]).sum() == 0
    o = oracle_mod.OracleSim(rho=0.85, n_cells=40, seed=1, dr_max=0.12)
    o.set_config(conf)
    rng = np.random.default_rng(0)
    for i in rng.integers(0, g.n, size=500):
        assert o.check_overlap_at(int(i), *conf[i, 1:]) == 0
    # integer g(r) counts of the full system: every pair counted from both ends
    hist = g.compute_rdf_counts(0.01, 5.0, 400)
    assert hist.sum() % 2 == 0 and hist[0] > 0


def test_error_paths_report_reference_messages(gpu_lib):
    conf = gpu_lib.lattice_config(0.5, (5, 5, 5))
    g = gpu_lib.HardSphereSystem(rho=0.5, cells=5, conf=conf)
    bad = conf.copy()
    bad[3, 1] = -0.5
    with pytest.raises(gpu_lib.HsmcError) as ei:
        g.upload(bad)
    assert ei.value.code == 8
    crowd = conf.copy()
    crowd[:, 1:] = 1.0  # every particle in one cell
    with pytest.raises(gpu_lib.HsmcError) as ei:
        g.upload(crowd)
    assert ei.value.code == 4
    g.upload(conf)
    g.sweep_nvt(2)
    # an NpT run re-derives its grid on the device with the standard edge
    with pytest.raises(gpu_lib.HsmcError) as ei:
        gpu_lib.HardSphereSystem(rho=0.5, cells=5, pressure=3.0, dv_max=0.01, min_cell_edge=1.2)
    assert ei.value.code == 1


@pytest.mark.parametrize("lanes", [1, 2, 4, 8])
def test_dataflow_schedule_is_the_pass_barrier_chain(gpu_lib, lanes):
    """All eight passes in one cooperative launch, each cell waiting only for
    its neighbourhood, give the chain of one launch per pass bit for bit."""
    confs = []
    for schedule in (0, 1):
        s = gpu_lib.HardSphereSystem(rho=0.8, cells=8, dr_max=0.15, seed=42)
        s.set_schedule(schedule, lanes)
        assert s.get_schedule() == (schedule, lanes)
        c = s.sweep_nvt(27)
        confs.append((s.download(), c))
    assert np.array_equal(confs[0][0], confs[1][0])
    assert np.array_equal(confs[0][1], confs[1][1])


@pytest.mark.parametrize("lanes", [1, 2, 4, 8])
def test_occupancy_order_is_the_grid_order_chain(gpu_lib, lanes):
    """The passes handing out each colour's cells fullest first (schedule 3)
    give the chain of the grid order bit for bit: the cells of one colour are
    independent and their random numbers are keyed by the cell."""
    confs = []
    for schedule in (0, 3):
        s = gpu_lib.HardSphereSystem(rho=0.8, cells=8, dr_max=0.15, seed=42)
        s.set_schedule(schedule, lanes)
        assert s.get_schedule() == (schedule, lanes)
        c = s.sweep_nvt(27)
        confs.append((s.download(), c))
    assert np.array_equal(confs[0][0], confs[1][0])
    assert np.array_equal(confs[0][1], confs[1][1])


def test_occupancy_order_npt_and_switches(gpu_lib):
    """NpT sweeps (the grid is re-derived after a volume move) and switches
    between the grid order and the occupancy order within one chain."""
    finals = []
    for plan in ((0, 0, 0), (3, 3, 3), (3, 0, 3)):
        s = gpu_lib.HardSphereSystem(rho=0.7, cells=6, dr_max=0.15, pressure=6.0, dv_max=0.05, seed=9)
        counts = []
        for sch in plan:
            s.set_schedule(sch, 2)
            counts.append(s.sweep_npt(13).copy())
        finals.append((s.download(), np.concatenate(counts)))
    for conf, c in finals[1:]:
        assert np.array_equal(conf, finals[0][0]) and np.array_equal(c, finals[0][1])
    assert finals[0][1].reshape(3, -1)[:, 4].sum() > 0  # volume moves were accepted: the grid changed


@pytest.mark.parametrize("rho,cells,lt,dr,seed,edge", [
    (0.80, 8, 2, 0.15, 42, 0.0),   # N = 2048 fluid
    (0.50, 7, 2, 0.30, 7, 0.0),    # N = 1372 at the C1 density
    (0.94, 5, 2, 0.06, 3, 0.0),    # dense crystal
    (0.30, 6, 1, 0.40, 11, 1.6),   # 32-slot cells
    (0.85, 4, 2, 0.12, 5, 0.0),    # N = 256, six cells per side
])
def test_one_block_schedule_is_the_pass_barrier_chain(gpu_lib, rho, cells, lt, dr, seed, edge):
    """Every sweep of a call in one block with the system in shared memory
    gives the chain of one launch per pass bit for bit, counters included,
    and leaves observables and later sweeps of the other schedule unchanged."""
    runs = []
    for schedule in (0, 2):
        s = gpu_lib.HardSphereSystem(rho=rho, cells=cells, lattice_type=lt, dr_max=dr, seed=seed,
                                     min_cell_edge=edge)
        s.set_schedule(schedule)
        assert s.get_schedule()[0] == schedule
        c1 = s.sweep_nvt(19)
        c2 = s.sweep_nvt(8)
        s.set_schedule(0)
        c3 = s.sweep_nvt(3)
        runs.append((s.download(), c1, c2, c3, s.compute_rdf_counts(0.02, 2.0, 50)))
    for a, b in zip(runs[0], runs[1]):
        assert np.array_equal(a, b)


def test_one_block_schedule_is_the_default_for_small_systems(gpu_lib):
    small = gpu_lib.HardSphereSystem(rho=0.85, cells=4, dr_max=0.12, seed=1)
    assert small.get_schedule()[0] == 2
    mid = gpu_lib.HardSphereSystem(rho=0.5, cells=10, dr_max=0.3, seed=1)  # fits, but one launch per pass is faster
    assert mid.get_schedule()[0] == 0
    big = gpu_lib.HardSphereSystem(rho=0.85, cells=20, dr_max=0.12, seed=1)
    assert big.get_schedule()[0] == 0
    npt = gpu_lib.HardSphereSystem(rho=0.85, cells=4, dr_max=0.12, dv_max=0.01, pressure=8.0, seed=1)
    assert npt.get_schedule()[0] == 2
    cav = gpu_lib.HardSphereSystem(rho=0.85, cells=4, dr_max=0.12, seed=1, cavity=(0.1, 1.2, 0.0))
    assert cav.get_schedule()[0] == 2


@pytest.mark.parametrize("rho,cells,lt,pcav,maxdr,mindr,seed", [
    (0.80, 10, 1, 0.10, 1.2, 0.0, 31),  # the reference's published cavity case, N = 1000
    (0.50, 4, 2, 0.30, 1.1, 0.6, 32),
    (0.40, 5, 2, 0.05, 0.7, 0.3, 33),
])
def test_one_block_cavity_is_the_pass_barrier_chain(gpu_lib, rho, cells, lt, pcav, maxdr, mindr, seed):
    """Cavity sweeps in one block (the cavity stage inside the launch) give
    the chain of the eight launches plus the cavity kernel bit for bit."""
    runs = []
    for schedule in (0, 2):
        s = gpu_lib.HardSphereSystem(rho=rho, cells=cells, lattice_type=lt, dr_max=0.15, seed=seed,
                                     cavity=(pcav, maxdr, mindr))
        s.set_schedule(schedule)
        c1 = s.sweep_nvt(25)
        c2 = s.sweep_nvt(7)
        runs.append((s.download(), c1, c2))
    for a, b in zip(runs[0], runs[1]):
        assert np.array_equal(a, b)
    assert runs[0][1][0] > 25 * runs[0][0].shape[0]  # the counters include the cavity trials


@pytest.mark.parametrize("rho,cells,P,dv,seed", [
    (0.50, 4, 3.0, 0.01, 21),   # expands toward its pressure
    (0.85, 4, 12.0, 0.004, 22), # dense
    (0.60, 6, 5.0, 0.005, 23),  # N = 864
])
def test_one_block_npt_is_the_pass_barrier_chain(gpu_lib, rho, cells, P, dv, seed):
    """NpT sweeps in one block (the volume move inside the launch) give the
    chain of the eight launches plus the volume-move kernels bit for bit:
    positions, box and counters."""
    runs = []
    for schedule in (0, 2):
        s = gpu_lib.HardSphereSystem(rho=rho, cells=cells, dr_max=0.15, dv_max=dv, pressure=P, seed=seed)
        s.set_schedule(schedule)
        c1 = s.sweep_npt(40)
        c2 = s.sweep_npt(9)
        runs.append((s.download(), np.array(s.get_box()), c1, c2))
    for a, b in zip(runs[0], runs[1]):
        assert np.array_equal(a, b)
    assert runs[0][2][4] > 0  # some volume moves were accepted


def test_dataflow_schedule_npt_matches(gpu_lib):
    confs = []
    for schedule in (0, 1):
        s = gpu_lib.HardSphereSystem(rho=0.6, cells=6, dr_max=0.2, dv_max=0.01, pressure=5.0, seed=7)
        s.set_schedule(schedule)
        s.sweep_npt(24)
        confs.append((s.download(), s.get_box()))
    assert np.array_equal(confs[0][0], confs[1][0])
    assert np.array_equal(confs[0][1], confs[1][1])


def test_dataflow_wait_runs_out_and_reports(gpu_lib):
    """Failure detection without a fault: one region that never publishes its
    progress (a flag nothing sets) makes its neighbours' waits run out, each
    bounded at 1 s; the sweep reports a time-out, and once the region is
    released the context carries on."""
    from hsmc_gb300.system import HsmcError

    s = gpu_lib.HardSphereSystem(rho=0.5, cells=4, dr_max=0.2, seed=3)
    s.set_schedule(1, 2)
    s.sweep_nvt(2)
    assert s._lib.hsmc_gpu_hold_region(s._h, 0) == 0
    with pytest.raises(HsmcError) as err:
        s.sweep_nvt(1)
    assert err.value.code == 7  # HSMC_ERR_TIMEOUT
    assert s._lib.hsmc_gpu_hold_region(s._h, -1) == 0
    s.rng_set_state(s.rng_state())  # rebuild the layout for the next sweep
    c = s.sweep_nvt(2)
    assert c[0] == 2 * s.n


def test_contexts_of_different_sizes_coexist(gpu_lib):
    """The shared-memory allowance of the one-block kernels is the kernel's,
    not a context's: creating a smaller system after a larger one must not
    stop the larger one from sweeping or making cluster moves."""
    big = gpu_lib.HardSphereSystem(rho=0.8, cells=6, dr_max=0.15, seed=1)     # N = 864
    big.sweep_nvt(1)
    big.cluster_moves(1)
    small = gpu_lib.HardSphereSystem(rho=0.5, cells=3, dr_max=0.3, seed=2)    # N = 108
    assert big.get_schedule()[0] == 2 and small.get_schedule()[0] == 2
    small.sweep_nvt(3)
    small.cluster_moves(2)
    c = big.sweep_nvt(5)
    assert c[0] == 5 * big.n
    assert len(big.cluster_moves(2)) == 2
    small.close()
    big.close()


def _host_optimizer(g, opt_sweeps, opt_samples, target, npt=False, vtarget=0.5):
    """opt_nvt / opt_npt (src/optimizer.c:23-148) restated on the host over
    single sweep calls, the arithmetic in Python floats (IEEE double)."""
    per = opt_sweeps // opt_samples

    def sample():
        c = (g.sweep_npt(per) if npt else g.sweep_nvt(per)).astype(np.float64)
        return c[1] / c[0], (c[4] / c[3] if npt else 0.0)

    a1, b1 = sample()
    d1, v1 = g.dr_max, g.dv_max
    g.set_step(d1 * 2 if a1 > target else d1 / 2, (v1 * 2 if b1 > vtarget else v1 / 2) if npt else v1)
    a2, b2 = sample()
    d2, v2 = g.dr_max, g.dv_max
    for _ in range(opt_samples):
        dr = d2 - (a2 - target) * (d2 - d1) / (a2 - a1)
        dv = v2 - (b2 - vtarget) * (v2 - v1) / (b2 - b1) if npt else v2
        if npt:
            if dr > 1.0:
                dr = 1.0
            if dr <= 0.0:
                dr = -dr
                if dr > 1.0:
                    dr = d2 / 2
            if dv <= 0.0:
                dv = -dv
                if dv > 0.1:
                    dv = v2 / 2
        elif dr > 1.0:
            dr = 1.0
        elif dr <= 0.0:
            dr = -dr
            if dr > 1.0:
                dr = d2 / 2
        g.set_step(dr, dv)
        d1, a1, v1, b1 = d2, a2, v2, b2
        a2, b2 = sample()
        d2, v2 = g.dr_max, g.dv_max
    return d2, a2, v2, b2


@pytest.mark.parametrize("rho,cells,dr,P,dv,seed", [
    (0.5, 5, 0.1, 0.0, 0.0, 61),      # N = 500: the one-block schedule
    (0.85, 10, 0.05, 0.0, 0.0, 62),   # N = 4000: graphs of eight launches per sweep
    (0.6, 5, 0.2, 5.0, 0.004, 63),    # NpT: particle and volume steps
])
def test_device_optimizer_is_the_host_loop(gpu_lib, rho, cells, dr, P, dv, seed):
    """hsmc_gpu_optimize (every sample and secant step on the device, one
    host wait) gives the host-side loop's steps, acceptances and chain bit
    for bit."""
    runs = []
    for device in (True, False):
        g = gpu_lib.HardSphereSystem(rho=rho, cells=cells, dr_max=dr, dv_max=dv or 0.001, pressure=P, seed=seed)
        if device:
            res = g.optimize(200, 10, 0.4, 0.5)
        else:
            res = _host_optimizer(g, 200, 10, 0.4, npt=P > 0, vtarget=0.5)
        runs.append((np.array(res), g.download(), np.array(g.get_box())))
        g.close()
    (r_dev, c_dev, b_dev), (r_host, c_host, b_host) = runs
    assert np.array_equal(r_dev, r_host), (r_dev, r_host)
    assert np.array_equal(c_dev, c_host)
    assert np.array_equal(b_dev, b_host)
    assert r_dev[0] != dr  # the step moved
