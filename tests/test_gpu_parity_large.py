"""Bit-exact decisions at the benchmarked geometries.

The single-precision screen of the move pass decides a pair outside a guard
band of contact whose width grows with the box side (single-precision
coordinates lose absolute precision as |x| grows).  These tests check the
decisions against the oracle (the reference's FP64 check_overlap and
part_move, src/moves.c:27-80, 157-212, 400-431) where the coordinates are
largest:

  * the large NVT fluid: N = 256,000 (40^3 FCC) at rho = 0.85, L = 67.03;
  * the NpT crystal's box: N = 1,048,576 (64^3 FCC) at rho = 1.04, L = 100.27.

Two kinds of evidence, every call through the C ABI:
  * adversarial trial positions: a particle moved toward its nearest
    neighbour until their distance is within a few ulp of contact, or at
    r^2 = 1 +- f * band with f on both sides of 1 (the pairs the single
    precision screen decides alone, just outside the band), drawn mostly
    near the box faces where coordinates are largest and images are added;
    screened exactly as a move-pass trial (k_replay shares its screen);
  * whole traced sweeps of the full systems replayed trial by trial by the
    oracle: decisions and final configurations bit-identical.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

C2 = dict(rho=0.85, cells=40, dr=0.13, melt=300)   # N = 256,000
C5 = dict(rho=1.04, cells=64, dr=0.11, melt=20)    # N = 1,048,576
# C5's box side with a dilute fluid (N = 296,352): at rho = 1.04 the system is
# a crystal in which no insertion point is free
C5_DILUTE = dict(rho=1.04 * (42 / 64) ** 3, cells=42, dr=0.4, melt=50)


def band_of(L):
    return float(np.float32(2.0**-24 * (48.0 * L + 16.0) + 1e-6))


def prepared(oracle_mod, gpu, cfg, seed):
    g = gpu.HardSphereSystem(rho=cfg["rho"], cells=cfg["cells"], dr_max=cfg["dr"], seed=seed)
    g.sweep_nvt(cfg["melt"])
    conf = g.download()
    o = oracle_mod.OracleSim(rho=cfg["rho"], n_cells=cfg["cells"], seed=seed, dr_max=cfg["dr"], neigh_dr=1.05,
                             neigh_max_part=10)
    o.set_config(conf)
    return o, g, conf


def adversarial_points(conf, L, band, rng, count):
    """Trial positions of particle i at a chosen distance from its nearest
    neighbour j: (kind 0) |r| = 1 + k 2^-52, k in [-4, 4]; (kind 1)
    r^2 = 1 + s f band, s = +-1, f in [0.5, 2].  Three quarters of the
    particles are taken with a coordinate within 1.5 of a box face."""
    from scipy.spatial import cKDTree

    x = conf[:, 1:].copy()
    near_face = np.any((x < 1.5) | (x > L - 1.5), axis=1)
    face_ids = np.flatnonzero(near_face)
    n_face = (3 * count) // 4
    ids = np.concatenate([rng.choice(face_ids, n_face), rng.integers(0, len(x), count - n_face)])
    tree = cKDTree(np.mod(x, L), boxsize=L)
    _, nn = tree.query(np.mod(x[ids], L), k=2)
    j = nn[:, 1]
    d = x[ids] - x[j]
    d -= L * np.round(d / L)
    r = np.linalg.norm(d, axis=1)
    kind = rng.integers(0, 2, count)
    k = rng.integers(-4, 5, count)
    f = rng.uniform(0.5, 2.0, count)
    s = np.where(rng.random(count) < 0.5, -1.0, 1.0)
    target = np.where(kind == 0, 1.0 + k * 2.0**-52, np.sqrt(1.0 + s * f * band))
    p = x[j] + d * (target / r)[:, None]
    p = np.where(p >= L, p - L, np.where(p < 0.0, p + L, p))
    return ids.astype(np.int32), p, kind, s * f


@pytest.mark.parametrize("cfg", [C2, C5], ids=["N256k_L67", "N1M_L100"])
def test_adversarial_screen_decisions_at_large_coordinates(oracle_mod, gpu_lib, cfg):
    o, g, conf = prepared(oracle_mod, gpu_lib, cfg, seed=17)
    L = o.box()["lx"]
    assert abs(L - g.get_box()[0]) == 0.0
    band = band_of(L)
    rng = np.random.default_rng(5)
    ids, pos, kind, sf = adversarial_points(conf, L, band, rng, 40000)
    got = g.overlap_replay(ids, pos)
    want = np.array([o.check_overlap_at(int(i), *p) for i, p in zip(ids, pos)], dtype=np.uint8)
    mism = np.flatnonzero(got != want)
    assert mism.size == 0, f"{mism.size} decisions differ, first at {ids[mism[0]]} {pos[mism[0]]}"
    # both outcomes occur where the single-precision screen decides alone,
    # just outside the band on either side, and in the FP64 recheck region
    outside = (kind == 1) & (np.abs(sf) > 1.0)
    assert want[outside & (sf < 0)].mean() > 0.99   # inside contact: overlap
    assert want[outside & (sf > 0)].mean() < 0.9    # beyond contact: mostly free
    assert 0 < want[kind == 0].sum() < (kind == 0).sum()
    g.close()


@pytest.mark.parametrize("cfg,sweeps,schedule", [(C2, 2, None), (C2, 1, 3), (C5, 1, None)],
                         ids=["N256k_L67", "N256k_L67_occupancy_order", "N1M_L100"])
def test_traced_full_size_sweeps_replay_bit_exact(oracle_mod, gpu_lib, cfg, sweeps, schedule):
    """Every trial of whole sweeps of the full system (512,000 trials at
    N = 256,000; 1,048,576 at N = 1,048,576) replayed by the oracle, at each
    size's default schedule (the grid order at N = 256,000, the occupancy
    order at N = 1,048,576) and with the occupancy order at N = 256,000."""
    o, g, _ = prepared(oracle_mod, gpu_lib, cfg, seed=23)
    if schedule is not None:
        g.set_schedule(schedule, 0)
    rec, cnt = g.sweeps_traced(sweeps)
    assert len(rec) == o.n * sweeps and cnt[0] == o.n * sweeps
    rec = rec[np.lexsort((rec[:, 2], rec[:, 1], rec[:, 0]))]
    nc, l32, iw, _ = g.grid_info()
    shifts = rec[:, 8:11].copy().view(np.float32)
    o.reset_counters()
    dec = o.replay_checkerboard(rec[:, 3].astype(np.int32), rec[:, 4:7], rec[:, 1], shifts, nc, l32, iw)
    assert not np.any(dec == 3), "a traced particle was not in its cell"
    mism = np.flatnonzero(dec != rec[:, 7].astype(np.int32))
    assert mism.size == 0, f"{mism.size} of {len(dec)} decisions differ"
    assert np.array_equal(o.get_config(), g.download())
    # the band was exercised: trials with at least one FP64 re-evaluation
    rechecked = int(rec[:, 11].sum())
    assert rechecked > 100, rechecked
    assert cnt[1] == np.sum(dec == 0)
    g.close()


def cavity_band_points(g, conf, L, band, rng, n_random=24_000_000, chunk=4_000_000, max_cav=2000):
    """Insertion points at a band edge of exactly one contact.  A dense
    fluid has few cavities (about one uniform point in 10^5 is free at
    rho = 0.85), so uniform points are screened for free ones first; each
    free point c is then pulled along the ray from its nearest particle j to
    |p - x_j| = t with t = 1 + k 2^-52 (kind 0) or t^2 = 1 + s f band
    (kind 1).  Every other particle stays at least t away from p (triangle
    inequality, since |c - x_k| >= |c - x_j| >= t), so j's band edge
    decides."""
    from scipy.spatial import cKDTree

    free, found = [], 0
    for _ in range(n_random // chunk):
        c = rng.random((chunk, 3)) * L
        free.append(c[g.widom_replay(c) == 0])
        found += len(free[-1])
        if found >= max_cav:
            break
    c = np.concatenate(free)[:max_cav]
    x = np.mod(conf[:, 1:], L)
    _, j = cKDTree(x, boxsize=L).query(np.mod(c, L), k=1)
    d = c - x[j]
    d -= L * np.round(d / L)
    r = np.linalg.norm(d, axis=1)
    keep = r * r > 1.0 + 2.0 * band + 1e-12   # every target t <= r: p lies between x_j and c
    c, j, d, r = c[keep], j[keep], d[keep], r[keep]
    per = 24
    count = len(c) * per
    kind = np.tile(np.repeat([0, 1], per // 2), len(c))
    k = rng.integers(-4, 5, count)
    f = rng.uniform(0.5, 2.0, count)
    s = np.where(rng.random(count) < 0.5, -1.0, 1.0)
    t = np.where(kind == 0, 1.0 + k * 2.0**-52, np.sqrt(1.0 + s * f * band))
    src = np.repeat(np.arange(len(c)), per)
    p = x[j[src]] + d[src] * (t / r[src])[:, None]
    p = np.where(p >= L, p - L, np.where(p < 0.0, p + L, p))
    return len(c), p, kind, s * f


@pytest.mark.parametrize("cfg", [C2, C5_DILUTE], ids=["N256k_L67", "N296k_L100"])
def test_widom_band_edge_insertions_at_large_coordinates(oracle_mod, gpu_lib, cfg):
    """Insertion points at |r| = 1 + k 2^-52 and r^2 = 1 +- f band from one
    particle and no closer to any other: the single-precision decisions
    outside the band and the FP64 ones inside it equal the reference's
    widom_compute_dist test (src/compute_widom_chem_pot.c:130-160).  At
    L = 100.27 the fluid is dilute: the rho = 1.04 crystal has no free
    insertion point, and the band depends on the box side only."""
    o, g, conf = prepared(oracle_mod, gpu_lib, cfg, seed=31)
    L = o.box()["lx"]
    band = band_of(L)
    rng = np.random.default_rng(9)
    n_cav, pos, kind, sf = cavity_band_points(g, conf, L, band, rng)
    print(f"L = {L:.4f}: {n_cav} cavities, {len(pos)} insertion points")
    assert n_cav >= 20, n_cav
    got = g.widom_replay(pos)
    want = o.widom_points(pos)
    mism = np.flatnonzero(got != want)
    assert mism.size == 0, f"{mism.size} of {len(want)} insertion decisions differ"
    outside = (kind == 1) & (np.abs(sf) > 1.0)
    assert want[outside & (sf < 0)].all()           # inside contact: overlap
    assert not want[outside & (sf > 0)].any()       # beyond contact, all others farther: free
    assert 0 < want[kind == 0].sum() < (kind == 0).sum()
    g.close()


@pytest.mark.parametrize("cfg", [C2, C5], ids=["N256k_L67", "N1M_L100"])
def test_scaled_scans_at_band_edges(oracle_mod, gpu_lib, cfg):
    """The thermodynamic-pressure scan and the volume-move scan at scale
    factors placed around the closest pair's contact: sf = (1 + d) / r_min
    with d a few ulps or a fraction of the guard band on either side, where
    the single-precision estimate decides alone or hands over to FP64
    (presst_compute_hist src/compute_press.c:243-273; vol_move
    src/moves.c:104-112)."""
    from scipy.spatial import cKDTree

    o, g, conf = prepared(oracle_mod, gpu_lib, cfg, seed=37)
    L = o.box()["lx"]
    band = band_of(L)
    x = np.mod(conf[:, 1:], L)
    dmin, _ = cKDTree(x, boxsize=L).query(x, k=2)
    rmin = float(dmin[:, 1].min())
    ds = [k * 2.0**-52 for k in (-3, -1, 0, 1, 3)] + [f * band for f in (-3.0, -1.5, -0.6, -0.3, 0.3, 0.6, 1.5, 3.0)]
    sfs = np.array([(1.0 + d) / rmin for d in ds])
    sfs = sfs[sfs < 1.0]
    got = g.compute_presst(sfs)
    want = o.presst_counts_sf(sfs)
    assert np.array_equal(got.astype(np.float64), want), (sfs, got, want)
    for sf in sfs:
        assert g.scan_overlap(float(sf)) == o.scan_overlap(float(sf)), sf
    # every bit set (the scan may stop early), all but one (sf = 1 has no
    # overlap: the scan runs to the end), and a mask of two words
    xi = np.arange(1, 21) * 0.0005
    bench_sf = (1.0 - xi) ** (1.0 / 3.0)
    for sfs in (bench_sf, np.append(bench_sf, 1.0), np.linspace(0.999, 1.0, 70)):
        got = g.compute_presst(sfs)
        assert np.array_equal(got.astype(np.float64), o.presst_counts_sf(sfs)), sfs
    g.close()


def test_pair_counts_at_the_benchmark_box(oracle_mod, gpu_lib):
    """g(r) on [1, 3) in bins of 0.01 and 0.005, and the virial bins, at
    N = 256,000, rho = 0.85: the counts of the single-precision path with
    exact bin thresholds equal an all-pairs count within r < 3 by a periodic
    k-d tree with the reference's bin formula in FP64."""
    from scipy.spatial import cKDTree

    o, g, conf = prepared(oracle_mod, gpu_lib, C2, seed=41)
    L = o.box()["lx"]
    x = conf[:, 1:].copy()
    pairs = cKDTree(np.mod(x, L), boxsize=L).query_pairs(3.0 + 1e-6, output_type="ndarray")
    d = x[pairs[:, 0]] - x[pairs[:, 1]]
    half = L / 2.0
    d = np.where(d > half, d - L, np.where(d < -half, d + L, d))
    r = np.sqrt((d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2])
    for dr, nb in ((0.01, 200), (0.005, 400), (0.01, 5)):
        rmax = 1.0 + dr * nb
        rr = r[r < rmax]
        b = np.trunc((rr - 1.0) / dr).astype(np.int64)
        want = 2 * np.bincount(b, minlength=nb).astype(np.uint64)
        got = g.compute_rdf_counts(dr, rmax, nb) if nb > 5 else g.compute_pressv_counts(dr, rmax, nb)
        assert np.array_equal(got, want)
    g.close()
