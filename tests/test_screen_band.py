"""The guard band of the move pass's single-precision screen, checked on the
CPU at the benchmarked box sides.

The screen (hsmc_gb300/csrc/screen.cuh) compares r^2 computed in single
precision from grid coordinates t = fl(fl(x) - s) (wrapped by +L32), with a
neighbour across a periodic face shifted by +-L32, against 1 +- band, where
band = 2^-24 (48 L + 16) + 1e-6 (make_box, hsmc_gb300/csrc/api.cu).  Pairs
outside the band are decided by single precision alone, so the band must
exceed the largest single-precision error of r^2 near contact.  This test
emulates that arithmetic in numpy float32 (with and without a fused
multiply-add in the squared sum) on pairs placed within two bands of contact
at random positions, most of them next to a box face, and requires the
largest error to stay below a quarter of the band at L = 20, 67.03 (N = 256,000 at
rho = 0.85), 100.27 (N = 1,048,576 at rho = 1.04) and 200.
"""
import numpy as np
import pytest

f32 = np.float32


def band_of(L):
    return float(f32(2.0**-24 * (48.0 * L + 16.0) + 1e-6))


def grid_coord(x, s32, L32, iw32, nc):
    """axis_cell (hsmc_gb300/csrc/common.cuh) in float32: t = x32 - s, wrapped
    once, and its cell index."""
    t = (x.astype(f32) - s32).astype(f32)
    t = np.where(t < 0, (t + L32).astype(f32), t)
    cell = (t * iw32).astype(f32).astype(np.int64)
    over = cell >= nc
    cell = np.where(over, cell - nc, cell)
    t = np.where(over, (t - L32).astype(f32), t)
    return t, cell


def screen_r2(xi, xj, L, nc, shift, fma):
    L32 = f32(L)
    iw32 = f32(nc / L)
    r2 = np.zeros(len(xi), dtype=f32)
    for d in range(3):
        ti, ci = grid_coord(xi[:, d], f32(shift[d]), L32, iw32, nc)
        tj, cj = grid_coord(xj[:, d], f32(shift[d]), L32, iw32, nc)
        # j seen from i's cell: a neighbour (or stencil) cell across the face
        # is shifted by -+L32
        img = np.where(cj - ci > nc // 2, -L32, np.where(ci - cj > nc // 2, L32, f32(0)))
        tj = np.where(img != 0, (tj + img).astype(f32), tj)
        dx = (ti - tj).astype(f32)
        sq = (dx.astype(np.float64) * dx.astype(np.float64))
        if d == 0 or not fma:
            r2 = (r2 + sq.astype(f32)).astype(f32) if d else sq.astype(f32)
        else:
            r2 = (r2.astype(np.float64) + sq).astype(f32)  # fused: one rounding
    return r2.astype(np.float64)


def reference_r2(xi, xj, L):
    d = xi - xj
    d = np.where(d > L / 2, d - L, np.where(d < -L / 2, d + L, d))
    return (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]


@pytest.mark.parametrize("L", [20.0, 67.0307, 100.27, 200.0])
def test_single_precision_error_below_half_band(L):
    rng = np.random.default_rng(int(L * 1000))
    band = band_of(L)
    u = 2.0**-24
    margin = u * (64.0 * L + 64.0)
    nc = 2 * int(np.floor(L / (2.0 * (1.0 + margin))))
    w = L / nc
    worst = 0.0
    for rep in range(8):
        n = 200000
        xi = rng.uniform(0, L, (n, 3))
        face = rng.random(n) < 0.75  # one coordinate within 1.5 of a face
        ax = rng.integers(0, 3, n)
        xi[face, ax[face]] = np.where(rng.random(face.sum()) < 0.5, rng.uniform(0, 1.5, face.sum()),
                                      rng.uniform(L - 1.5, L, face.sum()))
        v = rng.normal(size=(n, 3))
        v /= np.linalg.norm(v, axis=1)[:, None]
        r = np.sqrt(1.0 + rng.uniform(-2, 2, n) * band)
        xj = np.mod(xi + v * r[:, None], L)
        shift = rng.uniform(0, w, 3)
        ref = reference_r2(xi, xj, L)
        for fma in (False, True):
            err = np.abs(screen_r2(xi, xj, L, nc, shift, fma) - ref)
            worst = max(worst, float(err.max()))
    assert worst < 0.25 * band, (L, worst, band)


def approx_r2_f32(xi, xj, L, nc, shift):
    """approx_r2 (hsmc_gb300/csrc/cellview.cuh): the grid-coordinate
    difference shifted by the nearest multiple of L32 (rintf(dx / L32)),
    squares summed in float32; used by Widom insertions and the scaled
    overlap scans."""
    L32 = f32(L)
    iw32 = f32(nc / L)
    r2 = np.zeros(len(xi), dtype=f32)
    for d in range(3):
        ti, _ = grid_coord(xi[:, d], f32(shift[d]), L32, iw32, nc)
        tj, _ = grid_coord(xj[:, d], f32(shift[d]), L32, iw32, nc)
        dx = (ti - tj).astype(f32)
        dx = (dx - (L32 * np.rint((dx / L32).astype(f32))).astype(f32)).astype(f32)
        r2 = (r2 + (dx * dx).astype(f32)).astype(f32)
    return r2.astype(np.float64)


@pytest.mark.parametrize("L", [20.0, 67.0307, 100.27])
def test_minimum_image_form_below_half_band(L):
    """The same bound for the rintf minimum-image form of Widom insertions
    and the scaled scans."""
    rng = np.random.default_rng(int(L * 7))
    band = band_of(L)
    nc = 2 * int(np.floor(L / (2.0 * (1.0 + 2.0**-24 * (64.0 * L + 64.0)))))
    worst = 0.0
    for _ in range(6):
        n = 200000
        xi = rng.uniform(0, L, (n, 3))
        face = rng.random(n) < 0.75
        ax = rng.integers(0, 3, n)
        xi[face, ax[face]] = np.where(rng.random(face.sum()) < 0.5, rng.uniform(0, 1.5, face.sum()),
                                      rng.uniform(L - 1.5, L, face.sum()))
        v = rng.normal(size=(n, 3))
        v /= np.linalg.norm(v, axis=1)[:, None]
        r = np.sqrt(1.0 + rng.uniform(-2, 2, n) * band)
        xj = np.mod(xi + v * r[:, None], L)
        shift = rng.uniform(0, L / nc, 3)
        worst = max(worst, float(np.abs(approx_r2_f32(xi, xj, L, nc, shift) - reference_r2(xi, xj, L)).max()))
    assert worst < 0.25 * band, (L, worst, band)


@pytest.mark.parametrize("L", [20.0, 67.0307, 100.27])
def test_pair_count_error_below_band_times_one_plus_r2(L):
    """The pair counts bin a pair in single precision when its r^2 lies
    farther than band (1 + r^2) from every bin threshold: the error of the
    grid-coordinate r^2 at distances up to 5 stays below a quarter of that."""
    rng = np.random.default_rng(int(L * 13))
    band = band_of(L)
    nc = 2 * int(np.floor(L / (2.0 * (1.0 + 2.0**-24 * (64.0 * L + 64.0)))))
    worst = 0.0
    for _ in range(6):
        n = 200000
        xi = rng.uniform(0, L, (n, 3))
        face = rng.random(n) < 0.75
        ax = rng.integers(0, 3, n)
        xi[face, ax[face]] = np.where(rng.random(face.sum()) < 0.5, rng.uniform(0, 1.5, face.sum()),
                                      rng.uniform(L - 1.5, L, face.sum()))
        v = rng.normal(size=(n, 3))
        v /= np.linalg.norm(v, axis=1)[:, None]
        r = rng.uniform(1.0, 5.05, n)
        xj = np.mod(xi + v * r[:, None], L)
        shift = rng.uniform(0, L / nc, 3)
        ref = reference_r2(xi, xj, L)
        for fma in (False, True):
            err = np.abs(screen_r2(xi, xj, L, nc, shift, fma) - ref) / (1.0 + ref)
            worst = max(worst, float(err.max()))
    assert worst < 0.25 * band, (L, worst, band)
