"""The C-ABI library loads without a GPU and exports every entry point the
public header declares; host-side helpers agree with the reference."""
import ctypes as C
import os

import numpy as np
import pytest


def test_library_exports_every_declared_symbol(gpu_lib):
    from hsmc_gb300 import _native

    names = _native.declared_symbols()
    assert len(names) >= 20
    lib = C.CDLL(_native.LIB_PATH)
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_strerror_is_total(gpu_lib):
    lib = gpu_lib._native.load()
    for code in range(0, 12):
        assert lib.hsmc_gpu_strerror(code)


def test_create_without_gpu_fails_cleanly(gpu_lib):
    """Without a device the create call must report an error, never fall back."""
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(gpu_lib.HsmcError) as ei:
        gpu_lib.HardSphereSystem(rho=0.5, cells=5)
    assert ei.value.code in (2, 3)


@pytest.mark.parametrize("rho,n,lt", [(0.5, 5, 2), (0.85, 6, 2), (0.3, 4, 1), (0.94, 3, 2)])
def test_lattice_matches_reference(oracle_mod, gpu_lib, rho, n, lt):
    conf = gpu_lib.lattice_config(rho, (n, n, n), lt)
    o = oracle_mod.OracleSim(rho=rho, n_cells=n, lattice_type=lt, neigh_dr=1.0)
    assert np.array_equal(conf, o.get_config())
    box, vol, _ = gpu_lib.box_from_lattice(rho, (n, n, n), lt)
    b = o.box()
    assert box == (b["lx"], b["ly"], b["lz"]) and vol == b["vol"]


def test_cavity_range_thresholds_are_exact(gpu_lib):
    """The cavity stage tests the distance range [mindr, maxdr] on r2 against
    two host-computed thresholds; sqrt(r2) >= c must hold exactly when
    r2 >= r2_at_least(c), and sqrt(r2) <= c exactly when r2 <= r2_at_most(c),
    for every double near c * c (sqrt is correctly rounded in numpy, glibc
    and CUDA alike)."""
    lib = gpu_lib._native.load()
    lo_f, hi_f = lib.hsmc_cavity_r2_at_least, lib.hsmc_cavity_r2_at_most
    lo_f.restype = hi_f.restype = C.c_double
    lo_f.argtypes = hi_f.argtypes = [C.c_double]
    rng = np.random.default_rng(11)
    cs = np.concatenate([[0.0, 0.3, 0.6, 0.7, 1.0, 1.1, 1.2, 1.5], rng.uniform(0.0, 3.0, 2000)])
    steps = np.arange(-12, 13)
    for c in cs:
        lo, hi = lo_f(float(c)), hi_f(float(c))
        x = np.float64(c) * np.float64(c)
        near = np.array([x] * len(steps))
        for i, k in enumerate(steps):
            for _ in range(abs(int(k))):
                near[i] = np.nextafter(near[i], np.inf if k > 0 else 0.0)
        r = np.sqrt(near)
        assert np.array_equal(r >= c, near >= lo), c
        assert np.array_equal(r <= c, near <= hi), c
    assert lo_f(0.0) == 0.0 and hi_f(float("inf")) == float("inf")


@pytest.mark.parametrize("dr,nbins", [(0.01, 400), (0.005, 800), (0.01, 5), (0.02, 200), (0.0123, 17)])
def test_pair_bin_thresholds_are_the_reference_bins(gpu_lib, dr, nbins):
    """hsmc_pair_thresholds: for every k the threshold's bin
    (int)((sqrt(r2) - 1) / dr) reaches k and the double just below does not;
    the rmax threshold likewise; and binning by thresholds equals the
    reference's formula on random and boundary r2 (IEEE double here as on
    the device)."""
    lib = gpu_lib._native.load()
    fn = lib.hsmc_pair_thresholds
    fn.argtypes = [C.c_double, C.c_double, C.c_int, C.c_void_p]
    rmax = 1.0 + dr * nbins
    thr = np.zeros(nbins + 2)
    assert fn(dr, rmax, nbins, thr.ctypes.data) == 0

    def binf(r2):
        return np.trunc((np.sqrt(r2) - 1.0) / dr)

    assert thr[0] == 1.0 and np.all(np.diff(thr[:nbins + 1]) > 0)
    below = np.nextafter(thr, 0.0)
    ks = np.arange(1, nbins + 1)
    assert np.all(binf(thr[1:nbins + 1]) >= ks) and np.all(binf(below[1:nbins + 1]) < ks)
    assert np.sqrt(thr[nbins + 1]) >= rmax and np.sqrt(below[nbins + 1]) < rmax
    rng = np.random.default_rng(nbins)
    r2 = np.concatenate([rng.uniform(1.0, thr[nbins], 200000), thr[1:nbins], below[1:nbins],
                         np.nextafter(thr[1:nbins], 10.0)])
    r2 = r2[(r2 >= 1.0) & (r2 < thr[nbins])]
    by_thr = np.searchsorted(thr[:nbins], r2, side="right") - 1
    assert np.array_equal(by_thr, binf(r2).astype(int))
