"""hsmc_gpu_rdf_noalloc: the g(r) counts for callers that cannot let the
library allocate device memory (their device memory belongs to another
memory manager or to a fixed budget, or a first-call cudaMalloc would break a
time budget).  It must give exactly what hsmc_gpu_rdf gives, call after call,
through the C ABI, whether it runs first in a fresh process or after other
tests."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(lib, handle, dr, rmax, nbins):
    out = np.zeros(nbins, dtype=np.uint64)
    fn = lib.hsmc_gpu_rdf_noalloc
    fn.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_int, C.c_void_p]
    fn.restype = C.c_int
    code = fn(handle, dr, rmax, nbins, out.ctypes.data)
    return code, out


def test_noalloc_rdf_matches_allocating_entry_point(gpu_lib):
    from hsmc_gb300 import _native

    lib = _native.load()
    max_bins = 16384  # HSMC_RDF_NOALLOC_MAX_BINS in include/hsmc_gpu.h
    systems = [
        gpu_lib.HardSphereSystem(rho=0.85, cells=6, dr_max=0.12, seed=41),
        gpu_lib.HardSphereSystem(rho=0.50, cells=8, dr_max=0.30, seed=42),
    ]
    for g in systems:
        g.sweep_nvt(40)
    for g, (dr, rmax) in zip(systems, [(0.01, 4.0), (0.005, 5.0)]):
        nbins = int((rmax - 1.0) / dr)
        rmax_used = dr * nbins + 1.0
        want = g.compute_rdf_counts(dr, rmax_used, nbins)
        assert want.sum() > 0
        # two calls in a row: the shared array is cleared each time
        for _ in range(2):
            code, got = _noalloc(lib, g._h, dr, rmax_used, nbins)
            assert code == 0
            assert np.array_equal(got, want)
    # more bins than the fixed array holds: refused, nothing written
    code, got = _noalloc(lib, systems[0]._h, 0.0001, 1.0 + 0.0001 * (max_bins + 1), max_bins + 1)
    assert code == 1 and not got.any()
