"""hsmc_gpu_rdf_noalloc: the g(r) counts for callers that cannot let the
library allocate device memory (their device memory belongs to another
memory manager or to a fixed budget, or a first-call cudaMalloc would break a
time budget).  It must give exactly what hsmc_gpu_rdf gives, call after call,
through the C ABI.  Two cases: in this process after the other tests, and in
a fresh process where it is the first counting call the library sees (so its
first call does the device-address lookup with no earlier hsmc_gpu_rdf)."""
import ctypes as C
import os
import subprocess
import sys
import textwrap

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


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
    for g in systems:
        g.close()


_FRESH = textwrap.dedent("""
    import ctypes as C, sys
    import numpy as np
    sys.path.insert(0, {root!r})
    import hsmc_gb300
    from hsmc_gb300 import _native
    lib = _native.load()
    fn = lib.hsmc_gpu_rdf_noalloc
    fn.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_int, C.c_void_p]
    fn.restype = C.c_int
    g = hsmc_gb300.HardSphereSystem(rho=0.7, cells=7, dr_max=0.2, seed=7)
    g.sweep_nvt(30)
    dr, nbins = 0.01, 300
    rmax = 1.0 + dr * nbins
    got = []
    for _ in range(2):  # the first counting call of this process, then a second one
        out = np.zeros(nbins, dtype=np.uint64)
        assert fn(g._h, dr, rmax, nbins, out.ctypes.data) == 0
        got.append(out)
    want = g.compute_rdf_counts(dr, rmax, nbins)
    assert want.sum() > 0
    assert all(np.array_equal(x, want) for x in got)
    g.close()
    print("FRESH_OK", int(want.sum()))
""")


def test_noalloc_rdf_first_call_in_fresh_process(gpu_lib):
    r = subprocess.run([sys.executable, "-c", _FRESH.format(root=ROOT)], capture_output=True, text=True,
                       timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "FRESH_OK" in r.stdout
