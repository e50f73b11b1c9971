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
