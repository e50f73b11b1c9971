"""Batched replicas: many independent NVT systems advanced together through
the hsmc_batch_* entry points of include/hsmc_gpu.h."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native
from .system import HsmcError, _check, box_from_lattice, lattice_config


def _bind(lib):
    if getattr(lib, "_batch_bound", False):
        return
    vp, P = C.c_void_p, C.POINTER
    lib.hsmc_batch_create.argtypes = [vp, C.c_int, P(vp)]
    lib.hsmc_batch_destroy.argtypes = [vp]
    lib.hsmc_batch_destroy.restype = None
    lib.hsmc_batch_upload_config.argtypes = [vp, C.c_int, vp, C.c_int]
    lib.hsmc_batch_download_config.argtypes = [vp, C.c_int, vp, C.c_int]
    lib.hsmc_batch_set_steps.argtypes = [vp, vp]
    lib.hsmc_batch_sweeps.argtypes = [vp, C.c_int, vp]
    lib.hsmc_batch_pressv.argtypes = [vp, C.c_double, C.c_double, C.c_int, vp]
    lib.hsmc_batch_last_timing.argtypes = [vp, P(C.c_double)]
    lib._batch_bound = True


class ReplicaBatch:
    """Independent NVT systems on FCC/SC lattice starts, one per entry of
    ``systems`` = [(rho, cells, dr_max, seed), ...]."""

    def __init__(self, systems, lattice_type: int = 2):
        lib = _native.load()
        _bind(lib)
        self._lib = lib
        arr = (_native.HsmcParams * len(systems))()
        self.n = []
        self.box = []
        confs = []
        for k, (rho, cells, dr, seed) in enumerate(systems):
            cells = (cells,) * 3 if np.isscalar(cells) else tuple(cells)
            box, _, _ = box_from_lattice(rho, cells, lattice_type)
            conf = lattice_config(rho, cells, lattice_type)
            p = arr[k]
            p.n_particles = conf.shape[0]
            p.lattice_type = lattice_type
            for d in range(3):
                p.cells[d] = cells[d]
                p.box[d] = box[d]
            p.rho = rho
            p.dr_max = dr
            p.dv_max = 0.001
            p.seed = seed
            self.n.append(conf.shape[0])
            self.box.append(box)
            confs.append(conf)
        h = C.c_void_p()
        _check(lib.hsmc_batch_create(arr, len(systems), C.byref(h)), "hsmc_batch_create")
        self._h = h
        self.reps = len(systems)
        for k, conf in enumerate(confs):
            self.upload(k, conf)

    def close(self):
        if getattr(self, "_h", None):
            self._lib.hsmc_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload(self, k, conf):
        conf = np.ascontiguousarray(conf, dtype=np.float64)
        _check(self._lib.hsmc_batch_upload_config(self._h, k, conf.ctypes.data, self.n[k]), "hsmc_batch_upload_config")

    def download(self, k):
        out = np.empty((self.n[k], 4), dtype=np.float64)
        _check(self._lib.hsmc_batch_download_config(self._h, k, out.ctypes.data, self.n[k]),
               "hsmc_batch_download_config")
        return out

    def set_steps(self, dr):
        dr = np.ascontiguousarray(dr, dtype=np.float64)
        _check(self._lib.hsmc_batch_set_steps(self._h, dr.ctypes.data), "hsmc_batch_set_steps")

    def sweeps(self, n):
        c = np.zeros((self.reps, 6), dtype=np.uint64)
        _check(self._lib.hsmc_batch_sweeps(self._h, n, c.ctypes.data), "hsmc_batch_sweeps")
        return c

    def pressv_counts(self, dr, rmax, nbins):
        out = np.zeros((self.reps, nbins), dtype=np.uint64)
        _check(self._lib.hsmc_batch_pressv(self._h, dr, rmax, nbins, out.ctypes.data), "hsmc_batch_pressv")
        return out

    def last_timing(self):
        t = C.c_double()
        _check(self._lib.hsmc_batch_last_timing(self._h, C.byref(t)), "hsmc_batch_last_timing")
        return t.value


__all__ = ["ReplicaBatch", "HsmcError"]
