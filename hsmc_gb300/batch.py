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
    lib.hsmc_batch_set_schedule.argtypes = [vp, C.c_int, C.c_int, C.c_int]
    lib.hsmc_batch_get_schedule.argtypes = [vp, vp]
    lib.hsmc_batch_autotune.argtypes = [vp, C.c_int, vp]
    lib._batch_bound = True


class ReplicaBatch:
    """Independent NVT systems on FCC/SC lattice starts, one per entry of
    ``systems`` = [(rho, cells, dr_max, seed), ...].  min_cell_edge: a number
    for every replica, or "auto" for min(rho^(-1/3), 1.4), about one sphere
    per device cell (below 1.41 a cell holds at most 14)."""

    def __init__(self, systems, lattice_type: int = 2, min_cell_edge=0.0):
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
            p.min_cell_edge = (min(rho ** (-1.0 / 3.0), 1.4) if min_cell_edge == "auto"
                               else float(min_cell_edge))
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

    def tune_steps(self, dr0, target: float = 0.4, sweeps: int = 20, rounds: int = 8, melt: int = 50):
        """Per-replica secant search of dr_max toward the target acceptance
        (the reference's optimiser, src/optimizer.c:23-64, run on every
        replica at once).  Returns (dr, acceptance) arrays."""
        d1 = np.broadcast_to(np.asarray(dr0, dtype=np.float64), (self.reps,)).copy()

        def acc(d):
            self.set_steps(d)
            c = self.sweeps(sweeps).astype(np.float64)
            return c[:, 1] / c[:, 0]

        self.set_steps(d1)
        self.sweeps(melt)
        a1 = acc(d1)
        d2 = np.where(a1 > target, d1 * 2, d1 / 2)
        a2 = acc(d2)
        for _ in range(rounds):
            moving = a2 != a1
            if not moving.any():
                break
            d = np.where(moving, d2 - (a2 - target) * (d2 - d1) / np.where(moving, a2 - a1, 1.0), d2)
            d = np.minimum(np.maximum(np.abs(d), 1e-3), 1.0)
            d1, a1 = d2, a2
            d2 = d
            a2 = acc(d2)
        self.set_steps(d2)
        self.dr = d2
        return d2, a2

    def set_schedule(self, schedule: int, cluster_blocks: int = 4, tile: int = 2) -> None:
        """0: flat launches per colour pass (CUDA graphs of 8 sweeps); 1: every
        sweep of a call in one persistent launch of thread-block clusters, one
        cluster per bundle of replicas; 2: every sweep of a call in one
        cooperative launch over the whole device per cell capacity, with grid
        barriers between the phases; 3: the flat launches with each pass's
        cells in occupancy order (fullest first).  The same chain."""
        _check(self._lib.hsmc_batch_set_schedule(self._h, schedule, cluster_blocks, tile),
               "hsmc_batch_set_schedule")

    def get_schedule(self):
        out = np.zeros(3, dtype=np.int32)
        _check(self._lib.hsmc_batch_get_schedule(self._h, out.ctypes.data), "hsmc_batch_get_schedule")
        return tuple(int(x) for x in out)

    def autotune(self, sweeps_per_variant: int = 16):
        """Times the four schedules (every cluster size and tile for schedule
        1); keeps the fastest and returns (schedule, cluster_blocks, tile)."""
        out = np.zeros(3, dtype=np.int32)
        _check(self._lib.hsmc_batch_autotune(self._h, sweeps_per_variant, out.ctypes.data), "hsmc_batch_autotune")
        return tuple(int(x) for x in out)

    def last_timing(self):
        t = C.c_double()
        _check(self._lib.hsmc_batch_last_timing(self._h, C.byref(t)), "hsmc_batch_last_timing")
        return t.value


def contact_z(counts, samples: int, n: int, rho: float, dr: float, degree: int = 1):
    """Compressibility factor from the virial contact histogram, as the
    reference's analysis does (compute_pressv, src/compute_press.c:277-307;
    fit in python/hsmc_pressure.py): counts of ordered pairs with r in
    [1 + k dr, 1 + (k+1) dr), normalised to g(r) at the bin centres, a linear
    fit extrapolated to r = 1, Z = 1 + (2 pi / 3) rho g(1).  degree 2 fits a
    parabola instead, to gauge the bias of the straight line."""
    counts = np.asarray(counts, dtype=np.float64)
    nb = counts.shape[-1]
    r = 1.0 + (np.arange(nb) + 0.5) * dr
    shell = 4.0 * np.pi / 3.0 * ((r + dr / 2) ** 3 - (r - dr / 2) ** 3)
    g = counts / (samples * shell * rho * n)
    coef = np.polyfit(r, g, degree)
    return 1.0 + 2.0 * np.pi / 3.0 * rho * float(np.polyval(coef, 1.0))


def carnahan_starling(rho: float) -> float:
    """Z_CS = (1 + eta + eta^2 - eta^3) / (1 - eta)^3 (coeff_vw, src/analytic.c:112)."""
    eta = np.pi * rho / 6.0
    return (1 + eta + eta**2 - eta**3) / (1 - eta) ** 3


__all__ = ["ReplicaBatch", "HsmcError", "contact_z", "carnahan_starling"]
