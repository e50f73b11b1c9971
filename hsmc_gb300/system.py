"""Python mirror of the HSMC reference's local-move run loop on the GB300 engine.

``HardSphereSystem`` follows the reference's flow and names:

* construction = ``sim_box_init`` + ``part_alloc`` + ``part_init`` +
  ``cell_list_init`` (src/sim_info.c:32-156, src/cell_list.c:33-58)
* ``sweep_nvt(n)`` = n calls of ``sweep_nvt`` (src/nvt.c:201-209)
* ``get_moves_counters()`` = the six move counters (src/moves.c:231-241),
  64-bit and cumulative since ``reset_moves_counters()``
* ``compute_rdf_counts``, ``compute_pressv_counts``, ``compute_presst``,
  ``widom_insertion``, ``global_ql`` = the fill steps of the observables
  (src/compute_rdf.c:110-128, src/compute_press.c:123-165 and :243-273,
  src/compute_widom_chem_pot.c:44-71, src/compute_order_parameter.c:82-94)

Every call goes through the C ABI in ``include/hsmc_gpu.h``; errors raise
``HsmcError`` carrying the reference's message for the failure.
"""
from __future__ import annotations

import ctypes as C
import math
import weakref

import numpy as np

from . import _native


class HsmcError(RuntimeError):
    def __init__(self, code: int, where: str):
        lib = _native.load()
        msg = lib.hsmc_gpu_strerror(code).decode()
        super().__init__(f"{where}: {_native.STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


def _check(code: int, where: str) -> None:
    if code != _native.HSMC_OK:
        raise HsmcError(code, where)


def box_from_lattice(rho: float, cells, lattice_type: int = 2):
    """sim_box_init (src/sim_info.c:32-71): per-cell volume part_cell/rho,
    side n * cell_size with cell_size = pow(cell_vol, 1/3)."""
    per_cell = 1 if lattice_type == 1 else 4
    cell_vol = per_cell / rho
    cell_size = math.pow(cell_vol, 1.0 / 3.0)
    nx, ny, nz = cells
    box = (nx * cell_size, ny * cell_size, nz * cell_size)
    vol = (nx * ny * nz) * cell_vol
    return box, vol, cell_size


def cavity_start(conf: np.ndarray, box, maxdr: float, mindr: float) -> np.ndarray:
    """cavity_set_distance (src/cavity_nvt.c:172-186): particle 1 moved onto
    particle 0, shifted along z by (maxdr + mindr) / 2 with one periodic wrap."""
    conf = np.array(conf, dtype=np.float64, copy=True)
    ave = (maxdr + mindr) / 2.0
    conf[1, 1] = conf[0, 1]
    conf[1, 2] = conf[0, 2]
    z = conf[0, 3] + ave
    if z > box[2]:
        z -= box[2]
    elif z < 0.0:
        z += box[2]
    conf[1, 3] = z
    return conf


def lattice_config(rho: float, cells, lattice_type: int = 2) -> np.ndarray:
    """part_init_sc / part_init_fcc (src/sim_info.c:120-156) as double[N][4]
    rows (id, x, y, z) in the reference's order."""
    (_, _, _), _, a = box_from_lattice(rho, cells, lattice_type)
    nx, ny, nz = cells
    if lattice_type == 1:
        if a < 1:
            raise HsmcError(9, "lattice_config")
        sites = [(0.0, 0.0, 0.0)]
    else:
        if a / math.sqrt(2.0) < 1:
            raise HsmcError(9, "lattice_config")
        sites = [(0.0, 0.0, 0.0), (0.5, 0.5, 0.0), (0.5, 0.0, 0.5), (0.0, 0.5, 0.5)]
    ii, jj, kk = np.meshgrid(np.arange(nx, dtype=np.float64), np.arange(ny, dtype=np.float64),
                             np.arange(nz, dtype=np.float64), indexing="ij")
    blocks = []
    for (sx, sy, sz) in sites:
        blocks.append(np.stack([(ii + sx) * a if sx else ii * a, (jj + sy) * a if sy else jj * a,
                                (kk + sz) * a if sz else kk * a], axis=-1).reshape(-1, 3))
    xyz = np.stack(blocks, axis=1).reshape(-1, 3)
    conf = np.empty((xyz.shape[0], 4), dtype=np.float64)
    conf[:, 0] = np.arange(xyz.shape[0], dtype=np.float64)
    conf[:, 1:] = xyz
    return conf


class HardSphereSystem:
    """One periodic hard-sphere system on the GPU."""

    def __init__(self, rho: float, cells, lattice_type: int = 2, dr_max: float = 0.05, dv_max: float = 0.001,
                 pressure: float = 0.0, seed: int = 0, conf: np.ndarray | None = None, cell_capacity: int = 0,
                 box=None, lanes_per_cell: int = 0, min_cell_edge: float = 0.0, cavity=None):
        lib = _native.load()
        self._lib = lib
        if np.isscalar(cells):
            cells = (int(cells),) * 3
        self.cells = tuple(int(c) for c in cells)
        self.lattice_type = lattice_type
        self.rho = float(rho)
        if box is None:
            box, vol, _ = box_from_lattice(rho, self.cells, lattice_type)
        else:
            vol = box[0] * box[1] * box[2]
        self.box = tuple(float(b) for b in box)
        self.vol = vol
        if conf is None:
            conf = lattice_config(rho, self.cells, lattice_type)
            if cavity is not None:
                conf = cavity_start(conf, self.box, cavity[1], cavity[2])
        conf = np.ascontiguousarray(conf, dtype=np.float64)
        self.n = conf.shape[0]
        p = _native.HsmcParams()
        p.n_particles = self.n
        p.lattice_type = lattice_type
        for d in range(3):
            p.cells[d] = self.cells[d]
            p.box[d] = self.box[d]
        p.rho = self.rho
        p.dr_max = dr_max
        p.dv_max = dv_max
        p.pressure = pressure
        p.seed = seed
        p.cell_capacity = cell_capacity
        p.lanes_per_cell = lanes_per_cell
        p.min_cell_edge = min_cell_edge
        if cavity is not None:  # (p_cav, maxdr, mindr), the keyword "cavity" of the reference
            p.cavity_pcav, p.cavity_maxdr, p.cavity_mindr = (float(v) for v in cavity)
        self.cavity = cavity
        h = C.c_void_p()
        _check(lib.hsmc_gpu_create(C.byref(p), C.byref(h)), "hsmc_gpu_create")
        self._h = h
        self._dependents = []  # objects that use this context's stream (LearnedWidom), closed first
        self.dr_max = dr_max
        self.dv_max = dv_max
        self._counters = np.zeros(6, dtype=np.uint64)
        self.upload(conf)

    # -- lifecycle -----------------------------------------------------------
    def close(self) -> None:
        h = getattr(self, "_h", None)
        if h:
            for ref in getattr(self, "_dependents", ()):
                dep = ref()
                if dep is not None:
                    dep.close()
            self._lib.hsmc_gpu_destroy(h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- configuration -------------------------------------------------------
    def upload(self, conf: np.ndarray) -> None:
        conf = np.ascontiguousarray(conf, dtype=np.float64)
        if conf.shape != (self.n, 4):
            raise ValueError("configuration must be double[N][4]")
        _check(self._lib.hsmc_gpu_upload_config(self._h, conf.ctypes.data, self.n), "hsmc_gpu_upload_config")

    def download(self, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.empty((self.n, 4), dtype=np.float64)
        _check(self._lib.hsmc_gpu_download_config(self._h, out.ctypes.data, self.n), "hsmc_gpu_download_config")
        return out

    part_config_get = download

    def set_step(self, dr_max: float, dv_max: float | None = None) -> None:
        self.dr_max = dr_max
        if dv_max is not None:
            self.dv_max = dv_max
        _check(self._lib.hsmc_gpu_set_step(self._h, self.dr_max, self.dv_max), "hsmc_gpu_set_step")

    # -- moves ---------------------------------------------------------------
    def sweep_nvt(self, n_sweeps: int = 1) -> np.ndarray:
        c = np.zeros(6, dtype=np.uint64)
        _check(self._lib.hsmc_gpu_sweeps(self._h, n_sweeps, c.ctypes.data), "hsmc_gpu_sweeps")
        self._counters += c
        return c

    def sweep_npt(self, n_sweeps: int = 1) -> np.ndarray:
        c = np.zeros(6, dtype=np.uint64)
        _check(self._lib.hsmc_gpu_npt_sweeps(self._h, n_sweeps, c.ctypes.data), "hsmc_gpu_npt_sweeps")
        self._counters += c
        return c

    def sweeps_traced(self, n_sweeps: int, capacity: int | None = None):
        if capacity is None:
            capacity = self.n * n_sweeps + 16
        rec = np.zeros((capacity, 12), dtype=np.uint32)
        got = C.c_int64(0)
        c = np.zeros(6, dtype=np.uint64)
        _check(self._lib.hsmc_gpu_sweeps_traced(self._h, n_sweeps, rec.ctypes.data, capacity, C.byref(got),
                                                c.ctypes.data), "hsmc_gpu_sweeps_traced")
        self._counters += c
        return rec[: got.value].copy(), c

    def cluster_moves(self, n_moves: int, drawn: bool = False):
        """n_moves geometric cluster moves (cluster_sweep_nvt,
        src/cluster_nvt.c:221-228); returns the cluster sizes, and with
        drawn=True also each move's (pivot x, y, z, axis, seed particle)."""
        sizes = np.zeros(n_moves, dtype=np.int64)
        d = np.zeros((n_moves, 5), dtype=np.float64) if drawn else None
        _check(self._lib.hsmc_gpu_cluster_moves(self._h, n_moves, sizes.ctypes.data,
                                                d.ctypes.data if d is not None else None),
               "hsmc_gpu_cluster_moves")
        return (sizes, d) if drawn else sizes

    def cluster_move_at(self, pivot, axis: int, seed_particle: int) -> int:
        """One cluster move from a given pivot, axis (0, 1, 2) and seed
        particle; returns its size."""
        piv = np.ascontiguousarray(pivot, dtype=np.float64)
        size = C.c_int64(0)
        _check(self._lib.hsmc_gpu_cluster_move_at(self._h, piv.ctypes.data, int(axis), int(seed_particle),
                                                  C.byref(size)), "hsmc_gpu_cluster_move_at")
        return int(size.value)

    def cavity_psi(self, x) -> np.ndarray:
        """The umbrella potential psi(x) = ln y_GH(x) of a cavity run, as the
        device evaluates it (cavity_interaction, src/moves.c:434-440)."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        out = np.zeros_like(x)
        _check(self._lib.hsmc_gpu_cavity_psi(self._h, x.ctypes.data, x.size, out.ctypes.data),
               "hsmc_gpu_cavity_psi")
        return out

    def cavity_trace(self, capacity: int) -> None:
        _check(self._lib.hsmc_gpu_cavity_trace(self._h, capacity), "hsmc_gpu_cavity_trace")
        self._cav_cap = capacity

    def cavity_trace_read(self) -> np.ndarray:
        cap = max(getattr(self, "_cav_cap", 0), 1)
        rec = np.zeros((cap, 8), dtype=np.uint32)
        got = C.c_int64(0)
        _check(self._lib.hsmc_gpu_cavity_trace_read(self._h, rec.ctypes.data, cap, C.byref(got)),
               "hsmc_gpu_cavity_trace_read")
        return rec[: got.value].copy()

    def cavity_distance(self) -> float:
        """compute_dist(0, 1) of the reference (src/moves.c:400-431)."""
        c = self.download()
        d = c[0, 1:] - c[1, 1:]
        L = np.array(self.box)
        d = np.where(d > L / 2, d - L, np.where(d < -L / 2, d + L, d))
        return float(np.sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]))

    def get_moves_counters(self) -> np.ndarray:
        return self._counters.copy()

    def reset_moves_counters(self) -> None:
        self._counters[:] = 0

    def grid_info(self):
        nc = np.zeros(3, dtype=np.int32)
        l32 = np.zeros(3, dtype=np.float32)
        iw = np.zeros(3, dtype=np.float32)
        cap = C.c_int()
        _check(self._lib.hsmc_gpu_grid_info(self._h, nc.ctypes.data, l32.ctypes.data, iw.ctypes.data,
                                            C.byref(cap)), "hsmc_gpu_grid_info")
        return nc, l32, iw, cap.value

    def get_box(self):
        out = np.zeros(5, dtype=np.float64)
        _check(self._lib.hsmc_gpu_get_box(self._h, out.ctypes.data), "hsmc_gpu_get_box")
        return out

    # -- observables -----------------------------------------------------------
    def compute_rdf_counts(self, dr: float, rmax: float, nbins: int) -> np.ndarray:
        out = np.zeros(nbins, dtype=np.uint64)
        _check(self._lib.hsmc_gpu_rdf(self._h, dr, rmax, nbins, out.ctypes.data), "hsmc_gpu_rdf")
        return out

    def compute_pressv_counts(self, dr: float, rmax: float, nbins: int) -> np.ndarray:
        out = np.zeros(nbins, dtype=np.uint64)
        _check(self._lib.hsmc_gpu_pressv(self._h, dr, rmax, nbins, out.ctypes.data), "hsmc_gpu_pressv")
        return out

    def compute_presst(self, sf) -> np.ndarray:
        sf = np.ascontiguousarray(sf, dtype=np.float64)
        out = np.zeros(sf.size, dtype=np.uint64)
        _check(self._lib.hsmc_gpu_presst(self._h, sf.ctypes.data, sf.size, out.ctypes.data), "hsmc_gpu_presst")
        return out

    def scan_overlap(self, sf: float) -> int:
        ov = C.c_int()
        _check(self._lib.hsmc_gpu_scan_overlap(self._h, sf, C.byref(ov)), "hsmc_gpu_scan_overlap")
        return ov.value

    def widom_insertion(self, n: int) -> int:
        acc = C.c_uint64()
        _check(self._lib.hsmc_gpu_widom(self._h, n, C.byref(acc)), "hsmc_gpu_widom")
        return int(acc.value)

    def global_ql(self, l: int, rc: float, per_particle: bool = False):
        mean = C.c_double()
        per = np.zeros(self.n, dtype=np.float64) if per_particle else None
        _check(self._lib.hsmc_gpu_ql(self._h, l, rc, C.byref(mean), per.ctypes.data if per is not None else None),
               "hsmc_gpu_ql")
        return (mean.value, per) if per_particle else mean.value

    # -- replay ------------------------------------------------------------------
    def overlap_replay(self, ids, pos) -> np.ndarray:
        ids = np.ascontiguousarray(ids, dtype=np.int32)
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        out = np.zeros(ids.size, dtype=np.uint8)
        _check(self._lib.hsmc_gpu_overlap_replay(self._h, ids.ctypes.data, pos.ctypes.data, ids.size,
                                                 out.ctypes.data), "hsmc_gpu_overlap_replay")
        return out

    def widom_replay(self, pos) -> np.ndarray:
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        out = np.zeros(pos.shape[0], dtype=np.uint8)
        _check(self._lib.hsmc_gpu_widom_replay(self._h, pos.ctypes.data, pos.shape[0], out.ctypes.data),
               "hsmc_gpu_widom_replay")
        return out

    # -- rng / timing ----------------------------------------------------------
    def rng_state(self) -> np.ndarray:
        out = np.zeros(4, dtype=np.uint64)
        _check(self._lib.hsmc_gpu_rng_state(self._h, out.ctypes.data), "hsmc_gpu_rng_state")
        return out

    def rng_set_state(self, st) -> None:
        st = np.ascontiguousarray(st, dtype=np.uint64)
        _check(self._lib.hsmc_gpu_rng_set_state(self._h, st.ctypes.data), "hsmc_gpu_rng_set_state")

    def optimize(self, opt_sweeps: int, opt_samples: int, part_target: float = 0.4, vol_target: float = 0.5):
        """The reference's optimiser (opt_nvt / opt_npt, src/optimizer.c:23-148)
        in one device call; returns (dr_max, last acceptance, dv_max, last
        volume acceptance) and keeps the new steps."""
        out = np.zeros(4, dtype=np.float64)
        _check(self._lib.hsmc_gpu_optimize(self._h, opt_sweeps, opt_samples, part_target, vol_target,
                                           out.ctypes.data), "hsmc_gpu_optimize")
        self.dr_max, self.dv_max = float(out[0]), float(out[2])
        return float(out[0]), float(out[1]), float(out[2]), float(out[3])

    def autotune(self, sweeps_per_variant: int = 5) -> int:
        lanes = C.c_int()
        _check(self._lib.hsmc_gpu_autotune(self._h, sweeps_per_variant, C.byref(lanes)), "hsmc_gpu_autotune")
        return lanes.value

    def set_schedule(self, schedule: int, lanes_per_cell: int = 0) -> None:
        """0: one launch per colour pass; 1: dataflow sweep; 2: every sweep of
        a call in one block (small NVT systems); 3: one launch per colour
        pass with the cells in occupancy order.  The same chain."""
        _check(self._lib.hsmc_gpu_set_schedule(self._h, schedule, lanes_per_cell), "hsmc_gpu_set_schedule")

    def get_schedule(self):
        sch, lanes = C.c_int(), C.c_int()
        _check(self._lib.hsmc_gpu_get_schedule(self._h, C.byref(sch), C.byref(lanes)), "hsmc_gpu_get_schedule")
        return sch.value, lanes.value

    def set_profiling(self, on: bool) -> None:
        _check(self._lib.hsmc_gpu_set_profiling(self._h, 1 if on else 0), "hsmc_gpu_set_profiling")

    def last_timing(self):
        t = C.c_double()
        m = C.c_double()
        k = C.c_int()
        _check(self._lib.hsmc_gpu_last_timing(self._h, C.byref(t), C.byref(m), C.byref(k)), "hsmc_gpu_last_timing")
        return t.value, m.value, k.value


def compress_to(system: HardSphereSystem, rho_target: float, sweeps: int = 20, dr_max: float | None = None,
                max_rounds: int = 5000) -> HardSphereSystem:
    """Prepare a dense fluid (a preparation step of this package; the
    reference starts only from lattices): alternate `sweeps` NVT sweeps with
    an affine compression of the box by 90% of the largest scale factor that
    the reference's FP64 scaled-overlap scan (vol_move, src/moves.c:104-112)
    accepts, never past rho_target, until rho_target is reached exactly.
    Each compression uploads the scaled configuration into a new context;
    the old one is closed.  Returns the system at rho_target."""
    s = system
    for _ in range(max_rounds):
        if s.rho >= rho_target:
            return s
        s.sweep_nvt(sweeps)
        sf_t = (s.rho / rho_target) ** (1.0 / 3.0)
        if not s.scan_overlap(sf_t):
            sf = sf_t
        else:
            lo, hi = sf_t, 1.0  # overlap at lo, none at hi
            for _ in range(20):
                mid = 0.5 * (lo + hi)
                if s.scan_overlap(mid):
                    lo = mid
                else:
                    hi = mid
            sf = 1.0 - 0.9 * (1.0 - hi)
        conf = s.download()
        conf[:, 1:] *= sf
        box = tuple(b * sf for b in s.box)
        rho = rho_target if sf == sf_t else s.n / (box[0] * box[1] * box[2])
        step = dr_max if dr_max is not None else s.dr_max
        new = HardSphereSystem(rho=rho, cells=s.cells, lattice_type=s.lattice_type, dr_max=step, dv_max=s.dv_max,
                               seed=int(s.rng_state()[0]) + 1, conf=conf, box=box)
        s.close()
        s = new
    raise HsmcError(1, "compress_to: target density not reached")
