"""Oracle test infrastructure (not product code).

ctypes front-ends with one interface for the two CPU oracles:

* ``OracleSim`` -- the project's C restatement of the reference algorithm
  (``oracle/hsmc_oracle.c`` -> ``oracle/liboracle.so``).  It is built on every
  machine by ``build()`` and is the checker the GPU parity tests use.
* ``RefSim`` -- the HSMC reference's own sources compiled unmodified with a GSL
  stand-in (``oracle/Makefile`` -> ``oracle/_ref/libhsmc_ref.so``).  It only
  exists where the reference sources are present and is used to pin the
  restatement and to generate the golden fixtures.

Only tests, the smoke check and the benchmark's CPU-baseline leg import this
module.  The GPU product never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libhsmc_ref.so")
REF_EXE = os.path.join(HERE, "_ref", "hsmc_ref")
# The reference checkout: $HSMC_REFERENCE, else a directory named
# "reference" beside this repository.  Only the oracle's build and the
# fixture scripts read it; nothing that runs without it needs it.
REF_ROOT = os.environ.get("HSMC_REFERENCE") or os.path.join(os.path.dirname(HERE), "..", "reference")
REF_SRC = os.path.normpath(os.path.join(REF_ROOT, "src"))

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_u32p = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")
_u64p = np.ctypeslib.ndpointer(dtype=np.uint64, flags="C_CONTIGUOUS")
_f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")


def build_oracle(with_reference: bool | None = None) -> None:
    """Compile the restatement (always) and the reference build (when its
    sources are present, or when asked)."""
    targets = ["oracle"]
    if with_reference is None:
        with_reference = os.path.isdir(REF_SRC)
    if with_reference:
        targets.append("ref")
    subprocess.run(["make", "-s", "-C", HERE, "REF_SRC=" + REF_SRC] + targets, check=True)


def reference_available() -> bool:
    return os.path.exists(REF_SO)


def fcc_box(rho: float, n: int, lattice_type: int = 2) -> float:
    """Box side of the reference's lattice start (src/sim_info.c:32-71)."""
    per_cell = 1 if lattice_type == 1 else 4
    return n * (per_cell / rho) ** (1.0 / 3.0)


def write_input(path: str, **kw) -> None:
    """Write a keyword input file in the reference's format
    (src/read_input.c:138-441).  Values may be scalars or tuples."""
    lines = []
    for key, val in kw.items():
        if isinstance(val, (tuple, list)):
            lines.append(key + " " + " ".join(str(v) for v in val))
        else:
            lines.append(f"{key} {val}")
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + "\n")


def raw_to_unit(raw):
    """The reference's uniform: draw / (2^32 - 1) (src/rng.c:29-31)."""
    return np.asarray(raw, dtype=np.float64) / 4294967295.0


class _SimBase:
    n: int

    def get_config(self) -> np.ndarray:
        out = np.zeros((self.n, 4), dtype=np.float64)
        self._lib_get_config(out)
        return out

    def box(self) -> dict:
        out = np.zeros(9, dtype=np.float64)
        self._lib_box(out)
        keys = ["lx", "ly", "lz", "vol", "rho", "cell_size", "n_cells_x", "dr_max", "dv_max"]
        return dict(zip(keys, out.tolist()))

    def counters(self) -> np.ndarray:
        return self._counters()

    def replay_moves(self, ids, raw) -> np.ndarray:
        ids = np.ascontiguousarray(ids, dtype=np.int32)
        raw = np.ascontiguousarray(raw, dtype=np.uint32).reshape(-1)
        assert raw.size == 3 * ids.size
        acc = np.zeros(ids.size, dtype=np.int32)
        self._lib_replay(ids.size, ids, raw, acc)
        return acc

    def replay_moves_offsets(self, ids, raw) -> np.ndarray:
        """part_move with the device's exact step factor (2r - 2^32 + 1) * 2^-33."""
        ids = np.ascontiguousarray(ids, dtype=np.int32)
        raw = np.ascontiguousarray(raw, dtype=np.uint32).reshape(-1)
        assert raw.size == 3 * ids.size
        acc = np.zeros(ids.size, dtype=np.int32)
        self._lib_replay_offsets(ids.size, ids, raw, acc)
        return acc

    def rdf_counts(self, dr: float, rmax: float, max_bins: int = 100000):
        out = np.zeros(max_bins, dtype=np.float64)
        used = C.c_double()
        nb = self._lib_rdf(dr, rmax, out, max_bins, C.byref(used))
        if nb < 0:
            raise ValueError("too many bins")
        return out[:nb].copy(), used.value

    def pressv_counts(self, dr: float, max_bins: int = 10000):
        out = np.zeros(max_bins, dtype=np.float64)
        used = C.c_double()
        nb = self._lib_pressv(dr, out, max_bins, C.byref(used))
        if nb < 0:
            raise ValueError("too many bins")
        return out[:nb].copy(), used.value

    def presst_counts(self, dxi: float, xi_max: float, max_n: int = 10000):
        out = np.zeros(max_n, dtype=np.float64)
        nb = self._lib_presst(dxi, xi_max, out, max_n)
        if nb < 0:
            raise ValueError("too many steps")
        return out[:nb].copy()

    def widom(self, raw) -> int:
        raw = np.ascontiguousarray(raw, dtype=np.uint32).reshape(-1)
        return int(self._lib_widom(raw.size // 3, raw))

    def ql(self, l: int, rc: float):
        per = np.zeros(self.n, dtype=np.float64)
        used = C.c_double()
        mean = self._lib_ql(l, rc, per, C.byref(used))
        return mean, per, used.value


class OracleSim(_SimBase):
    """The project's C restatement (``hsmc_oracle.c``)."""

    _lib = None

    @classmethod
    def lib(cls):
        if cls._lib is None:
            if not os.path.exists(ORACLE_SO):
                build_oracle(with_reference=False)
            L = C.CDLL(ORACLE_SO)
            L.hso_create.restype = C.c_void_p
            L.hso_create.argtypes = [C.c_double, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int,
                                     C.c_double, C.c_double, C.c_double, C.c_ulong, C.POINTER(C.c_int)]
            L.hso_destroy.argtypes = [C.c_void_p]
            L.hso_n.argtypes = [C.c_void_p]
            L.hso_box.argtypes = [C.c_void_p, _dp]
            L.hso_get_config.argtypes = [C.c_void_p, _dp]
            L.hso_set_config.argtypes = [C.c_void_p, _dp]
            L.hso_reset_lattice.argtypes = [C.c_void_p]
            L.hso_set_steps.argtypes = [C.c_void_p, C.c_double, C.c_double]
            L.hso_last_error.argtypes = [C.c_void_p]
            L.hso_sweeps_nvt.argtypes = [C.c_void_p, C.c_int]
            L.hso_sweeps_npt.argtypes = [C.c_void_p, C.c_int]
            L.hso_counters.argtypes = [C.c_void_p, _u64p]
            L.hso_reset_counters.argtypes = [C.c_void_p]
            L.hso_replay_moves.argtypes = [C.c_void_p, C.c_int, _i32p, _u32p, _i32p]
            L.hso_replay_moves_offsets.argtypes = [C.c_void_p, C.c_int, _i32p, _u32p, _i32p]
            L.hso_widom_points.argtypes = [C.c_void_p, C.c_int, _dp, _u8p]
            L.hso_check_overlap_at.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_double]
            L.hso_scan_overlap.argtypes = [C.c_void_p, C.c_double]
            L.hso_vol_move_replay.argtypes = [C.c_void_p, _u32p, C.c_int]
            L.hso_rdf_counts.argtypes = [C.c_void_p, C.c_double, C.c_double, _dp, C.c_int, C.POINTER(C.c_double)]
            L.hso_pressv_counts.argtypes = [C.c_void_p, C.c_double, _dp, C.c_int, C.POINTER(C.c_double)]
            L.hso_presst_counts.argtypes = [C.c_void_p, C.c_double, C.c_double, _dp, C.c_int]
            L.hso_presst_counts_sf.argtypes = [C.c_void_p, _dp, C.c_int, _dp]
            L.hso_widom.argtypes = [C.c_void_p, C.c_int, _u32p]
            L.hso_widom_decisions.argtypes = [C.c_void_p, C.c_int, _u32p, _u8p]
            L.hso_widom_rng.argtypes = [C.c_void_p, C.c_int]
            L.hso_ql.restype = C.c_double
            L.hso_ql.argtypes = [C.c_void_p, C.c_int, C.c_double, _dp, C.POINTER(C.c_double)]
            L.hso_opt_nvt.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_double, C.POINTER(C.c_double),
                                      C.POINTER(C.c_double)]
            L.hso_rng_raw.argtypes = [C.c_ulong, C.c_int, _u32p]
            L.hso_rng_uniform_int.argtypes = [C.c_ulong, C.c_ulong, C.c_int, _i32p]
            L.hso_brute_overlap.argtypes = [_dp, C.c_int, C.c_double, C.c_double, C.c_double, C.c_int,
                                            C.c_double, C.c_double, C.c_double]
            L.hso_brute_pair_hist.argtypes = [_dp, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                                              C.c_double, C.c_int, _u64p]
            L.hso_replay_checkerboard.argtypes = [C.c_void_p, C.c_int, _i32p, _u32p, _u32p, _f32p, _i32p,
                                                  _f32p, _f32p, _i32p]
            L.hso_cell_of32.restype = C.c_uint32
            L.hso_cell_of32.argtypes = [C.c_float, C.c_float, C.c_float, C.c_float, C.c_int]
            L.hso_cluster_move_at.argtypes = [C.c_void_p, _dp, C.c_int, C.c_int, _i32p]
            L.hso_cavity_psi.argtypes = [C.c_double, C.c_int, _dp, _dp]
            L.hso_cavity_coeffs.argtypes = [C.c_double, _dp]
            L.hso_cavity_setup.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_double]
            L.hso_cavity_sweeps.argtypes = [C.c_void_p, C.c_int]
            L.hso_cavity_replay.argtypes = [C.c_void_p, C.c_int, _i32p, _u32p, _u32p, _i32p]
            L.hso_cluster_moves.argtypes = [C.c_void_p, C.c_int, _i32p]
            cls._lib = L
        return cls._lib

    def __init__(self, rho=0.5, n_cells=5, lattice_type=2, neigh_dr=1.05, neigh_max_part=10, dr_max=0.1,
                 dv_max=0.001, press=0.0, seed=1):
        L = self.lib()
        err = C.c_int(0)
        nx, ny, nz = (n_cells, n_cells, n_cells) if np.isscalar(n_cells) else n_cells
        self._h = L.hso_create(rho, nx, ny, nz, lattice_type, neigh_dr, neigh_max_part, dr_max, dv_max, press,
                               seed, C.byref(err))
        if not self._h:
            raise RuntimeError(f"oracle create failed with code {err.value}")
        self.n = L.hso_n(self._h)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and self._lib is not None:
            self._lib.hso_destroy(h)
            self._h = None

    def _lib_get_config(self, out):
        self._lib.hso_get_config(self._h, out)

    def _lib_box(self, out):
        self._lib.hso_box(self._h, out)

    def set_config(self, conf):
        conf = np.ascontiguousarray(conf, dtype=np.float64)
        e = self._lib.hso_set_config(self._h, conf)
        if e:
            raise RuntimeError(f"oracle set_config failed with code {e}")

    def reset_lattice(self):
        return self._lib.hso_reset_lattice(self._h)

    def set_steps(self, dr_max, dv_max=0.001):
        self._lib.hso_set_steps(self._h, dr_max, dv_max)

    def sweeps_nvt(self, k):
        e = self._lib.hso_sweeps_nvt(self._h, k)
        if e:
            raise RuntimeError(f"oracle sweep failed with code {e}")

    def sweeps_npt(self, k):
        e = self._lib.hso_sweeps_npt(self._h, k)
        if e:
            raise RuntimeError(f"oracle sweep failed with code {e}")

    def _counters(self):
        out = np.zeros(6, dtype=np.uint64)
        self._lib.hso_counters(self._h, out)
        return out

    def reset_counters(self):
        self._lib.hso_reset_counters(self._h)

    def _lib_replay(self, n, ids, raw, acc):
        self._lib.hso_replay_moves(self._h, n, ids, raw, acc)

    def _lib_replay_offsets(self, n, ids, raw, acc):
        self._lib.hso_replay_moves_offsets(self._h, n, ids, raw, acc)

    def widom_points(self, pts):
        pts = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1, 3)
        ov = np.zeros(pts.shape[0], dtype=np.uint8)
        if self._lib.hso_widom_points(self._h, pts.shape[0], pts, ov) < 0:
            raise ValueError("insertion point outside the cell table")
        return ov

    def check_overlap_at(self, i, x, y, z) -> int:
        return self._lib.hso_check_overlap_at(self._h, i, x, y, z)

    def scan_overlap(self, sf) -> int:
        return self._lib.hso_scan_overlap(self._h, sf)

    def vol_move_replay(self, raw) -> int:
        raw = np.ascontiguousarray(raw, dtype=np.uint32)
        return self._lib.hso_vol_move_replay(self._h, raw, raw.size)

    def _lib_rdf(self, *a):
        return self._lib.hso_rdf_counts(self._h, *a)

    def _lib_pressv(self, *a):
        return self._lib.hso_pressv_counts(self._h, *a)

    def _lib_presst(self, *a):
        return self._lib.hso_presst_counts(self._h, *a)

    def presst_counts_sf(self, sf):
        sf = np.ascontiguousarray(sf, dtype=np.float64)
        out = np.zeros(sf.size, dtype=np.float64)
        self._lib.hso_presst_counts_sf(self._h, sf, sf.size, out)
        return out

    def _lib_widom(self, n, raw):
        return self._lib.hso_widom(self._h, n, raw)

    def widom_decisions(self, raw):
        raw = np.ascontiguousarray(raw, dtype=np.uint32).reshape(-1)
        n = raw.size // 3
        ov = np.zeros(n, dtype=np.uint8)
        ok = self._lib.hso_widom_decisions(self._h, n, raw, ov)
        if ok < 0:
            raise ValueError("insertion point outside the cell table")
        return ov

    def widom_rng(self, n) -> int:
        return self._lib.hso_widom_rng(self._h, n)

    def _lib_ql(self, *a):
        return self._lib.hso_ql(self._h, *a)

    def opt_nvt(self, opt_sweeps, opt_samples, target):
        dr = C.c_double()
        acc = C.c_double()
        self._lib.hso_opt_nvt(self._h, opt_sweeps, opt_samples, target, C.byref(dr), C.byref(acc))
        return dr.value, acc.value

    def cluster_move_at(self, pivot, axis, seed_id) -> int:
        """One cluster move (src/cluster_nvt.c:232-310) from the given pivot,
        axis and seed particle; returns the cluster size."""
        piv = np.ascontiguousarray(pivot, dtype=np.float64)
        size = np.zeros(1, dtype=np.int32)
        e = self._lib.hso_cluster_move_at(self._h, piv, int(axis), int(seed_id), size)
        if e:
            raise RuntimeError(f"oracle cluster move failed ({e})")
        return int(size[0])

    def cavity_setup(self, pcav, maxdr=1.2, mindr=0.0):
        e = self._lib.hso_cavity_setup(self._h, pcav, maxdr, mindr)
        if e:
            raise RuntimeError(f"oracle cavity setup failed ({e})")

    def cavity_sweeps(self, n):
        e = self._lib.hso_cavity_sweeps(self._h, n)
        if e:
            raise RuntimeError(f"oracle cavity sweeps failed ({e})")

    def cavity_replay(self, which, raw, uacc):
        which = np.ascontiguousarray(which, dtype=np.int32)
        raw = np.ascontiguousarray(raw, dtype=np.uint32)
        uacc = np.ascontiguousarray(uacc, dtype=np.uint32)
        dec = np.zeros(which.size, dtype=np.int32)
        e = self._lib.hso_cavity_replay(self._h, which.size, which, raw, uacc, dec)
        if e:
            raise RuntimeError(f"oracle cavity replay failed ({e})")
        return dec

    @classmethod
    def cavity_psi(cls, rho, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        out = np.zeros_like(x)
        cls.lib().hso_cavity_psi(rho, x.size, x, out)
        return out

    @classmethod
    def cavity_coeffs(cls, rho):
        out = np.zeros(20)
        cls.lib().hso_cavity_coeffs(rho, out)
        return out

    def cluster_moves(self, n):
        """n cluster moves with the reference's draws; their sizes."""
        sizes = np.zeros(n, dtype=np.int32)
        e = self._lib.hso_cluster_moves(self._h, n, sizes)
        if e:
            raise RuntimeError(f"oracle cluster moves failed ({e})")
        return sizes

    def replay_checkerboard(self, ids, raw, cells, shift32, nc, len32, inv_w32):
        ids = np.ascontiguousarray(ids, dtype=np.int32)
        raw = np.ascontiguousarray(raw, dtype=np.uint32).reshape(-1)
        cells = np.ascontiguousarray(cells, dtype=np.uint32)
        shift32 = np.ascontiguousarray(shift32, dtype=np.float32).reshape(-1)
        dec = np.zeros(ids.size, dtype=np.int32)
        e = self._lib.hso_replay_checkerboard(self._h, ids.size, ids, raw, cells, shift32,
                                              np.ascontiguousarray(nc, dtype=np.int32),
                                              np.ascontiguousarray(len32, dtype=np.float32),
                                              np.ascontiguousarray(inv_w32, dtype=np.float32), dec)
        if e:
            raise RuntimeError(f"oracle replay failed with code {e}")
        return dec

    @classmethod
    def rng_raw(cls, seed, n):
        out = np.zeros(n, dtype=np.uint32)
        cls.lib().hso_rng_raw(seed, n, out)
        return out

    @classmethod
    def rng_uniform_int(cls, seed, rng_range, n):
        out = np.zeros(n, dtype=np.int32)
        cls.lib().hso_rng_uniform_int(seed, rng_range, n, out)
        return out

    @classmethod
    def brute_overlap(cls, conf, box, skip, x, y, z) -> int:
        conf = np.ascontiguousarray(conf, dtype=np.float64)
        return cls.lib().hso_brute_overlap(conf, conf.shape[0], box[0], box[1], box[2], skip, x, y, z)

    @classmethod
    def brute_pair_hist(cls, conf, box, dr, rmax, nbins):
        conf = np.ascontiguousarray(conf, dtype=np.float64)
        out = np.zeros(nbins, dtype=np.uint64)
        e = cls.lib().hso_brute_pair_hist(conf, conf.shape[0], box[0], box[1], box[2], dr, rmax, nbins, out)
        if e:
            raise ValueError("pair outside the histogram")
        return out

    @classmethod
    def cell_of32(cls, x32, shift32, len32, inv_w32, nc):
        return cls.lib().hso_cell_of32(x32, shift32, len32, inv_w32, nc)


class RefSim(_SimBase):
    """The reference's own code (one instance per process: it keeps global
    state)."""

    _lib = None

    @classmethod
    def lib(cls):
        if cls._lib is None:
            if not os.path.exists(REF_SO):
                raise FileNotFoundError("reference build missing; run build_oracle(with_reference=True)")
            L = C.CDLL(REF_SO)
            L.ref_init_from_file.argtypes = [C.c_char_p]
            L.ref_n.argtypes = []
            L.ref_box.argtypes = [_dp]
            L.ref_get_config.argtypes = [_dp]
            L.ref_set_config.argtypes = [_dp]
            L.ref_set_steps.argtypes = [C.c_double, C.c_double]
            L.ref_sweeps_nvt.argtypes = [C.c_int]
            L.ref_sweeps_npt.argtypes = [C.c_int]
            L.ref_counters.argtypes = [_u64p]
            L.ref_replay_moves.argtypes = [C.c_int, _i32p, _u32p, _i32p]
            L.ref_replay_moves_offsets.argtypes = [C.c_int, _i32p, _u32p, _i32p]
            L.ref_check_overlap_at.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double]
            L.ref_scan_overlap.argtypes = [C.c_double]
            L.ref_vol_move_replay.argtypes = [_u32p, C.c_int]
            L.ref_rdf_counts.argtypes = [C.c_double, C.c_double, _dp, C.c_int, C.POINTER(C.c_double)]
            L.ref_pressv_counts.argtypes = [C.c_double, _dp, C.c_int, C.POINTER(C.c_double)]
            L.ref_presst_counts.argtypes = [C.c_double, C.c_double, _dp, C.c_int]
            L.ref_widom.argtypes = [C.c_int, _u32p]
            L.ref_widom_rng.argtypes = [C.c_int]
            L.ref_ql.restype = C.c_double
            L.ref_ql.argtypes = [C.c_int, C.c_double, _dp, C.POINTER(C.c_double)]
            L.ref_rng_raw.argtypes = [C.c_ulong, C.c_int, _u32p]
            L.ref_rng_uniform_int.argtypes = [C.c_ulong, C.c_ulong, C.c_int, _i32p]
            L.ref_cluster_moves.argtypes = [C.c_int, _i32p]
            L.ref_cluster_move_at.argtypes = [_dp, C.c_int, C.c_int]
            L.ref_cavity_setup.argtypes = [C.c_double, C.c_double, C.c_double]
            L.ref_cavity_sweeps.argtypes = [C.c_int]
            L.ref_cavity_psi.argtypes = [C.c_int, _dp, _dp]
            L.ref_cavity_replay.argtypes = [C.c_int, _i32p, _u32p, _u32p, _i32p, _i32p]
            cls._lib = L
        return cls._lib

    def __init__(self, rho=0.5, n_cells=5, lattice_type=2, neigh_dr=1.05, neigh_max_part=10, dr_max=0.1,
                 dv_max=0.001, press=0.0, seed=1):
        L = self.lib()
        nx, ny, nz = (n_cells, n_cells, n_cells) if np.isscalar(n_cells) else n_cells
        kw = dict(rho=repr(float(rho)), cells_x=nx, cells_y=ny, cells_z=nz, type=lattice_type,
                  neigh_list=(repr(float(neigh_dr)), neigh_max_part), dr_max=repr(float(dr_max)), seed=seed,
                  out=1000)
        if press > 0:
            kw["npt"] = (repr(float(press)), repr(float(dv_max)))
        with tempfile.TemporaryDirectory() as td:
            path = os.path.join(td, "in.dat")
            write_input(path, **kw)
            L.ref_init_from_file(path.encode())
        # the parser's default dv_max is used unless npt set it
        L.ref_set_steps(dr_max, dv_max)
        self.n = L.ref_n()

    def _lib_get_config(self, out):
        self._lib.ref_get_config(out)

    def _lib_box(self, out):
        self._lib.ref_box(out)

    def set_config(self, conf):
        self._lib.ref_set_config(np.ascontiguousarray(conf, dtype=np.float64))

    def set_steps(self, dr_max, dv_max=0.001):
        self._lib.ref_set_steps(dr_max, dv_max)

    def sweeps_nvt(self, k):
        self._lib.ref_sweeps_nvt(k)

    def sweeps_npt(self, k):
        self._lib.ref_sweeps_npt(k)

    def _counters(self):
        out = np.zeros(6, dtype=np.uint64)
        self._lib.ref_counters(out)
        return out

    def reset_counters(self):
        self._lib.ref_reset_counters()

    def _lib_replay(self, n, ids, raw, acc):
        self._lib.ref_replay_moves(n, ids, raw, acc)

    def _lib_replay_offsets(self, n, ids, raw, acc):
        self._lib.ref_replay_moves_offsets(n, ids, raw, acc)

    def check_overlap_at(self, i, x, y, z) -> int:
        return self._lib.ref_check_overlap_at(i, x, y, z)

    def scan_overlap(self, sf) -> int:
        return self._lib.ref_scan_overlap(sf)

    def vol_move_replay(self, raw) -> int:
        raw = np.ascontiguousarray(raw, dtype=np.uint32)
        return self._lib.ref_vol_move_replay(raw, raw.size)

    def cluster_moves(self, n):
        sizes = np.zeros(n, dtype=np.int32)
        self._lib.ref_cluster_moves(n, sizes)
        return sizes

    def cavity_setup(self, pcav, maxdr=1.2, mindr=0.0):
        self._lib.ref_cavity_setup(pcav, maxdr, mindr)

    def cavity_sweeps(self, n):
        self._lib.ref_cavity_sweeps(n)

    def cavity_replay(self, which, raw, uacc, draws_acc):
        which = np.ascontiguousarray(which, dtype=np.int32)
        acc = np.zeros(which.size, dtype=np.int32)
        e = self._lib.ref_cavity_replay(which.size, which, np.ascontiguousarray(raw, dtype=np.uint32),
                                        np.ascontiguousarray(uacc, dtype=np.uint32),
                                        np.ascontiguousarray(draws_acc, dtype=np.int32), acc)
        if e:
            raise RuntimeError("reference cavity replay consumed an unexpected number of draws")
        return acc

    def cavity_psi_ref(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        out = np.zeros_like(x)
        self._lib.ref_cavity_psi(x.size, x, out)
        return out

    def cluster_move_at(self, pivot, axis, seed_id) -> int:
        return self._lib.ref_cluster_move_at(np.ascontiguousarray(pivot, dtype=np.float64), int(axis), int(seed_id))

    def _lib_rdf(self, *a):
        return self._lib.ref_rdf_counts(*a)

    def _lib_pressv(self, *a):
        return self._lib.ref_pressv_counts(*a)

    def _lib_presst(self, *a):
        return self._lib.ref_presst_counts(*a)

    def _lib_widom(self, n, raw):
        return self._lib.ref_widom(n, raw)

    def widom_rng(self, n) -> int:
        return self._lib.ref_widom_rng(n)

    def _lib_ql(self, *a):
        return self._lib.ref_ql(*a)

    @classmethod
    def rng_raw(cls, seed, n):
        out = np.zeros(n, dtype=np.uint32)
        cls.lib().ref_rng_raw(seed, n, out)
        return out

    @classmethod
    def rng_uniform_int(cls, seed, rng_range, n):
        out = np.zeros(n, dtype=np.int32)
        cls.lib().ref_rng_uniform_int(seed, rng_range, n, out)
        return out
