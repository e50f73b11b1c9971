"""Learned Widom proposal over the hsmc_lwidom_* entry points of
include/hsmc_gpu.h: importance-sampled test-particle insertions
(compute_mu, src/compute_widom_chem_pot.c:32-182) whose points come from a
mixture of a learned sub-cell proposal and the uniform one."""
from __future__ import annotations

import ctypes as C
import math
import weakref

import numpy as np

from . import _native
from .system import HsmcError, _check

NPARAMS = 6273


class Stats(C.Structure):
    _fields_ = [("sum_w", C.c_double), ("sum_w2", C.c_double), ("n", C.c_uint64), ("n_ok", C.c_uint64),
                ("n_learned", C.c_uint64)]

    def estimate(self):
        """Insertion probability, its per-insertion variance, and beta mu_ex."""
        n = max(int(self.n), 1)
        p = self.sum_w / n
        var = max(self.sum_w2 / n - p * p, 0.0)
        return p, var, (-math.log(p) if p > 0 else float("inf"))


def _bind(lib):
    if getattr(lib, "_lwidom_bound", False):
        return
    vp, P = C.c_void_p, C.POINTER
    lib.hsmc_lwidom_create.argtypes = [vp, C.c_double, C.c_uint64, C.c_int64, P(vp)]
    lib.hsmc_lwidom_destroy.argtypes = [vp]
    lib.hsmc_lwidom_destroy.restype = None
    lib.hsmc_lwidom_set_params.argtypes = [vp, vp]
    lib.hsmc_lwidom_get_params.argtypes = [vp, vp]
    lib.hsmc_lwidom_subgrid.argtypes = [vp, vp]
    lib.hsmc_lwidom_refresh.argtypes = [vp]
    lib.hsmc_lwidom_patterns.argtypes = [vp, vp, C.c_int64]
    lib.hsmc_lwidom_proposal.argtypes = [vp, vp, vp, C.c_int64]
    lib.hsmc_lwidom_logits.argtypes = [vp, vp, C.c_int64, vp]
    lib.hsmc_lwidom_grad.argtypes = [vp, vp, C.c_int64, C.c_float, C.c_float, vp, P(C.c_double)]
    lib.hsmc_lwidom_adam_step.argtypes = [vp, vp, C.c_float]
    lib.hsmc_lwidom_insert.argtypes = [vp, C.c_int64, C.c_double, C.c_double, P(Stats)]
    lib.hsmc_lwidom_insert_traced.argtypes = [vp, C.c_int64, C.c_double, vp, vp, vp, vp, vp, P(Stats)]
    lib.hsmc_lwidom_uniform.argtypes = [vp, C.c_int64, P(C.c_uint64)]
    lib.hsmc_lwidom_train.argtypes = [vp, C.c_int, C.c_int64, C.c_float, C.c_float, C.c_float, P(C.c_double)]
    lib.hsmc_lwidom_samples.argtypes = [vp, P(C.c_int64), P(C.c_int64)]
    lib.hsmc_lwidom_clear_samples.argtypes = [vp]
    lib.hsmc_lwidom_last_timing.argtypes = [vp, P(C.c_double)]
    lib._lwidom_bound = True


class LearnedWidom:
    """Learned insertion proposal attached to a HardSphereSystem."""

    def __init__(self, system, subcell_edge: float = 0.5, seed: int = 1, train_capacity: int = 0):
        lib = _native.load()
        _bind(lib)
        self._lib = lib
        self.system = system
        h = C.c_void_p()
        _check(lib.hsmc_lwidom_create(system._h, subcell_edge, seed, train_capacity, C.byref(h)),
               "hsmc_lwidom_create")
        self._h = h
        # runs on the system's stream: the system closes this first, in
        # whatever order the two are collected
        system._dependents.append(weakref.ref(self))
        ns = np.zeros(3, dtype=np.int32)
        _check(lib.hsmc_lwidom_subgrid(h, ns.ctypes.data), "hsmc_lwidom_subgrid")
        self.ns = ns

    def close(self):
        if getattr(self, "_h", None):
            self._lib.hsmc_lwidom_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def n_subcells(self) -> int:
        return int(np.prod(self.ns))

    def params(self) -> np.ndarray:
        out = np.empty(NPARAMS, dtype=np.float32)
        _check(self._lib.hsmc_lwidom_get_params(self._h, out.ctypes.data), "hsmc_lwidom_get_params")
        return out

    def set_params(self, p) -> None:
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.shape == (NPARAMS,)
        _check(self._lib.hsmc_lwidom_set_params(self._h, p.ctypes.data), "hsmc_lwidom_set_params")

    def use_prior(self, beta: float = 1.5, z0: float = -5.0) -> None:
        """Start from a network whose output is z0 - beta * (occupied
        neighbour sub-cells) plus its small random part: hidden unit 0 of both
        layers carries 27 - count (exact in bfloat16)."""
        p = self.params()
        w1 = p[:64 * 32].reshape(64, 32)
        w2 = p[2048:6144].reshape(64, 64)
        b2 = p[6144:6208]
        w3 = p[6208:6272]
        w1[0, :27] = -1.0
        w1[0, 27] = 27.0
        w2[0, :] = 0.0
        w2[0, 0] = 1.0
        b2[0] = 0.0
        w3 *= 0.01
        w3[0] = beta
        p[6272] = z0 - 27.0 * beta
        self.set_params(p)

    def refresh(self) -> float:
        _check(self._lib.hsmc_lwidom_refresh(self._h), "hsmc_lwidom_refresh")
        ns = np.zeros(3, dtype=np.int32)
        _check(self._lib.hsmc_lwidom_subgrid(self._h, ns.ctypes.data), "hsmc_lwidom_subgrid")
        self.ns = ns
        return self.last_ms()

    def patterns(self) -> np.ndarray:
        out = np.empty(self.n_subcells, dtype=np.uint32)
        _check(self._lib.hsmc_lwidom_patterns(self._h, out.ctypes.data, out.shape[0]), "hsmc_lwidom_patterns")
        return out

    def proposal(self):
        pi = np.empty(self.n_subcells, dtype=np.float64)
        cdf = np.empty(self.n_subcells, dtype=np.float64)
        _check(self._lib.hsmc_lwidom_proposal(self._h, pi.ctypes.data, cdf.ctypes.data, pi.shape[0]),
               "hsmc_lwidom_proposal")
        return pi, cdf

    def logits(self, patterns) -> np.ndarray:
        pat = np.ascontiguousarray(patterns, dtype=np.uint32)
        out = np.empty(pat.shape[0], dtype=np.float32)
        _check(self._lib.hsmc_lwidom_logits(self._h, pat.ctypes.data, pat.shape[0], out.ctypes.data),
               "hsmc_lwidom_logits")
        return out

    def grad(self, samples, w_pos: float = 1.0, w_neg: float = 1.0):
        smp = np.ascontiguousarray(samples, dtype=np.uint32)
        g = np.empty(NPARAMS, dtype=np.float32)
        loss = C.c_double()
        _check(self._lib.hsmc_lwidom_grad(self._h, smp.ctypes.data, smp.shape[0], w_pos, w_neg, g.ctypes.data,
                                          C.byref(loss)), "hsmc_lwidom_grad")
        return loss.value, g

    def adam_step(self, grad, lr: float) -> None:
        g = np.ascontiguousarray(grad, dtype=np.float32)
        _check(self._lib.hsmc_lwidom_adam_step(self._h, g.ctypes.data, lr), "hsmc_lwidom_adam_step")

    def insert(self, n: int, alpha: float = 0.1, keep_failures: float | None = None) -> Stats:
        """n insertions; with keep_failures set, every success and that
        fraction of the failures go to the training buffer."""
        st = Stats()
        keep = -1.0 if keep_failures is None else float(keep_failures)
        _check(self._lib.hsmc_lwidom_insert(self._h, n, alpha, keep, C.byref(st)), "hsmc_lwidom_insert")
        return st

    def insert_traced(self, n: int, alpha: float = 0.1):
        pts = np.empty((n, 3), dtype=np.float64)
        cell = np.empty(n, dtype=np.int32)
        uni = np.empty(n, dtype=np.uint8)
        w = np.empty(n, dtype=np.float64)
        ok = np.empty(n, dtype=np.uint8)
        st = Stats()
        _check(self._lib.hsmc_lwidom_insert_traced(self._h, n, alpha, pts.ctypes.data, cell.ctypes.data,
                                                   uni.ctypes.data, w.ctypes.data, ok.ctypes.data, C.byref(st)),
               "hsmc_lwidom_insert_traced")
        return pts, cell, uni, w, ok, st

    def uniform(self, n: int) -> int:
        acc = C.c_uint64()
        _check(self._lib.hsmc_lwidom_uniform(self._h, n, C.byref(acc)), "hsmc_lwidom_uniform")
        return int(acc.value)

    def train(self, epochs: int = 1, batch: int = 65536, lr: float = 1e-3, w_pos: float = 1.0,
              w_neg: float = 1.0) -> float:
        loss = C.c_double()
        _check(self._lib.hsmc_lwidom_train(self._h, epochs, batch, lr, w_pos, w_neg, C.byref(loss)),
               "hsmc_lwidom_train")
        return loss.value

    def samples(self):
        n, npos = C.c_int64(), C.c_int64()
        _check(self._lib.hsmc_lwidom_samples(self._h, C.byref(n), C.byref(npos)), "hsmc_lwidom_samples")
        return n.value, npos.value

    def clear_samples(self) -> None:
        _check(self._lib.hsmc_lwidom_clear_samples(self._h), "hsmc_lwidom_clear_samples")

    def last_ms(self) -> float:
        t = C.c_double()
        _check(self._lib.hsmc_lwidom_last_timing(self._h, C.byref(t)), "hsmc_lwidom_last_timing")
        return t.value

    def fit(self, rounds: int = 8, per_round: int = 125_000_000, keep_failures: float = 0.01,
            alpha: float = 0.1, epochs: int = 2, batch: int = 65536, lr: float = 2e-3, sweeps_between: int = 20,
            max_w_pos: float = 1e4):
        """Self-training loop.  Each round draws per_round insertions from the
        current mixture (the first round from the initial network), keeps
        every success and keep_failures of the failures, and trains on all
        outcomes kept so far: failures weighted 1 / keep_failures, successes
        by min(weighted failures / successes, max_w_pos).  Conditional on its
        sub-cell a point is uniform whatever the proposal, so the labels are
        unbiased samples of P(success | pattern) in every round.  Returns
        per-round (kept outcomes, kept successes, loss, device ms)."""
        log = []
        w_neg = 1.0 / keep_failures
        for _ in range(rounds):
            ms = 0.0
            if sweeps_between:
                self.system.sweep_nvt(sweeps_between)
            ms += self.refresh()
            self.insert(per_round, alpha=alpha, keep_failures=keep_failures)
            ms += self.last_ms()
            n, npos = self.samples()
            w_pos = min((n - npos) * w_neg / max(npos, 1), max_w_pos)
            loss = self.train(epochs=epochs, batch=batch, lr=lr, w_pos=float(w_pos), w_neg=float(w_neg))
            ms += self.last_ms()
            log.append((n, npos, loss, ms))
        return log


__all__ = ["LearnedWidom", "Stats", "HsmcError", "NPARAMS"]
