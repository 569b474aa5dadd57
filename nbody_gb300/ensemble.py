"""Batched ensemble of independent systems (nbg_ensemble_* in the C ABI).

Each system advances with its own adaptive Dormand-Prince step around the
mixed-precision direct sum; a whole step for all systems is one captured
CUDA graph.  A one-system ensemble is the engine-owned fused RK step.
"""
from __future__ import annotations

import ctypes as C
from typing import Sequence

import numpy as np

from . import _lib
from ._lib import EnsembleParams, NbgError


class Ensemble:
    def __init__(self, device: int = 0, softening: float = 1e-3, tolerance: float = 1e-8,
                 dt_initial: float = 1e-3, dt_min: float = 1e-9, dt_max: float = 1e-1,
                 use_graph: bool = True):
        self._lib = _lib.load()
        p = EnsembleParams()
        self._lib.nbg_ensemble_params_default(C.byref(p))
        p.device, p.softening, p.tolerance = device, softening, tolerance
        p.dt_initial, p.dt_min, p.dt_max = dt_initial, dt_min, dt_max
        p.use_graph = 1 if use_graph else 0
        h = C.c_void_p()
        st = self._lib.nbg_ensemble_create(C.byref(p), C.byref(h))
        if st != 0:
            raise NbgError(st, "nbg_ensemble_create failed")
        self._h = h.value
        self.device = device
        self.softening = softening
        self.counts = np.zeros(0, dtype=np.uint32)

    def _check(self, st: int, what: str) -> None:
        if st != 0:
            raise NbgError(st, f"{what}: {self._lib.nbg_ensemble_last_error(self._h).decode()}")

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.nbg_ensemble_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def tune_set(self, key: str, value: int) -> None:
        self._check(self._lib.nbg_ensemble_tune_set(self._h, key.encode(), int(value)), "tune_set")

    def autotune(self, reps: int = 3) -> dict:
        """nbg_ensemble_autotune: force-kernel tile shape and grid, timed on
        the current state; keeps the fastest; returns the JSON report."""
        import json
        buf = C.create_string_buffer(8192)
        self._check(self._lib.nbg_ensemble_autotune(self._h, int(reps), buf, len(buf)),
                    "autotune")
        return json.loads(buf.value.decode())

    def tune_variant(self) -> str:
        return f"ensemble/{'soft' if self.softening > 0 else 'clamp'}"

    def init(self, systems: Sequence) -> None:
        """systems: NBodyData-like objects (vertices, velocities, mass)."""
        self.counts = np.array([s.get_count() for s in systems], dtype=np.uint32)
        v = np.ascontiguousarray(np.concatenate([s.vertices for s in systems]), dtype=np.float64)
        u = np.ascontiguousarray(np.concatenate([s.velocities for s in systems]), dtype=np.float64)
        m = np.ascontiguousarray(np.concatenate([s.mass for s in systems]), dtype=np.float64)
        self._check(self._lib.nbg_ensemble_init(
            self._h, len(systems), self.counts.ctypes.data_as(C.POINTER(C.c_uint32)),
            v.ctypes.data, u.ctypes.data, m.ctypes.data), "init")

    def step(self, steps: int = 1) -> None:
        self._check(self._lib.nbg_ensemble_step(self._h, steps), "step")

    def synchronize(self) -> None:
        self._check(self._lib.nbg_ensemble_synchronize(self._h), "synchronize")

    def status(self):
        ns = self.counts.size
        t, dt = np.zeros(ns), np.zeros(ns)
        acc = np.zeros(ns, dtype=np.uint32)
        rej = np.zeros(ns, dtype=np.uint32)
        dp = C.POINTER(C.c_double)
        up = C.POINTER(C.c_uint32)
        self._check(self._lib.nbg_ensemble_status(self._h, t.ctypes.data_as(dp),
                                                  dt.ctypes.data_as(dp), acc.ctypes.data_as(up),
                                                  rej.ctypes.data_as(up)), "status")
        return t, dt, acc, rej

    def get_state(self):
        b = int(self.counts.sum())
        v, u = np.zeros((b, 3)), np.zeros((b, 3))
        self._check(self._lib.nbg_ensemble_get_state(self._h, v.ctypes.data, u.ctypes.data),
                    "get_state")
        return v, u

    def fcompute(self) -> np.ndarray:
        b = int(self.counts.sum())
        f = np.zeros(6 * b)
        self._check(self._lib.nbg_ensemble_fcompute(self._h, f.ctypes.data_as(C.POINTER(C.c_double))),
                    "fcompute")
        return f

    def statistics(self) -> np.ndarray:
        out = np.zeros((self.counts.size, 12))
        self._check(self._lib.nbg_ensemble_statistics(self._h, out.ctypes.data_as(C.POINTER(C.c_double))),
                    "statistics")
        return out

    def launch_count(self) -> int:
        return int(self._lib.nbg_ensemble_launch_count(self._h))

    def profile(self, enable: bool):
        ms = C.c_double(0.0)
        n = C.c_uint64(0)
        self._check(self._lib.nbg_ensemble_profile(self._h, 1 if enable else 0, C.byref(ms),
                                                   C.byref(n)), "profile")
        return ms.value, n.value
