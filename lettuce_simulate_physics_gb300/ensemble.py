"""Batched ensembles of independent systems over the engine's C ABI (lg_ensemble_*).

No counterpart in the reference: many systems of uneven N advance together, each with the
reference's single-system physics (kick-drift-kick steps; direct or Barnes-Hut quadrupole forces)
and its own softening and opening angle. Systems are passed back to back; results come back in the
same system order, each system's bodies in the engine's current order (ids identify them).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from .backend import ForceMethod, _CEnsStats, _CEnsTuning, _check, _d, _f, _lib, _u
from .bodies import Bodies


@dataclass
class EnsembleStats:
    run_ms: float
    steps: int
    used_graph: bool
    captures: int
    recoveries: int
    nsys: int
    nsys_tree: int
    nsys_direct: int
    n: int
    n_tree: int
    n_direct: int
    launches_per_step: int
    last_interactions: int


@dataclass
class EnsembleTuning:
    direct_ipt: tuple
    walk_group: int
    tuned: bool
    direct_tile: tuple = (256, 256, 256)


class Ensemble:
    def __init__(self, device: int = 0):
        lib = _lib()
        h = C.c_void_p()
        _check(lib.lg_ensemble_create(int(device), C.byref(h)))
        self._h = h
        self._lib = lib
        self._counts = np.zeros(0, np.uint32)

    def close(self) -> None:
        if self._h:
            self._lib.lg_ensemble_destroy(self._h)
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

    def upload(self, bodies: Bodies, counts, eps, theta, method, G: float = 1.0) -> None:
        """bodies: all systems back to back; counts[s] bodies of system s; eps[s] > 0; theta[s]
        (tree systems); method[s] ForceMethod.direct or ForceMethod.tree."""
        counts = np.ascontiguousarray(counts, np.uint32)
        eps = np.ascontiguousarray(eps, np.float64)
        theta = np.ascontiguousarray(theta, np.float64)
        method = np.ascontiguousarray([int(m) for m in method], np.int32)
        ns = len(counts)
        if not (len(eps) == len(theta) == len(method) == ns):
            raise ValueError("counts, eps, theta and method need one entry per system")
        if int(counts.sum()) != len(bodies):
            raise ValueError("sum of counts differs from the number of bodies")
        b = bodies
        _check(self._lib.lg_ensemble_upload(
            self._h, ns, counts.ctypes.data_as(_u), eps.ctypes.data_as(_d), theta.ctypes.data_as(_d),
            method.ctypes.data_as(C.POINTER(C.c_int)), float(G), *(a.ctypes.data_as(_f) for a in
                                                                   (b.x, b.y, b.z, b.vx, b.vy, b.vz, b.m)),
            b.id.ctypes.data_as(_u)))
        self._counts = counts

    def run(self, dt: float, steps: int, use_graph: bool = True) -> None:
        _check(self._lib.lg_ensemble_run(self._h, float(dt), int(steps), int(bool(use_graph))))

    def energy(self):
        """(E, KE, PE) per system, FP64, evaluated with fresh forces at the current state."""
        ns = len(self._counts)
        out = np.zeros((3, max(ns, 1)), np.float64)
        _check(self._lib.lg_ensemble_energy(self._h, *(out[k].ctypes.data_as(_d) for k in range(3))))
        return out[0, :ns].copy(), out[1, :ns].copy(), out[2, :ns].copy()

    def download(self) -> Bodies:
        n = int(self._counts.sum())
        out = Bodies.empty(n)
        _check(self._lib.lg_ensemble_download(self._h, *(a.ctypes.data_as(_f) for a in
                                                         (out.x, out.y, out.z, out.vx, out.vy, out.vz, out.m)),
                                              out.id.ctypes.data_as(_u)))
        return out

    def accel(self) -> np.ndarray:
        """(4, n) ax, ay, az, phi of the last force phase, in download order."""
        n = int(self._counts.sum())
        a = np.zeros((4, max(n, 1)), np.float32)
        _check(self._lib.lg_ensemble_read_accel(self._h, *(a[k].ctypes.data_as(_f) for k in range(4))))
        return a[:, :n]

    def tune(self) -> EnsembleTuning:
        _check(self._lib.lg_ensemble_tune(self._h))
        return self.tuning()

    def tuning(self) -> EnsembleTuning:
        t = _CEnsTuning()
        _check(self._lib.lg_ensemble_get_tuning(self._h, C.byref(t)))
        return EnsembleTuning(tuple(int(v) for v in t.direct_ipt), int(t.walk_group), bool(t.tuned),
                              tuple(int(v) for v in t.direct_tile))

    def set_tuning(self, direct_ipt, walk_group: int, direct_tile=(256, 256, 256)) -> None:
        t = _CEnsTuning()
        for k in range(3):
            t.direct_ipt[k] = int(direct_ipt[k])
            t.direct_tile[k] = int(direct_tile[k])
        t.walk_group = int(walk_group)
        t.tuned = 1
        _check(self._lib.lg_ensemble_set_tuning(self._h, C.byref(t)))

    def stats(self) -> EnsembleStats:
        s = _CEnsStats()
        _check(self._lib.lg_ensemble_get_stats(self._h, C.byref(s)))
        return EnsembleStats(float(s.run_ms), int(s.steps), bool(s.used_graph), int(s.captures), int(s.recoveries),
                             int(s.nsys), int(s.nsys_tree), int(s.nsys_direct), int(s.n), int(s.n_tree),
                             int(s.n_direct), int(s.launches_per_step), int(s.last_interactions))


def split(bodies: Bodies, counts):
    """Per-system views of back-to-back bodies: list of index slices."""
    off = np.concatenate([[0], np.cumsum(np.asarray(counts, np.int64))])
    return [slice(int(off[k]), int(off[k + 1])) for k in range(len(counts))]


def methods_by_size(counts, direct_max: int = 8192):
    return [ForceMethod.direct if int(c) <= direct_max else ForceMethod.tree for c in counts]
