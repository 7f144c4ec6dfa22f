"""The reference's Backend interface (src/backend.hpp:89-148) over the engine's C ABI.

This is the Python face of include/lettuce_gb300.h, shaped like the reference's C++ class so the
parity tests read like the reference's own tests (tests/test_cuda_backend.cpp): the same method
names, argument meaning and error behaviour. Errors map as the reference's do: std::logic_error ->
LogicError, std::runtime_error -> RuntimeError, and make_cuda_backend returns (None, why) when no
usable device exists.

The library is the in-tree build (lettuce_simulate_physics_gb300/_build/liblettuce_gb300.so). There
is no fallback: without it every call fails loudly.
"""
from __future__ import annotations

import ctypes as C
import enum
import os
from dataclasses import dataclass, field

import numpy as np

from .bodies import Bodies

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "liblettuce_gb300.so")

LG_OK, LG_ERR_RUNTIME, LG_ERR_LOGIC, LG_ERR_ARG, LG_ERR_UNAVAILABLE = range(5)


class LogicError(Exception):
    """A call made in the wrong state (the reference's std::logic_error)."""


class UnavailableError(RuntimeError):
    """No usable CUDA device, or no sm_103a image for it."""


class ForceMethod(enum.IntEnum):
    direct = 0
    tree = 1


@dataclass
class ForceParams:
    G: float = 1.0
    eps: float = 0.01
    theta: float = 0.6
    method: ForceMethod = ForceMethod.direct


@dataclass
class Diag:
    mass: float = 0.0
    ke: float = 0.0
    pe: float = 0.0
    has_pe: bool = False
    px: float = 0.0
    py: float = 0.0
    pz: float = 0.0
    lx: float = 0.0
    ly: float = 0.0
    lz: float = 0.0
    cx: float = 0.0
    cy: float = 0.0
    cz: float = 0.0


@dataclass
class PhaseTimes:
    force_ms: float = 0.0
    sort_ms: float = 0.0
    build_ms: float = 0.0
    walk_ms: float = 0.0
    step_ms: float = 0.0
    interactions: int = 0
    comm_ms: float = 0.0
    balance_ms: float = 0.0


@dataclass
class Box3:
    lo: tuple = (0.0, 0.0, 0.0)
    hi: tuple = (0.0, 0.0, 0.0)


@dataclass
class MemoryNeed:
    device: int = 0
    host: int = 0


class _CForceParams(C.Structure):
    _fields_ = [("G", C.c_double), ("eps", C.c_double), ("theta", C.c_double), ("method", C.c_int32),
                ("reserved", C.c_int32)]


class _CDiag(C.Structure):
    _fields_ = [("mass", C.c_double), ("ke", C.c_double), ("pe", C.c_double), ("has_pe", C.c_int32),
                ("reserved", C.c_int32)] + [(k, C.c_double) for k in ("px", "py", "pz", "lx", "ly", "lz",
                                                                         "cx", "cy", "cz")]


class _CTimes(C.Structure):
    _fields_ = [("force_ms", C.c_double), ("sort_ms", C.c_double), ("build_ms", C.c_double),
                ("walk_ms", C.c_double), ("step_ms", C.c_double), ("interactions", C.c_uint64),
                ("comm_ms", C.c_double), ("balance_ms", C.c_double)]


class _CMem(C.Structure):
    _fields_ = [("device", C.c_uint64), ("host", C.c_uint64)]


class _CEnsStats(C.Structure):
    _fields_ = [("run_ms", C.c_double), ("steps", C.c_int), ("used_graph", C.c_int), ("captures", C.c_int),
                ("recoveries", C.c_int), ("nsys", C.c_int), ("nsys_tree", C.c_int), ("nsys_direct", C.c_int),
                ("n", C.c_size_t), ("n_tree", C.c_size_t), ("n_direct", C.c_size_t),
                ("launches_per_step", C.c_ulonglong), ("last_interactions", C.c_ulonglong)]


class _CEnsTuning(C.Structure):
    _fields_ = [("direct_ipt", C.c_int * 3), ("walk_group", C.c_int), ("tuned", C.c_int), ("direct_tile", C.c_int * 3)]


# LetNode (src/backend.hpp:62-75): the 60-byte record of a locally-essential tree node.
LET_NODE_DTYPE = np.dtype([("cx", "<f4"), ("cy", "<f4"), ("cz", "<f4"), ("mass", "<f4"), ("qxx", "<f4"),
                           ("qxy", "<f4"), ("qxz", "<f4"), ("qyy", "<f4"), ("qyz", "<f4"), ("qzz", "<f4"),
                           ("rcrit2", "<f4"), ("first_child", "<i4"), ("child_count", "<i4"),
                           ("body_first", "<i4"), ("body_count", "<i4")])
assert LET_NODE_DTYPE.itemsize == 60


@dataclass
class LetTree:
    """LetTree (src/backend.hpp:83-86): nodes (root first) and their bodies."""
    nodes: np.ndarray = field(default_factory=lambda: np.zeros(0, LET_NODE_DTYPE))
    bx: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float32))
    by: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float32))
    bz: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float32))
    bm: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float32))


class _CRenderOptions(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("view", C.c_char_p), ("extent", C.c_double),
                ("color", C.c_int32), ("reserved", C.c_int32)]


class _CLetTree(C.Structure):
    _fields_ = [("nodes", C.c_void_p), ("nnodes", C.c_size_t), ("bx", C.POINTER(C.c_float)),
                ("by", C.POINTER(C.c_float)), ("bz", C.POINTER(C.c_float)), ("bm", C.POINTER(C.c_float)),
                ("nbodies", C.c_size_t)]


_f = C.POINTER(C.c_float)
_u = C.POINTER(C.c_uint32)
_d = C.POINTER(C.c_double)
_lib_handle = None


def library_path() -> str:
    return LIB_PATH


def _lib() -> C.CDLL:
    global _lib_handle
    if _lib_handle is not None:
        return _lib_handle
    if not os.path.isfile(LIB_PATH):
        raise RuntimeError(f"engine library {LIB_PATH} is not built; run lettuce_simulate_physics_gb300.build.build()")
    lib = C.CDLL(LIB_PATH)
    vp = C.c_void_p
    st = C.c_int
    sigs = {
        "lg_last_error": (C.c_char_p, []),
        "lg_compiled": (C.c_int, []),
        "lg_device_count": (C.c_int, []),
        "lg_create": (st, [C.c_int, C.POINTER(vp)]),
        "lg_destroy": (None, [vp]),
        "lg_name": (st, [vp, C.c_char_p, C.c_size_t]),
        "lg_upload": (st, [vp, C.c_size_t, _f, _f, _f, _f, _f, _f, _f, _u]),
        "lg_size": (st, [vp, C.POINTER(C.c_size_t)]),
        "lg_download": (st, [vp, _f, _f, _f, _f, _f, _f, _f, _u]),
        "lg_compute_forces": (st, [vp, C.POINTER(_CForceParams), C.c_int]),
        "lg_kick": (st, [vp, C.c_double]),
        "lg_drift": (st, [vp, C.c_double]),
        "lg_diagnostics": (st, [vp, C.POINTER(_CDiag)]),
        "lg_exact_potential_energy": (st, [vp, C.c_double, C.c_double, _d]),
        "lg_times": (st, [vp, C.POINTER(_CTimes)]),
        "lg_local_bounds": (st, [vp, _f, _f]),
        "lg_build_tree": (st, [vp, C.POINTER(_CForceParams)]),
        "lg_compute_forces_with": (st, [vp, C.POINTER(_CForceParams), C.c_int, C.POINTER(_CLetTree), C.c_size_t]),
        "lg_export_let": (st, [vp, _f, _f, C.POINTER(_CForceParams), C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]),
        "lg_export_let_read": (st, [vp, C.c_void_p, _f, _f, _f, _f]),
        "lg_upload64": (st, [vp, C.c_size_t, _d, _d, _d, _f, _f, _f, _f, _u]),
        "lg_render": (st, [vp, C.POINTER(_CRenderOptions), C.POINTER(C.c_ubyte), _d]),
        "lg_block_step": (st, [vp, C.POINTER(_CForceParams), C.c_double, C.c_int, C.c_double, C.c_int]),
        "lg_block_levels": (st, [vp, C.POINTER(C.c_uint8), C.c_size_t]),
        "lg_write_fp64_sidecar": (st, [vp, C.c_char_p, C.c_uint64]),
        "lg_read_fp64_sidecar": (st, [C.c_char_p, C.c_size_t, _u, _f, _f, _f, _d, _d, _d, C.POINTER(C.c_uint64)]),
        "lg_memory_need": (st, [C.c_uint64, C.c_int, C.POINTER(_CMem)]),
        "lg_device_memory": (st, [vp, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
        "lg_body_costs": (st, [vp, _f, C.c_size_t, C.POINTER(C.c_int)]),
        "lg_read_accel": (st, [vp, _f, _f, _f, _f]),
        "lg_read_pos64": (st, [vp, _d, _d, _d]),
        "lg_tree_counts": (st, [vp, C.POINTER(C.c_size_t), C.POINTER(C.c_size_t), C.POINTER(C.c_size_t),
                                C.POINTER(C.c_int)]),
        "lg_tree_keys": (st, [vp, C.POINTER(C.c_uint64), C.c_size_t]),
        "lg_tree_nodes": (st, [vp, _u, _f, _f, C.c_size_t]),
        "lg_tree_groups": (st, [vp, _f, _u, C.c_size_t]),
        "lg_event_record": (st, [vp, C.c_int]),
        "lg_event_elapsed": (st, [vp, C.c_int, C.c_int, C.POINTER(C.c_float)]),
        "lg_synchronize": (st, [vp]),
        "lg_flush_l2": (st, [vp]),
        "lg_launch_count": (st, [vp, C.POINTER(C.c_uint64)]),
        "lg_interaction_split": (st, [vp, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
        "lg_probe_fp32_peak": (st, [vp, C.POINTER(C.c_double)]),
        "lg_probe_wait_timeout": (st, [vp, C.c_uint]),
        "lg_host_alloc": (st, [C.c_size_t, C.POINTER(vp)]),
        "lg_adjoint_forward": (st, [vp, C.POINTER(_CForceParams), C.c_double, C.c_int, C.c_int]),
        "lg_adjoint_backward": (st, [vp, _d, _d, _d, _d, _d, _d, _d, _d, _d, _d, _d]),
        "lg_adjoint_backward_seeded": (st, [vp, _d, _d, _d, _d, _d, _d, _d, _d, _d, _d]),
        "lg_host_free": (st, [vp]),
        "lg_ensemble_create": (st, [C.c_int, C.POINTER(vp)]),
        "lg_ensemble_destroy": (st, [vp]),
        "lg_ensemble_upload": (st, [vp, C.c_size_t, _u, _d, _d, C.POINTER(C.c_int), C.c_double,
                                    _f, _f, _f, _f, _f, _f, _f, _u]),
        "lg_ensemble_run": (st, [vp, C.c_double, C.c_int, C.c_int]),
        "lg_ensemble_energy": (st, [vp, _d, _d, _d]),
        "lg_ensemble_download": (st, [vp, _f, _f, _f, _f, _f, _f, _f, _u]),
        "lg_ensemble_read_accel": (st, [vp, _f, _f, _f, _f]),
        "lg_ensemble_tune": (st, [vp]),
        "lg_ensemble_get_tuning": (st, [vp, C.POINTER(_CEnsTuning)]),
        "lg_ensemble_set_tuning": (st, [vp, C.POINTER(_CEnsTuning)]),
        "lg_ensemble_get_stats": (st, [vp, C.POINTER(_CEnsStats)]),
    }
    for name, (res, args) in sigs.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib_handle = lib
    return lib


def last_error() -> str:
    return _lib().lg_last_error().decode()


def _check(status: int) -> None:
    if status == LG_OK:
        return
    msg = last_error()
    if status == LG_ERR_LOGIC:
        raise LogicError(msg)
    if status == LG_ERR_UNAVAILABLE:
        raise UnavailableError(msg)
    if status == LG_ERR_ARG:
        raise ValueError(msg)
    raise RuntimeError(msg)


def _fp(a):
    return a.ctypes.data_as(_f)


def _up(a):
    return a.ctypes.data_as(_u)


def _cparams(p: ForceParams) -> _CForceParams:
    return _CForceParams(float(p.G), float(p.eps), float(p.theta), int(p.method), 0)


def read_fp64_sidecar(path: str, b: Bodies):
    """FP64 positions (n, 3) of the snapshot bodies b from their sidecar, and the step it records."""
    n = len(b)
    out = np.zeros((3, max(n, 1)), np.float64)
    step = C.c_uint64()
    _check(_lib().lg_read_fp64_sidecar(os.fsencode(path), n, _up(b.id), _fp(b.x), _fp(b.y), _fp(b.z),
                                       *(out[k].ctypes.data_as(_d) for k in range(3)), C.byref(step)))
    return out[:, :n].T.copy(), int(step.value)


def cuda_compiled() -> bool:
    return bool(_lib().lg_compiled())


def cuda_device_count() -> int:
    return int(_lib().lg_device_count())


class CudaBackend:
    """Backend (src/backend.hpp:89-141) on one GB300 through the engine's C ABI."""

    def __init__(self, device: int = 0):
        lib = _lib()
        h = C.c_void_p()
        _check(lib.lg_create(int(device), C.byref(h)))
        self._h = h
        self._lib = lib

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.lg_destroy(self._h)
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

    # ---- Backend ----
    def name(self) -> str:
        buf = C.create_string_buffer(512)
        _check(self._lib.lg_name(self._h, buf, 512))
        return buf.value.decode()

    def upload(self, b: Bodies) -> None:
        _check(self._lib.lg_upload(self._h, len(b), _fp(b.x), _fp(b.y), _fp(b.z), _fp(b.vx), _fp(b.vy), _fp(b.vz),
                                   _fp(b.m), _up(b.id)))

    def upload64(self, b: Bodies, pos64) -> None:
        """upload with FP64 positions pos64 (n, 3) (b's positions are ignored)."""
        p = np.ascontiguousarray(np.asarray(pos64, np.float64).reshape(len(b), 3).T)
        _check(self._lib.lg_upload64(self._h, len(b), *(p[k].ctypes.data_as(_d) for k in range(3)), _fp(b.vx),
                                     _fp(b.vy), _fp(b.vz), _fp(b.m), _up(b.id)))

    def render(self, width: int = 1024, height: int = 1024, view: str = "xy", extent: float = 0.0,
               color: str = "density"):
        """Density render of the resident bodies (render_image): ((height, width, 3) uint8, extent)."""
        o = _CRenderOptions(int(width), int(height), view.encode(), float(extent), 1 if color == "speed" else 0, 0)
        rgb = np.zeros((int(height), int(width), 3), np.uint8)
        ext = C.c_double()
        _check(self._lib.lg_render(self._h, C.byref(o), rgb.ctypes.data_as(C.POINTER(C.c_ubyte)), C.byref(ext)))
        return rgb, float(ext.value)

    def block_step(self, p: ForceParams, dt: float, max_level: int, eta: float, steps: int = 1) -> None:
        """Block (hierarchical) time steps: `steps` steps of dt, bodies on levels dt / 2^k."""
        cp = _cparams(p)
        _check(self._lib.lg_block_step(self._h, C.byref(cp), float(dt), int(max_level), float(eta), int(steps)))

    def block_levels(self) -> np.ndarray:
        n = self.size()
        lv = np.zeros(max(n, 1), np.uint8)
        _check(self._lib.lg_block_levels(self._h, lv.ctypes.data_as(C.POINTER(C.c_uint8)), n))
        return lv[:n]

    def write_fp64_sidecar(self, path: str, step: int = 0) -> None:
        """The low parts of the FP64 positions, in download order, next to a float snapshot."""
        _check(self._lib.lg_write_fp64_sidecar(self._h, os.fsencode(path), int(step)))

    def size(self) -> int:
        n = C.c_size_t()
        _check(self._lib.lg_size(self._h, C.byref(n)))
        return int(n.value)

    def download(self, out: Bodies | None = None) -> Bodies:
        """The resident bodies in the backend's current order (src/backend.hpp:96). With ``out``
        (for instance PinnedBodies(n).bodies) the arrays are written in place: each must be a
        contiguous float32 (id: uint32) array of exactly size() elements."""
        n = self.size()
        if out is None:
            out = Bodies.empty(n)
        else:
            for f in ("x", "y", "z", "vx", "vy", "vz", "m", "id"):
                a = getattr(out, f)
                want = np.uint32 if f == "id" else np.float32
                if a.dtype != want or a.shape != (n,) or not a.flags.c_contiguous or not a.flags.writeable:
                    raise ValueError(f"download: out.{f} must be a writable contiguous {np.dtype(want).name} "
                                     f"array of {n} elements")
        _check(self._lib.lg_download(self._h, _fp(out.x), _fp(out.y), _fp(out.z), _fp(out.vx), _fp(out.vy),
                                     _fp(out.vz), _fp(out.m), _up(out.id)))
        return out

    def compute_forces(self, p: ForceParams, potential: bool = False) -> None:
        cp = _cparams(p)
        _check(self._lib.lg_compute_forces(self._h, C.byref(cp), int(bool(potential))))

    def kick(self, dt: float) -> None:
        _check(self._lib.lg_kick(self._h, float(dt)))

    def drift(self, dt: float) -> None:
        _check(self._lib.lg_drift(self._h, float(dt)))

    def diagnostics(self) -> Diag:
        d = _CDiag()
        _check(self._lib.lg_diagnostics(self._h, C.byref(d)))
        return Diag(d.mass, d.ke, d.pe, bool(d.has_pe), d.px, d.py, d.pz, d.lx, d.ly, d.lz, d.cx, d.cy, d.cz)

    def exact_potential_energy(self, G: float, eps: float) -> float:
        out = C.c_double()
        _check(self._lib.lg_exact_potential_energy(self._h, float(G), float(eps), C.byref(out)))
        return float(out.value)

    def times(self) -> PhaseTimes:
        t = _CTimes()
        _check(self._lib.lg_times(self._h, C.byref(t)))
        return PhaseTimes(t.force_ms, t.sort_ms, t.build_ms, t.walk_ms, t.step_ms, int(t.interactions), t.comm_ms,
                          t.balance_ms)

    def local_bounds(self) -> Box3:
        lo = np.zeros(3, np.float32)
        hi = np.zeros(3, np.float32)
        _check(self._lib.lg_local_bounds(self._h, _fp(lo), _fp(hi)))
        return Box3(tuple(lo.tolist()), tuple(hi.tolist()))

    def build_tree(self, p: ForceParams) -> None:
        cp = _cparams(p)
        _check(self._lib.lg_build_tree(self._h, C.byref(cp)))

    def compute_forces_with(self, p: ForceParams, potential: bool = False, remote=()) -> None:
        """Forces from the own tree (or direct sum) plus other ranks' locally-essential trees."""
        cp = _cparams(p)
        keep = []
        arr = (_CLetTree * max(len(remote), 1))()
        for k, t in enumerate(remote):
            if not isinstance(t, LetTree):
                raise TypeError("remote entries must be LetTree")
            nodes = np.ascontiguousarray(t.nodes, LET_NODE_DTYPE)
            cols = [np.ascontiguousarray(getattr(t, c), np.float32) for c in ("bx", "by", "bz", "bm")]
            keep += [nodes, *cols]
            arr[k] = _CLetTree(nodes.ctypes.data if len(nodes) else None, len(nodes), *(_fp(c) for c in cols),
                               len(cols[0]))
        _check(self._lib.lg_compute_forces_with(self._h, C.byref(cp), int(bool(potential)), arr, len(remote)))

    def export_let(self, lo, hi, p: ForceParams) -> LetTree:
        """The part of this engine's tree any target in the box lo..hi could open."""
        cp = _cparams(p)
        lo = np.ascontiguousarray(lo, np.float32)
        hi = np.ascontiguousarray(hi, np.float32)
        nn, nb = C.c_size_t(), C.c_size_t()
        _check(self._lib.lg_export_let(self._h, _fp(lo), _fp(hi), C.byref(cp), C.byref(nn), C.byref(nb)))
        t = LetTree(np.zeros(nn.value, LET_NODE_DTYPE), *(np.zeros(nb.value, np.float32) for _ in range(4)))
        _check(self._lib.lg_export_let_read(self._h, t.nodes.ctypes.data if nn.value else None, _fp(t.bx),
                                            _fp(t.by), _fp(t.bz), _fp(t.bm)))
        return t

    @staticmethod
    def memory_need(n: int, method: ForceMethod) -> MemoryNeed:
        m = _CMem()
        _check(_lib().lg_memory_need(int(n), int(method), C.byref(m)))
        return MemoryNeed(int(m.device), int(m.host))

    def device_memory(self):
        f = C.c_uint64()
        t = C.c_uint64()
        _check(self._lib.lg_device_memory(self._h, C.byref(f), C.byref(t)))
        return True, int(f.value), int(t.value)

    def body_costs(self):
        n = self.size()
        c = np.zeros(max(n, 1), np.float32)
        valid = C.c_int()
        _check(self._lib.lg_body_costs(self._h, _fp(c), n, C.byref(valid)))
        return bool(valid.value), c[:n]

    # ---- extensions ----
    def accel(self) -> np.ndarray:
        """(4, n) float32: ax, ay, az, phi in the current body order."""
        n = self.size()
        a = np.zeros((4, max(n, 1)), np.float32)
        _check(self._lib.lg_read_accel(self._h, _fp(a[0]), _fp(a[1]), _fp(a[2]), _fp(a[3])))
        return a[:, :n]

    def pos64(self) -> np.ndarray:
        n = self.size()
        p = np.zeros((3, max(n, 1)), np.float64)
        d = [p[k].ctypes.data_as(_d) for k in range(3)]
        _check(self._lib.lg_read_pos64(self._h, *d))
        return p[:, :n]

    def tree_counts(self):
        a, b, c, d = C.c_size_t(), C.c_size_t(), C.c_size_t(), C.c_int()
        _check(self._lib.lg_tree_counts(self._h, C.byref(a), C.byref(b), C.byref(c), C.byref(d)))
        return dict(nodes=int(a.value), leaves=int(b.value), groups=int(c.value), max_depth=int(d.value))

    def tree_keys(self) -> np.ndarray:
        n = self.size()
        k = np.zeros(max(n, 1), np.uint64)
        _check(self._lib.lg_tree_keys(self._h, k.ctypes.data_as(C.POINTER(C.c_uint64)), n))
        return k[:n]

    def tree_nodes(self):
        """Nodes in the reference CPU backend's order: (range (T,4) u32 lo/hi/first/nchild,
        moments (T,11) f32 cx cy cz m qxx qxy qxz qyy qyz qzz rcrit2, geo (T,4) f32)."""
        T = self.tree_counts()["nodes"]
        r = np.zeros((T, 4), np.uint32)
        mo = np.zeros((T, 11), np.float32)
        g = np.zeros((T, 4), np.float32)
        _check(self._lib.lg_tree_nodes(self._h, _up(r), _fp(mo), _fp(g), T))
        return r, mo, g

    def tree_groups(self):
        G = self.tree_counts()["groups"]
        box = np.zeros((G, 6), np.float32)
        lohi = np.zeros((G, 2), np.uint32)
        _check(self._lib.lg_tree_groups(self._h, _fp(box), _up(lohi), G))
        return box, lohi

    def event_record(self, slot: int) -> None:
        _check(self._lib.lg_event_record(self._h, int(slot)))

    def event_elapsed(self, a: int, b: int) -> float:
        ms = C.c_float()
        _check(self._lib.lg_event_elapsed(self._h, int(a), int(b), C.byref(ms)))
        return float(ms.value)

    def synchronize(self) -> None:
        _check(self._lib.lg_synchronize(self._h))

    def flush_l2(self) -> None:
        _check(self._lib.lg_flush_l2(self._h))

    def interaction_split(self):
        """(body pairs, cell terms) of the last force call."""
        a, b = C.c_uint64(), C.c_uint64()
        _check(self._lib.lg_interaction_split(self._h, C.byref(a), C.byref(b)))
        return int(a.value), int(b.value)

    def probe_fp32_peak(self) -> float:
        t = C.c_double()
        _check(self._lib.lg_probe_fp32_peak(self._h, C.byref(t)))
        return float(t.value)

    def probe_wait_timeout(self, polls: int = 4096) -> None:
        """Self-test of failure detection: device waits that are never satisfied give up after
        `polls` polls and the call raises RuntimeError("... device wait timed out ..."); the engine
        stays usable."""
        _check(self._lib.lg_probe_wait_timeout(self._h, int(polls)))

    def adjoint_forward(self, p: ForceParams, dt: float, steps: int, checkpoint_every: int) -> None:
        """Runs `steps` KDK steps from the resident state, keeping adjoint checkpoints."""
        cp = _cparams(p)
        _check(self._lib.lg_adjoint_forward(self._h, C.byref(cp), float(dt), int(steps), int(checkpoint_every)))

    def adjoint_backward(self, target):
        """Loss sum m |x(T) - target|^2 and its gradients with respect to the initial positions,
        velocities and masses, all indexed by body id: (loss, gx (n,3), gv (n,3), gm (n,))."""
        n = self.size()
        t = np.ascontiguousarray(np.asarray(target, np.float64).reshape(n, 3).T)
        out = np.zeros((7, n), np.float64)
        loss = C.c_double()
        ptr = [out[k].ctypes.data_as(_d) for k in range(7)]
        _check(self._lib.lg_adjoint_backward(self._h, t[0].ctypes.data_as(_d), t[1].ctypes.data_as(_d),
                                             t[2].ctypes.data_as(_d), C.byref(loss), *ptr))
        return float(loss.value), out[0:3].T.copy(), out[3:6].T.copy(), out[6].copy()

    def adjoint_backward_seeded(self, dldx):
        """Gradients for a caller's loss of the final positions: dldx (n, 3) = dL/dx(T) by body id.
        Returns (gx (n,3), gv (n,3), gm (n,)) by id; gm excludes explicit mass dependence of L."""
        n = self.size()
        t = np.ascontiguousarray(np.asarray(dldx, np.float64).reshape(n, 3).T)
        out = np.zeros((7, n), np.float64)
        ptr = [out[k].ctypes.data_as(_d) for k in range(7)]
        _check(self._lib.lg_adjoint_backward_seeded(self._h, t[0].ctypes.data_as(_d), t[1].ctypes.data_as(_d),
                                                    t[2].ctypes.data_as(_d), *ptr))
        return out[0:3].T.copy(), out[3:6].T.copy(), out[6].copy()

    def launch_count(self) -> int:
        c = C.c_uint64()
        _check(self._lib.lg_launch_count(self._h, C.byref(c)))
        return int(c.value)


class PinnedBodies:
    """Bodies whose arrays live in page-locked host memory (lg_host_alloc), for transfers at full
    PCIe/C2C bandwidth. Call free() when done."""

    def __init__(self, n: int):
        lib = _lib()
        self._ptr = C.c_void_p()
        _check(lib.lg_host_alloc(max(n, 1) * 32, C.byref(self._ptr)))
        buf = (C.c_char * (max(n, 1) * 32)).from_address(self._ptr.value)
        raw = np.frombuffer(buf, dtype=np.uint8)
        cols = [raw[k * 4 * max(n, 1):(k + 1) * 4 * max(n, 1)] for k in range(8)]
        f = [c.view(np.float32)[:n] for c in cols[:7]]
        self.bodies = Bodies.__new__(Bodies)
        for name, arr in zip(("x", "y", "z", "vx", "vy", "vz", "m"), f):
            setattr(self.bodies, name, arr)
        self.bodies.id = cols[7].view(np.uint32)[:n]

    def free(self):
        if self._ptr:
            _lib().lg_host_free(self._ptr)
            self._ptr = None


def make_cuda_backend(device: int = 0):
    """(backend, "") or (None, why), as make_cuda_backend(device, why) (src/backend.hpp:145)."""
    try:
        return CudaBackend(device), ""
    except UnavailableError as e:
        return None, str(e)
