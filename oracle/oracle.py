"""ctypes access to the CPU oracle libraries.

TEST INFRASTRUCTURE. Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module, as the checker or the timed CPU baseline; the GPU engine never
calls it.

Two libraries share one interface:
  "port"  _build/liboracle.so   C restatement of the reference CPU backend (lettuce_oracle.c)
  "ref"   _ref/libref_cpu.so    the reference's own src/cpu_backend.cpp behind ref_shim.cpp; only
                                where the reference sources were present at build time
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libref_cpu.so")
# The reference's sources: LETTUCE_REF_SRC (its src/), or LETTUCE_REF (a checkout), else the staged
# copy that baseline/stage.py makes (git-ignored).
STAGED_REF_SRC = os.path.join(os.path.dirname(HERE), "baseline", "_ref", "lettuce", "src")


def reference_src() -> str:
    if os.environ.get("LETTUCE_REF_SRC"):
        return os.environ["LETTUCE_REF_SRC"]
    if os.environ.get("LETTUCE_REF"):
        return os.path.join(os.environ["LETTUCE_REF"], "src")
    return STAGED_REF_SRC


NODE_DTYPE = np.dtype([("cx", "<f4"), ("cy", "<f4"), ("cz", "<f4"), ("m", "<f4"), ("qxx", "<f4"), ("qxy", "<f4"),
                       ("qxz", "<f4"), ("qyy", "<f4"), ("qyz", "<f4"), ("qzz", "<f4"), ("rcrit2", "<f4"),
                       ("first", "<u4"), ("nchild", "<u4"), ("lo", "<u4"), ("hi", "<u4")])
GEO_DTYPE = np.dtype([("gx", "<f4"), ("gy", "<f4"), ("gz", "<f4"), ("half", "<f4")])
GROUP_DTYPE = np.dtype([("bx", "<f4"), ("by", "<f4"), ("bz", "<f4"), ("hx", "<f4"), ("hy", "<f4"), ("hz", "<f4"),
                        ("lo", "<u4"), ("hi", "<u4")])
assert NODE_DTYPE.itemsize == 60 and GROUP_DTYPE.itemsize == 32

DIRECT, TREE = 0, 1


def build(ref_src: str | None = None, quiet: bool = True) -> None:
    """Builds the port; also the reference library when its sources are present."""
    out = subprocess.DEVNULL if quiet else None
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True, stdout=out)
    src = ref_src or reference_src()
    if os.path.isfile(os.path.join(src, "cpu_backend.cpp")):
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF_SRC={src}"], check=True, stdout=out)


def available(kind: str) -> bool:
    return os.path.isfile(PORT_SO if kind == "port" else REF_SO)


_libs: dict[str, C.CDLL] = {}

_f = C.POINTER(C.c_float)
_u = C.POINTER(C.c_uint32)
_d = C.POINTER(C.c_double)


def _lib(kind: str) -> C.CDLL:
    if kind in _libs:
        return _libs[kind]
    path = PORT_SO if kind == "port" else REF_SO
    if not os.path.isfile(path):
        raise FileNotFoundError(f"oracle library {path} is not built (oracle.build())")
    lib = C.CDLL(path)
    p = "or_" if kind == "port" else "ref_"
    vp = C.c_void_p
    sig = {
        "create": (vp, [C.c_int]),
        "destroy": (None, [vp]),
        "upload": (None, [vp, C.c_size_t, _f, _f, _f, _f, _f, _f, _f, _u]),
        "size": (C.c_size_t, [vp]),
        "download": (None, [vp, _f, _f, _f, _f, _f, _f, _f, _u]),
        "accel": (None, [vp, _f, _f, _f, _f]),
        "build_tree": (None, [vp, C.c_int, C.c_double]),
        "kick": (None, [vp, C.c_double]),
        "drift": (None, [vp, C.c_double]),
        "diagnostics": (C.c_int, [vp, _d]),
        "exact_potential_energy": (C.c_double, [vp, C.c_double, C.c_double]),
        "times": (C.c_uint64, [vp, _d]),
        "body_costs": (C.c_int, [vp, _f]),
        "num_nodes": (C.c_size_t, [vp]),
        "num_groups": (C.c_size_t, [vp]),
        "num_leaves": (C.c_size_t, [vp]),
        "max_depth": (C.c_int, [vp]),
        "get_nodes": (None, [vp, vp]),
        "get_geo": (None, [vp, vp]),
        "get_groups": (None, [vp, vp]),
        "get_leaves": (None, [vp, _u]),
        "get_keys": (None, [vp, C.POINTER(C.c_uint64)]),
        "get_frame": (None, [vp, _d]),
    }
    if kind == "port":
        sig["threads"] = (C.c_int, [vp])
    else:
        sig["export_let"] = (None, [vp, _f, _f, C.c_int, C.c_double, C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)])
        sig["export_let_read"] = (None, [vp, _f, _f, _f, _f])
        sig["compute_forces_remote"] = (None, [vp, C.c_int, C.c_double, C.c_double, C.c_double, C.c_int, vp,
                                               C.c_size_t, _f, _f, _f, _f, C.c_size_t])
    for name, (res, args) in sig.items():
        fn = getattr(lib, p + name)
        fn.restype = res
        fn.argtypes = args
    cf = getattr(lib, p + "compute_forces")
    cf.restype = None
    cf.argtypes = [vp, C.c_int, C.c_double, C.c_double, C.c_double, C.c_int]
    if kind == "port":
        lib.or_direct_fp64.restype = None
        lib.or_direct_fp64.argtypes = [C.c_size_t, _f, _f, _f, _f, C.c_double, C.c_double, _d, _d, _d, _d, C.c_int]
        lib.or_adjoint_direct_fp64.restype = C.c_double
        lib.or_adjoint_direct_fp64.argtypes = [C.c_size_t, _d, _d, _d, C.c_double, C.c_double, C.c_double, C.c_int,
                                               _d, _d, _d, _d, C.c_int]
        lib.or_loss_direct_fp64.restype = C.c_double
        lib.or_loss_direct_fp64.argtypes = [C.c_size_t, _d, _d, _d, C.c_double, C.c_double, C.c_double, C.c_int,
                                            _d, C.c_int]
        lib.or_frozen_create.restype = vp
        lib.or_frozen_create.argtypes = [C.c_size_t, C.c_int, _u, _u, _u, _u, _f, _u, _f]
        lib.or_frozen_destroy.restype = None
        lib.or_frozen_destroy.argtypes = [vp]
        lib.or_frozen_loss.restype = C.c_double
        lib.or_frozen_loss.argtypes = [vp, _d, _d, _d, C.c_double, C.c_double, C.c_double, _d, C.c_int]
        lib.or_block_direct_fp64.restype = None
        lib.or_block_direct_fp64.argtypes = [C.c_size_t, _d, _d, _d, C.c_double, C.c_double, C.c_double, C.c_int,
                                             C.c_double, C.c_int, C.POINTER(C.c_uint8), C.c_int]
        lib.or_frozen_accel.restype = None
        lib.or_frozen_accel.argtypes = [vp, C.c_int, _d, _d, C.c_double, C.c_double, _d, C.c_int]
    _libs[kind] = lib
    return lib


def _fp(a):
    return a.ctypes.data_as(_f)


def _up(a):
    return a.ctypes.data_as(_u)


def _dp(a):
    return a.ctypes.data_as(_d)


class OracleBackend:
    """The reference CPU backend's interface (src/backend.hpp:89-141) over either library."""

    def __init__(self, kind: str = "port", threads: int = 0):
        self.kind = kind
        self._lib = _lib(kind)
        self._p = "or_" if kind == "port" else "ref_"
        self._h = self._call("create", threads)

    def _call(self, name, *args):
        return getattr(self._lib, self._p + name)(*args)

    def threads(self) -> int:
        """Host threads the backend uses."""
        if self.kind == "port":
            return int(self._call("threads", self._h))
        import os
        return os.cpu_count() or 1

    def close(self):
        if self._h:
            self._call("destroy", self._h)
            self._h = None

    __del__ = close

    def upload(self, b):
        self._call("upload", self._h, len(b), _fp(b.x), _fp(b.y), _fp(b.z), _fp(b.vx), _fp(b.vy), _fp(b.vz),
                   _fp(b.m), _up(b.id))

    def __len__(self):
        return int(self._call("size", self._h))

    def download(self):
        from lettuce_simulate_physics_gb300.bodies import Bodies
        out = Bodies.empty(len(self))
        self._call("download", self._h, _fp(out.x), _fp(out.y), _fp(out.z), _fp(out.vx), _fp(out.vy), _fp(out.vz),
                   _fp(out.m), _up(out.id))
        return out

    def accel(self):
        n = len(self)
        a = np.zeros((4, n), np.float32)
        self._call("accel", self._h, _fp(a[0]), _fp(a[1]), _fp(a[2]), _fp(a[3]))
        return a

    def build_tree(self, method=TREE, theta=0.6):
        self._call("build_tree", self._h, int(method), float(theta))

    def compute_forces(self, method=DIRECT, G=1.0, eps=0.01, theta=0.6, potential=False):
        self._call("compute_forces", self._h, int(method), float(G), float(eps), float(theta), int(bool(potential)))

    def kick(self, dt):
        self._call("kick", self._h, float(dt))

    def drift(self, dt):
        self._call("drift", self._h, float(dt))

    def diagnostics(self):
        out = np.zeros(12)
        has_pe = self._call("diagnostics", self._h, _dp(out))
        keys = ("mass", "ke", "pe", "px", "py", "pz", "lx", "ly", "lz", "cx", "cy", "cz")
        d = dict(zip(keys, out.tolist()))
        d["has_pe"] = bool(has_pe)
        return d

    def exact_potential_energy(self, G, eps):
        return float(self._call("exact_potential_energy", self._h, float(G), float(eps)))

    def times(self):
        out = np.zeros(5)
        inter = self._call("times", self._h, _dp(out))
        return dict(force_ms=out[0], sort_ms=out[1], build_ms=out[2], walk_ms=out[3], step_ms=out[4],
                    interactions=int(inter))

    def body_costs(self):
        c = np.zeros(len(self), np.float32)
        return c if self._call("body_costs", self._h, _fp(c)) else None

    # ---- locally-essential trees (reference library only) ----
    def export_let(self, lo, hi, method=TREE, theta=0.6):
        """(nodes: 60-byte records as a uint8 (k, 60) array, bx, by, bz, bm) of the reference's export."""
        lo = np.ascontiguousarray(lo, np.float32)
        hi = np.ascontiguousarray(hi, np.float32)
        nn, nb = C.c_size_t(), C.c_size_t()
        self._call("export_let", self._h, _fp(lo), _fp(hi), int(method), float(theta), C.byref(nn), C.byref(nb))
        nodes = np.zeros((nn.value, 60), np.uint8)
        cols = [np.zeros(nb.value, np.float32) for _ in range(4)]
        self._lib.ref_export_let_read(nodes.ctypes.data, *(_fp(c) for c in cols))
        return nodes, cols

    def compute_forces_remote(self, method, G, eps, theta, potential, nodes, cols):
        nodes = np.ascontiguousarray(nodes, np.uint8)
        cols = [np.ascontiguousarray(c, np.float32) for c in cols]
        self._call("compute_forces_remote", self._h, int(method), float(G), float(eps), float(theta),
                   int(bool(potential)), nodes.ctypes.data if len(nodes) else None, len(nodes),
                   *(_fp(c) for c in cols), len(cols[0]))

    # ---- tree introspection ----
    def keys(self):
        k = np.zeros(len(self), np.uint64)
        self._call("get_keys", self._h, k.ctypes.data_as(C.POINTER(C.c_uint64)))
        return k

    def frame(self):
        f = np.zeros(4)
        self._call("get_frame", self._h, _dp(f))
        return f

    def nodes(self):
        out = np.zeros(int(self._call("num_nodes", self._h)), NODE_DTYPE)
        self._call("get_nodes", self._h, out.ctypes.data_as(C.c_void_p))
        return out

    def geo(self):
        out = np.zeros(int(self._call("num_nodes", self._h)), GEO_DTYPE)
        self._call("get_geo", self._h, out.ctypes.data_as(C.c_void_p))
        return out

    def groups(self):
        out = np.zeros(int(self._call("num_groups", self._h)), GROUP_DTYPE)
        self._call("get_groups", self._h, out.ctypes.data_as(C.c_void_p))
        return out

    def leaves(self):
        out = np.zeros(int(self._call("num_leaves", self._h)), np.uint32)
        self._call("get_leaves", self._h, _up(out))
        return out

    def max_depth(self):
        return int(self._call("max_depth", self._h))


def direct_fp64(b, G=1.0, eps=0.01, threads=0):
    """FP64 brute-force accelerations and potential, in b's order: array (4, n)."""
    lib = _lib("port")
    n = len(b)
    out = np.zeros((4, n), np.float64)
    lib.or_direct_fp64(n, _fp(b.x), _fp(b.y), _fp(b.z), _fp(b.m), float(G), float(eps), _dp(out[0]), _dp(out[1]),
                       _dp(out[2]), _dp(out[3]), int(threads))
    return out


def adjoint_direct_fp64(x0, v0, m, G, eps, dt, steps, xstar, threads=0):
    """FP64 reference adjoint of the direct-sum KDK leapfrog: (loss, gx, gv, gm)."""
    lib = _lib("port")
    x0 = np.ascontiguousarray(x0, np.float64)
    v0 = np.ascontiguousarray(v0, np.float64)
    m = np.ascontiguousarray(m, np.float64)
    xstar = np.ascontiguousarray(xstar, np.float64)
    n = m.shape[0]
    gx = np.zeros((n, 3))
    gv = np.zeros((n, 3))
    gm = np.zeros(n)
    L = lib.or_adjoint_direct_fp64(n, _dp(x0), _dp(v0), _dp(m), float(G), float(eps), float(dt), int(steps),
                                   _dp(xstar), _dp(gx), _dp(gv), _dp(gm), int(threads))
    return L, gx, gv, gm


def loss_direct_fp64(x0, v0, m, G, eps, dt, steps, xstar, threads=0):
    lib = _lib("port")
    x0 = np.ascontiguousarray(x0, np.float64)
    v0 = np.ascontiguousarray(v0, np.float64)
    m = np.ascontiguousarray(m, np.float64)
    xstar = np.ascontiguousarray(xstar, np.float64)
    return lib.or_loss_direct_fp64(m.shape[0], _dp(x0), _dp(v0), _dp(m), float(G), float(eps), float(dt),
                                   int(steps), _dp(xstar), int(threads))


def block_direct_fp64(x0, v0, m, G, eps, dt, K, eta, steps, threads=0):
    """FP64 block time steps with direct forces: (x (n, 3), v (n, 3), levels (n,))."""
    lib = _lib("port")
    x = np.ascontiguousarray(x0, np.float64).copy()
    v = np.ascontiguousarray(v0, np.float64).copy()
    m = np.ascontiguousarray(m, np.float64)
    lv = np.zeros(len(m), np.uint8)
    lib.or_block_direct_fp64(len(m), _dp(x), _dp(v), _dp(m), float(G), float(eps), float(dt), int(K), float(eta),
                             int(steps), lv.ctypes.data_as(C.POINTER(C.c_uint8)), int(threads))
    return x, v, lv


def render_ref(b, width, height, view="xy", extent=0.0, color=0):
    """The reference's render_image (src/render.cpp) through oracle/_ref: ((h, w, 3) uint8, extent)."""
    lib = _lib("ref")
    fn = lib.ref_render
    fn.restype = None
    fn.argtypes = [C.c_size_t, _f, _f, _f, _f, _f, _f, _f, C.c_int, C.c_int, C.c_char_p, C.c_double, C.c_int,
                   C.POINTER(C.c_ubyte), _d]
    rgb = np.zeros((int(height), int(width), 3), np.uint8)
    ext = C.c_double()
    fn(len(b), _fp(b.x), _fp(b.y), _fp(b.z), _fp(b.vx), _fp(b.vy), _fp(b.vz), _fp(b.m), int(width), int(height),
       view.encode(), float(extent), int(color), rgb.ctypes.data_as(C.POINTER(C.c_ubyte)), C.byref(ext))
    return rgb, float(ext.value)


class FrozenTree:
    """FP64 tree forces over frozen interaction lists for a trajectory (or_frozen_*): `calls` is a
    list, one per force call s = 0 .. steps-1, of dicts with the engine's tree after that call:
    perm (sorted position -> id), range4 (nn, 4), moments11 (nn, 11: cx cy cz m q.. rcrit2),
    glohi (ng, 2), box6 (ng, 6). loss(x0, v0, m, xstar) runs the KDK steps in FP64 with those lists
    and cell moments recomputed from the positions."""

    def __init__(self, n, calls):
        lib = _lib("port")
        self._lib = lib
        self.n = int(n)
        self.steps = len(calls)
        nn = np.array([len(c["range4"]) for c in calls], np.uint32)
        ng = np.array([len(c["glohi"]) for c in calls], np.uint32)
        perm = np.ascontiguousarray(np.concatenate([np.asarray(c["perm"], np.uint32) for c in calls]))
        r4 = np.ascontiguousarray(np.concatenate([np.asarray(c["range4"], np.uint32).reshape(-1) for c in calls]))
        crc = np.ascontiguousarray(np.concatenate(
            [np.asarray(c["moments11"], np.float32)[:, [0, 1, 2, 10]].reshape(-1) for c in calls]))
        gl = np.ascontiguousarray(np.concatenate([np.asarray(c["glohi"], np.uint32).reshape(-1) for c in calls]))
        gb = np.ascontiguousarray(np.concatenate([np.asarray(c["box6"], np.float32).reshape(-1) for c in calls]))
        self._h = lib.or_frozen_create(self.n, self.steps, _up(nn), _up(ng), _up(perm), _up(r4), _fp(crc), _up(gl),
                                       _fp(gb))

    def loss(self, x0, v0, m, G, eps, dt, xstar, threads=0):
        x0 = np.ascontiguousarray(x0, np.float64)
        v0 = np.ascontiguousarray(v0, np.float64)
        m = np.ascontiguousarray(m, np.float64)
        xstar = np.ascontiguousarray(xstar, np.float64)
        return self._lib.or_frozen_loss(self._h, _dp(x0), _dp(v0), _dp(m), float(G), float(eps), float(dt),
                                        _dp(xstar), int(threads))

    def accel(self, s, x, m, G, eps, threads=0):
        """(n, 3) FP64 accelerations of force call s at positions x (n, 3) by id."""
        x = np.ascontiguousarray(x, np.float64)
        m = np.ascontiguousarray(m, np.float64)
        a = np.zeros((self.n, 3))
        self._lib.or_frozen_accel(self._h, int(s), _dp(x), _dp(m), float(G), float(eps), _dp(a), int(threads))
        return a

    def close(self):
        if self._h:
            self._lib.or_frozen_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


if __name__ == "__main__":
    build(quiet=False)
    sys.exit(0)
