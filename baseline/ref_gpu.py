"""Times the reference's own CUDA backend (src/cuda_backend.cu, built unmodified for sm_103a by
baseline/Makefile) on the same GPU and the same bodies as the engine, through the reference's public
Backend interface. Prints one JSON line.

  python baseline/ref_gpu.py [--workload disk1m] [--steps 20] [--warmup 3]

A step is the reference's lettuce-bench step (src/bench.cpp:174-189): kick(dt/2), drift(dt),
compute_forces, kick(dt/2), then times(), which waits for the device; ms/step is the wall clock
over the timed steps. The reference's own force/sort/build/walk split (its CUDA events) is reported
beside it, and its force error against an FP64 direct sum on sampled bodies (accelerations read
through kick(1) from zero velocity, the reference tests' accessor, tests/test_cuda_backend.cpp:93-112).
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)
LIB = os.path.join(HERE, "_ref", "build", "libref_cuda.so")

_f = C.POINTER(C.c_float)
_u = C.POINTER(C.c_uint32)


def available() -> bool:
    return os.path.isfile(LIB)


class RefCuda:
    def __init__(self, device: int = 0):
        lib = C.CDLL(LIB)
        vp = C.c_void_p
        for name, res, args in (
                ("refgpu_error", C.c_char_p, []),
                ("refgpu_create", vp, [C.c_int]),
                ("refgpu_destroy", None, [vp]),
                ("refgpu_name", C.c_int, [vp, C.c_char_p, C.c_size_t]),
                ("refgpu_upload", C.c_int, [vp, C.c_size_t, _f, _f, _f, _f, _f, _f, _f, _u]),
                ("refgpu_download", C.c_int, [vp, _f, _f, _f, _f, _f, _f, _f, _u]),
                ("refgpu_compute_forces", C.c_int, [vp, C.c_int, C.c_double, C.c_double, C.c_double, C.c_int]),
                ("refgpu_kick", C.c_int, [vp, C.c_double]),
                ("refgpu_drift", C.c_int, [vp, C.c_double]),
                ("refgpu_times", C.c_int, [vp, C.POINTER(C.c_double), C.POINTER(C.c_uint64)])):
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        self.lib = lib
        self.h = lib.refgpu_create(device)
        if not self.h:
            raise RuntimeError(f"reference CUDA backend unavailable: {lib.refgpu_error().decode()}")
        self.n = 0

    def _ok(self, rc):
        if rc != 0:
            raise RuntimeError(self.lib.refgpu_error().decode())

    def name(self) -> str:
        buf = C.create_string_buffer(256)
        self._ok(self.lib.refgpu_name(self.h, buf, 256))
        return buf.value.decode()

    def upload(self, b):
        arrs = [np.ascontiguousarray(getattr(b, f), np.float32) for f in ("x", "y", "z", "vx", "vy", "vz", "m")]
        ids = np.ascontiguousarray(b.id, np.uint32)
        self.n = len(ids)
        self._ok(self.lib.refgpu_upload(self.h, self.n, *[a.ctypes.data_as(_f) for a in arrs],
                                        ids.ctypes.data_as(_u)))

    def download(self):
        out = [np.empty(self.n, np.float32) for _ in range(7)]
        ids = np.empty(self.n, np.uint32)
        self._ok(self.lib.refgpu_download(self.h, *[a.ctypes.data_as(_f) for a in out], ids.ctypes.data_as(_u)))
        return out, ids

    def compute_forces(self, method, G, eps, theta, pot=False):
        self._ok(self.lib.refgpu_compute_forces(self.h, 1 if method == "tree" else 0, G, eps, theta, int(pot)))

    def kick(self, dt):
        self._ok(self.lib.refgpu_kick(self.h, dt))

    def drift(self, dt):
        self._ok(self.lib.refgpu_drift(self.h, dt))

    def times(self):
        out = (C.c_double * 5)()
        inter = C.c_uint64()
        self._ok(self.lib.refgpu_times(self.h, out, C.byref(inter)))
        return dict(force_ms=out[0], sort_ms=out[1], build_ms=out[2], walk_ms=out[3], step_ms=out[4],
                    interactions=int(inter.value))

    def close(self):
        if self.h:
            self.lib.refgpu_destroy(self.h)
            self.h = None


def run(workload: str, steps: int, warmup: int, device: int = 0) -> dict:
    import bench
    w = bench.WORKLOADS[workload]
    b = bench.make_bodies(w)
    n = len(b)
    G, eps, theta, dt, method = 1.0, w["eps"], w["theta"], w["dt"], w["method"]
    be = RefCuda(device)
    name = be.name()
    # Accuracy: accelerations through kick(1) from zero velocity.
    z = b.copy()
    z.vx[:] = 0
    z.vy[:] = 0
    z.vz[:] = 0
    be.upload(z)
    be.compute_forces(method, G, eps, theta)
    be.kick(1.0)
    (_, _, _, vx, vy, vz, _), ids = be.download()
    pos = np.stack([b.x, b.y, b.z], 1).astype(np.float64)
    acc = np.zeros((n, 3))
    acc[ids] = np.stack([vx, vy, vz], 1)
    med, mx = bench.fp64_direct_error(pos, b.m.astype(np.float64), acc, eps, count=256)
    # Timing: the lettuce-bench step.
    be.upload(b)
    be.compute_forces(method, G, eps, theta)

    def step():
        be.kick(0.5 * dt)
        be.drift(dt)
        be.compute_forces(method, G, eps, theta)
        be.kick(0.5 * dt)
        return be.times()

    for _ in range(max(warmup, 1)):
        step()
    wall, force, sort, build, walk, inter = [], [], [], [], [], []
    for _ in range(steps):
        t0 = time.perf_counter()
        t = step()
        wall.append((time.perf_counter() - t0) * 1e3)
        force.append(t["force_ms"])
        sort.append(t["sort_ms"])
        build.append(t["build_ms"])
        walk.append(t["walk_ms"])
        inter.append(t["interactions"])
    be.close()
    mean = statistics.fmean
    return {"impl": "reference-cuda", "device": name, "workload": workload, "n": n, "method": method,
            "theta": theta, "steps": steps, "warmup": max(warmup, 1),
            "ms_per_step_wall": round(mean(wall), 4), "median_ms_per_step_wall": round(statistics.median(wall), 4),
            "phases_ms": {"force": round(mean(force), 4), "sort": round(mean(sort), 4),
                          "build": round(mean(build), 4), "walk": round(mean(walk), 4)},
            "interactions_per_step": int(mean(inter)),
            "ginteractions_per_s": round(mean(inter) / (mean(force) * 1e-3) / 1e9, 2),
            "force_error_vs_fp64": {"median": med, "max": mx, "sample_bodies": 256},
            "step": "kick(dt/2), drift(dt), compute_forces, kick(dt/2), times() (the reference's lettuce-bench step)"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="disk1m")
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--device", type=int, default=0)
    a = ap.parse_args()
    if not available():
        print(json.dumps({"impl": "reference-cuda", "unavailable": f"{LIB} not built (make -C baseline)"}))
        return 0
    print(json.dumps(run(a.workload, a.steps, a.warmup, a.device)), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
