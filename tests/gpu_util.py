"""Shared helpers of the GPU tests: the reference test accessor and error measures."""
from __future__ import annotations

import numpy as np

import lettuce_simulate_physics_gb300 as L


def params(method, eps, theta=0.6, G=1.0):
    return L.ForceParams(G=G, eps=eps, theta=theta, method=L.ForceMethod(method))


def zero_v(b):
    b = b.copy()
    b.vx[:] = 0
    b.vy[:] = 0
    b.vz[:] = 0
    return b


class Got:
    pass


def accel(be, b, p, potential):
    """The reference's test accessor (tests/test_cuda_backend.cpp:93-112): upload with v = 0,
    compute, read times and diagnostics, kick(1), download and read v as a, indexed by id."""
    be.upload(zero_v(b))
    be.compute_forces(p, potential)
    g = Got()
    g.times = be.times()
    g.diag = be.diagnostics()
    be.kick(1.0)
    out = be.download()
    a = np.zeros((3, len(out)), np.float64)
    a[0, out.id] = out.vx
    a[1, out.id] = out.vy
    a[2, out.id] = out.vz
    g.a = a
    g.out = out
    return g


def rel_rms(a, ref):
    num = float(((np.asarray(a, np.float64) - ref) ** 2).sum())
    den = float((np.asarray(ref, np.float64) ** 2).sum())
    return (num / den) ** 0.5 if den > 0 else num ** 0.5


def per_body_rel(a, ref):
    """|a_i - ref_i| / |ref_i| for (3, n) arrays."""
    a = np.asarray(a, np.float64)
    d = np.sqrt(((a - ref) ** 2).sum(0))
    r = np.sqrt((np.asarray(ref, np.float64) ** 2).sum(0))
    return d / np.where(r > 0, r, 1.0)


def by_id(ids, a):
    out = np.zeros_like(np.asarray(a))
    out[..., ids] = a
    return out
