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


def deep_radial(n, seed, decades):
    """n equal-mass bodies at radii log-uniform over `decades` decades below 1, isotropic, at rest:
    every octave of radius holds bodies, so the octree around the centre branches fully for dozens
    of levels (past MAX_LEVEL into key restarts) and its traversal stacks grow deep."""
    from lettuce_simulate_physics_gb300.bodies import Bodies
    rng = np.random.Generator(np.random.PCG64(seed))
    r = 10.0 ** rng.uniform(-decades, 0.0, n)
    u = rng.normal(size=(n, 3))
    p = u / np.linalg.norm(u, axis=1)[:, None] * r[:, None]
    z = np.zeros(n)
    return Bodies(x=p[:, 0].copy(), y=p[:, 1].copy(), z=p[:, 2].copy(), vx=z.copy(), vy=z.copy(), vz=z.copy(),
                  m=np.full(n, 1.0 / n), id=np.arange(n, dtype=np.uint32))


def traversal_stack_depth(port, groups):
    """The largest number of child-block entries the warp-cooperative traversal holds on its stack
    for each of the given groups of the oracle's tree (its last tree call): the engine's step order
    restated (the top entries give the next 32 nodes, the first taken first, a block partly taken
    keeps its tail on top; every node the group opens and that has children pushes one entry, in
    node order). The opening test is the walk's FP32 box distance against rcrit2."""
    nd, gr = port.nodes(), port.groups()
    com = np.stack([nd["cx"], nd["cy"], nd["cz"]], 1).astype(np.float32)
    rc2 = np.asarray(nd["rcrit2"], np.float32)
    lo, hi = nd["lo"].astype(np.int64), nd["hi"].astype(np.int64)
    first, nch = nd["first"].astype(np.int64), nd["nchild"].astype(np.int64)
    out = []
    for g in groups:
        G = gr[g]
        bc = np.array([G["bx"], G["by"], G["bz"]], np.float32)
        bh = np.array([G["hx"], G["hy"], G["hz"]], np.float32)
        glo, ghi = int(G["lo"]), int(G["hi"])
        stack, deepest = [(0, 1)], 1
        while stack:
            nodes = []
            while stack and len(nodes) < 32:
                f, c = stack.pop()
                t = min(c, 32 - len(nodes))
                nodes.extend(range(f, f + t))
                if t < c:
                    stack.append((f + t, c - t))
            nodes = np.array(nodes)
            d = np.maximum(np.abs(com[nodes] - bc) - bh, np.float32(0))
            d2 = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]
            contains = (lo[nodes] <= glo) & (ghi <= hi[nodes])
            opened = (contains | (d2 < rc2[nodes])) & (nch[nodes] > 0)
            stack.extend((int(first[k]), int(nch[k])) for k in nodes[opened])
            deepest = max(deepest, len(stack))
        out.append(deepest)
    return np.array(out)
