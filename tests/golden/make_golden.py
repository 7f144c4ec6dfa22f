"""Generates the golden vectors in this directory from the reference's own CPU backend.

Run here, where the reference sources are present:  python tests/golden/make_golden.py [prefix ...]
(with prefixes, only the fixtures whose names start with one of them are written).
It builds oracle/_ref/libref_cpu.so (the reference's src/cpu_backend.cpp, compiled unmodified by
oracle/Makefile) and records, for seeded inputs, what the reference computes: Morton keys, the
sort permutation, the octree (nodes, cells, groups, leaves), direct and tree accelerations and
potentials, interaction counts, per-body costs, diagnostics and the exact potential energy. The
inputs are stored with the outputs, so the fixtures do not depend on the generator's RNG stream.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from lettuce_simulate_physics_gb300 import scenarios as S  # noqa: E402
from lettuce_simulate_physics_gb300.bodies import Bodies  # noqa: E402
from oracle import oracle as O  # noqa: E402


def _bodies_fields(prefix, b):
    return {f"{prefix}{f}": getattr(b, f) for f in ("x", "y", "z", "vx", "vy", "vz", "m", "id")}


def _zero_v(b):
    b = b.copy()
    b.vx[:] = 0
    b.vy[:] = 0
    b.vz[:] = 0
    return b


def force_case(b, method, G, eps, theta, potential):
    be = O.OracleBackend("ref", 0)
    be.upload(_zero_v(b))
    be.compute_forces(method, G, eps, theta, potential)
    out = {}
    t = be.times()
    out["interactions"] = np.uint64(t["interactions"])
    d = be.diagnostics()
    out["pe"] = np.float64(d["pe"])
    out["has_pe"] = np.bool_(d["has_pe"])
    dn = be.download()
    out["order_id"] = dn.id
    acc = be.accel()
    out["acc"] = acc
    c = be.body_costs()
    out["costs"] = c if c is not None else np.zeros(0, np.float32)
    if method == O.TREE:
        out["keys"] = be.keys()
        out["frame"] = be.frame()
        out["nodes"] = be.nodes()
        out["geo"] = be.geo()
        out["groups"] = be.groups()
        out["leaves"] = be.leaves()
        out["max_depth"] = np.int32(be.max_depth())
        out["sorted_x"] = dn.x
        out["sorted_y"] = dn.y
        out["sorted_z"] = dn.z
    be.close()
    return out


ONLY: list[str] = []


def save(name, inputs, params, **cases):
    if ONLY and not any(name.startswith(o) for o in ONLY):
        return
    rec = _bodies_fields("in_", inputs)
    for k, v in params.items():
        rec[f"param_{k}"] = np.asarray(v)
    for cname, c in cases.items():
        for k, v in c.items():
            rec[f"{cname}__{k}"] = v
    path = os.path.join(HERE, f"{name}.npz")
    np.savez_compressed(path, **rec)
    print(f"{path}: {os.path.getsize(path) / 1024:.0f} KiB")


def main():
    ONLY.extend(sys.argv[1:])
    O.build(quiet=False)
    G = 1.0
    # Direct, Plummer 4096 (tests/test_cuda_backend.cpp:180-198 shape).
    b = S.plummer(4096, 1, cut=20)
    save("direct_plummer4096", b, dict(G=G, eps=0.01),
         nopot=force_case(b, O.DIRECT, G, 0.01, 0.6, False), pot=force_case(b, O.DIRECT, G, 0.01, 0.6, True))
    # Direct at the benchmark's direct workload: Plummer N = 16384, seed 1, r < 10a, eps 0.01.
    b = S.plummer(16384, 1, cut=10)
    save("direct_plummer16384", b, dict(G=G, eps=0.01), pot=force_case(b, O.DIRECT, G, 0.01, 0.6, True))
    # Tree, Plummer 8192, theta 0.6 and 0.
    b = S.plummer(8192, 3, cut=20)
    save("tree_plummer8192", b, dict(G=G, eps=0.01),
         t06=force_case(b, O.TREE, G, 0.01, 0.6, True), t03=force_case(b, O.TREE, G, 0.01, 0.3, False),
         t00=force_case(b, O.TREE, G, 0.01, 0.0, True))
    # Tree, exponential disk 8192 (the headline workload's recipe at small N).
    b = S.disk(8192, 7)
    save("tree_disk8192", b, dict(G=G, eps=0.005), t06=force_case(b, O.TREE, G, 0.005, 0.6, True))
    # Coincident bodies and a clump within 1e-7 (tests/test_cuda_backend.cpp:223-256 shape).
    b = S.cube(300, 7)
    b.x[:150] = 0.25; b.y[:150] = -0.5; b.z[:150] = 0.125
    k = np.arange(40, dtype=np.float32)
    b.x[150:190] = np.float32(-0.3) + np.float32(1e-7) * k; b.y[150:190] = 0.1; b.z[150:190] = 0.2
    save("tree_coincident300", b, dict(G=G, eps=0.05),
         t00=force_case(b, O.TREE, G, 0.05, 0.0, True), t06=force_case(b, O.TREE, G, 0.05, 0.6, True))
    # 200 coincident in a cube of 3000 (tests/test_cuda_backend.cpp:463-485 shape).
    b = S.cube(3000, 9)
    b.x[:200] = 0.25; b.y[:200] = -0.5; b.z[:200] = 0.125
    save("tree_dup3000", b, dict(G=G, eps=0.05), t00=force_case(b, O.TREE, G, 0.05, 0.0, True),
         t06=force_case(b, O.TREE, G, 0.05, 0.6, True))
    # Far escaper: key restarts (tests/test_cuda_backend.cpp:489-538 shape).
    base = S.plummer(5000, 10, cut=20)
    esc = Bodies.from_arrays(np.array([[1e8, 0, 0]]), np.zeros((1, 3)), np.array([base.m[0]], np.float64))
    b = base.append(esc)
    save("tree_escaper5001", b, dict(G=G, eps=0.01), t06=force_case(b, O.TREE, G, 0.01, 0.6, True),
         t00=force_case(b, O.TREE, G, 0.01, 0.0, False))
    # Escaper plus coincident bodies: nested key restarts end in a coincident leaf (:540-574 shape).
    b = S.cube(3000, 11)
    b.x[:100] = 0.25; b.y[:100] = -0.5; b.z[:100] = 0.125
    b = b.append(Bodies.from_arrays(np.array([[1e8, 0, 0]]), np.zeros((1, 3)), np.array([b.m[0]], np.float64)))
    save("tree_escaper_dup3001", b, dict(G=G, eps=0.05), t00=force_case(b, O.TREE, G, 0.05, 0.0, True),
         t06=force_case(b, O.TREE, G, 0.05, 0.6, True))
    # Radii log-uniform over 34 decades (down to 1e-34): runs of identical keys are re-keyed again
    # and again (src/cpu_backend.cpp:536-544), a 113-level tree with five key frames.
    rng = np.random.Generator(np.random.PCG64(6))
    n = 10000
    u = rng.normal(size=(n, 3))
    p = u / np.linalg.norm(u, axis=1)[:, None] * (10.0 ** rng.uniform(-34, 0, n))[:, None]
    b = Bodies.from_arrays(p, np.zeros((n, 3)), np.full(n, 1.0 / n))
    save("tree_deep10000", b, dict(G=G, eps=0.01), t06=force_case(b, O.TREE, G, 0.01, 0.6, True),
         t00=force_case(b, O.TREE, G, 0.01, 0.0, False))
    # Small and odd N, direct and tree(theta=0) (:200-221 shape).
    for n in (1, 2, 3, 31, 32, 33, 64, 255, 257, 1000, 1023):
        b = S.cube(n, 100 + n)
        save(f"small_n{n}", b, dict(G=G, eps=0.05), direct=force_case(b, O.DIRECT, G, 0.05, 0.0, True),
             tree=force_case(b, O.TREE, G, 0.05, 0.0, True))
    # Locally-essential trees (tests/test_cuda_let.cpp shapes): Plummer 8000 split at x = 0; the
    # x >= 0 half exports for the x < 0 half's box (tree theta 0.6, and direct); the x < 0 half
    # receives it (its own forces plus the remote tree).
    b = S.plummer(8000, 17, cut=20)
    left = b.x < 0
    h0, h1 = b.subset(left), b.subset(~left)
    lo = np.array([h0.x.min(), h0.y.min(), h0.z.min()], np.float32)
    hi = np.array([h0.x.max(), h0.y.max(), h0.z.max()], np.float32)
    cases = {}
    for cname, method in (("tree", O.TREE), ("direct", O.DIRECT)):
        ex = O.OracleBackend("ref", 0)
        ex.upload(h1)
        ex.build_tree(method, 0.6)
        nodes, cols = ex.export_let(lo, hi, method, 0.6)
        ex.close()
        rx = O.OracleBackend("ref", 0)
        rx.upload(_zero_v(h0))
        rx.build_tree(method, 0.6)
        rx.compute_forces_remote(method, G, 0.01, 0.6, True, nodes, cols)
        dn = rx.download()
        c = rx.body_costs()
        cases[cname] = dict(let_nodes=nodes, let_bx=cols[0], let_by=cols[1], let_bz=cols[2], let_bm=cols[3],
                            order_id=dn.id, acc=rx.accel(), interactions=np.uint64(rx.times()["interactions"]),
                            costs=c if c is not None else np.zeros(0, np.float32))
        rx.close()
    save("let_plummer8000", h0, dict(G=G, eps=0.01, theta=0.6, box_lo=lo, box_hi=hi),
         exporter=_bodies_fields("", h1), **cases)
    # Density renders (src/render.cpp render_image): a disk with its rotation velocities and a
    # Plummer sphere, several views, fitted and fixed extents, density and speed colouring.
    for name, b in (("render_disk20000", S.disk(20000, 5)), ("render_plummer5000", S.plummer(5000, 6, cut=20))):
        cases = {}
        for cname, (w, h, view, ext, color) in {"xy": (256, 256, "xy", 0.0, 0), "tilt": (200, 160, "30,60", 0.0, 1),
                                                 "xz": (128, 128, "xz", 3.0, 0)}.items():
            rgb, used = O.render_ref(b, w, h, view, ext, color)
            cases[cname] = dict(rgb=rgb, extent=np.float64(used), width=np.int32(w), height=np.int32(h),
                                view=np.array(view), extent_in=np.float64(ext), color=np.int32(color))
        save(name, b, dict(G=G), **cases)
    # KDK step sequence with diagnostics (:290-343 shape): force, kick, drift, force, kick.
    b = S.plummer(2000, 4, cut=20)
    be = O.OracleBackend("ref", 0)
    be.upload(b)
    be.compute_forces(O.DIRECT, G, 0.01, 0.6, True)
    be.kick(0.01)
    be.drift(0.01)
    be.compute_forces(O.DIRECT, G, 0.01, 0.6, True)
    be.kick(0.01)
    d = be.diagnostics()
    dn = be.download()
    epe = be.exact_potential_energy(G, 0.01)
    diag = np.array([d[k] for k in ("mass", "ke", "pe", "px", "py", "pz", "lx", "ly", "lz", "cx", "cy", "cz")])
    save("kdk_plummer2000", b, dict(G=G, eps=0.01, dt=0.01),
         out=dict(diag=diag, exact_pe=np.float64(epe), **_bodies_fields("", dn)))


if __name__ == "__main__":
    main()
