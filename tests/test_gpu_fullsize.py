"""Parity at the sizes the benchmark workloads are quoted on.

- Tree, N = 1e6 exponential disk (the benchmark's disk1m input, theta 0.6, eps 0.005): against the
  live reference CPU backend (oracle/_ref, the reference's src/cpu_backend.cpp compiled from its
  sources; the C restatement where that library is absent) on the same uploaded bodies. Morton
  keys, sort permutation, node arrays, cell geometry, all ten moments, groups, leaf count, depth,
  rcrit2, interaction counts and per-body costs bit for bit; accelerations within 1e-5 relative rms
  and per-body median 1e-5 of the reference's (same lists; FP32 summation order and rsqrt differ).
- Direct, N = 16384 Plummer (seed 1, r < 10a, eps 0.01; the benchmark's plummer16k input): against
  the reference's own direct forces (golden direct_plummer16384, tests/golden/make_golden.py) and
  the FP64 direct sum: relative rms 1e-5, every body within 1e-4, interactions N(N-1).
- Adjoint, N = 65536 Plummer (seed 2, eps 0.01, dt 1e-3, checkpoints every 32): the gradient along
  a seeded random direction of (x0, v0) against an FP64 central difference (h = 1e-5) of the FP64
  oracle loss, over 34 steps (two checkpoint segments). The FP64 loss costs about 1 s per step at
  this N on 16 host cores (measured on a GB300 host: 72 s for the two 34-step losses), so the
  benchmark's 1000 steps with 64 per-component differences (about 36 hours) are out of reach here;
  the directional form checks the whole gradient at once. Stated tolerance: 1e-4 relative (FP32
  pair arithmetic in the forward and the VJP; measured 3.0e-5).
"""
import numpy as np
import pytest

import lettuce_simulate_physics_gb300 as L
from golden_io import Golden, by_id as g_by_id
from gpu_util import accel, by_id, params, per_body_rel, rel_rms, zero_v
from lettuce_simulate_physics_gb300 import scenarios as S
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def be():
    from lettuce_simulate_physics_gb300 import build as B
    B.build()
    be, why = L.make_cuda_backend(0)
    if be is None:
        pytest.fail(f"no usable device: {why}")
    yield be
    be.close()


def test_disk1m_tree_bit_exact_vs_live_reference(be):
    kind = "ref" if O.available("ref") else "port"
    b = zero_v(S.disk(1_000_000, 1))
    n = len(b)
    p = params(1, 0.005, 0.6)
    cpu = O.OracleBackend(kind, 0)
    cpu.upload(b)
    cpu.compute_forces(O.TREE, 1.0, 0.005, 0.6, False)
    be.upload(b)
    be.compute_forces(p, False)
    assert np.array_equal(be.tree_keys(), cpu.keys()), "Morton keys"
    assert np.array_equal(be.download().id, cpu.download().id), "sort permutation"
    rng, mom, geo = be.tree_nodes()
    rn = cpu.nodes()
    assert len(rng) == len(rn), "node count"
    for k, f in enumerate(("lo", "hi", "first", "nchild")):
        assert np.array_equal(rng[:, k], rn[f]), f
    rg = cpu.geo()
    for k, f in enumerate(("gx", "gy", "gz", "half")):
        assert np.array_equal(geo[:, k], rg[f]), f
    for k, f in enumerate(("cx", "cy", "cz", "m", "qxx", "qxy", "qxz", "qyy", "qyz", "qzz")):
        assert np.array_equal(mom[:, k], rn[f]), f
    assert np.array_equal(mom[:, 10], rn["rcrit2"]), "rcrit2"
    box, lohi = be.tree_groups()
    cg = cpu.groups()
    assert np.array_equal(lohi[:, 0], cg["lo"]) and np.array_equal(lohi[:, 1], cg["hi"]), "groups"
    for k, f in enumerate(("bx", "by", "bz", "hx", "hy", "hz")):
        assert np.array_equal(box[:, k], cg[f]), f
    cnt = be.tree_counts()
    assert cnt["leaves"] == len(cpu.leaves())
    assert cnt["max_depth"] == cpu.max_depth()
    # The reference counts each body's own list entry; this engine does not.
    ti = cpu.times()["interactions"]
    assert be.times().interactions == ti - n
    ok, cost = be.body_costs()
    assert ok and np.array_equal(cost, cpu.body_costs() - 1), "per-body costs"
    a, ra = be.accel()[:3], cpu.accel()[:3]
    e = rel_rms(a, ra)
    med = float(np.median(per_body_rel(a, ra)))
    print(f"disk1m vs {kind}: {len(rn)} nodes, {len(cg)} groups, {ti} interactions; "
          f"acc rel rms {e:.3g}, per-body median {med:.3g}")
    assert e <= 1e-5 and med <= 1e-5
    cpu.close()


def test_collision16m_tree_bit_exact_vs_live_reference(be):
    """Configuration 4's initial condition, two inclined 8e6-body disks (1.6e7 bodies): keys,
    permutation, node arrays, groups, interaction counts and per-body costs bit for bit against
    the reference CPU backend, forces within relative rms 1e-5."""
    kind = "ref" if O.available("ref") else "port"
    b, _ = S.collision(8_000_000)
    b = zero_v(b)
    n = len(b)
    p = params(1, 0.005, 0.6)
    cpu = O.OracleBackend(kind, 0)
    cpu.upload(b)
    cpu.compute_forces(O.TREE, 1.0, 0.005, 0.6, False)
    be.upload(b)
    be.compute_forces(p, False)
    assert np.array_equal(be.tree_keys(), cpu.keys()), "Morton keys"
    assert np.array_equal(be.download().id, cpu.download().id), "sort permutation"
    rng, mom, _ = be.tree_nodes()
    rn = cpu.nodes()
    assert len(rng) == len(rn), "node count"
    for k, f in enumerate(("lo", "hi", "first", "nchild")):
        assert np.array_equal(rng[:, k], rn[f]), f
    for k, f in enumerate(("cx", "cy", "cz", "m", "qxx", "qxy", "qxz", "qyy", "qyz", "qzz", "rcrit2")):
        assert np.array_equal(mom[:, k], rn[f]), f
    box, lohi = be.tree_groups()
    cg = cpu.groups()
    assert np.array_equal(lohi[:, 0], cg["lo"]) and np.array_equal(lohi[:, 1], cg["hi"]), "groups"
    ti = cpu.times()["interactions"]
    assert be.times().interactions == ti - n
    ok, cost = be.body_costs()
    assert ok and np.array_equal(cost, cpu.body_costs() - 1), "per-body costs"
    e = rel_rms(be.accel()[:3], cpu.accel()[:3])
    print(f"collision16m vs {kind}: {len(rn)} nodes, {len(cg)} groups, {ti} interactions; acc rel rms {e:.3g}")
    assert e <= 1e-5
    cpu.close()


def test_plummer16k_direct_vs_reference_golden_and_fp64(be):
    g = Golden("direct_plummer16384")
    b = g.inputs()
    n = len(b)
    eps = g.param("eps")
    got = accel(be, b, params(0, eps), True)
    ref = g.case("pot")
    ar = g_by_id(ref["order_id"], ref["acc"])[:3].astype(np.float64)
    assert rel_rms(got.a, ar) <= 1e-5
    assert per_body_rel(got.a, ar).max() <= 1e-4
    exact = O.direct_fp64(b, 1.0, eps)
    ex = by_id(b.id, exact[:3])
    assert rel_rms(got.a, ex) <= 1e-5
    assert per_body_rel(got.a, ex).max() <= 1e-4
    ref_pe = 0.5 * float((b.m.astype(np.float64) * exact[3]).sum())
    assert abs(got.diag.pe / ref_pe - 1) <= 1e-5
    assert got.times.interactions == n * (n - 1)


def test_plummer65k_adjoint_directional_central_difference(be):
    n, steps, every = 65536, 34, 32
    G, eps, dt = 1.0, 0.01, 1e-3
    b = S.plummer(n, 2, cut=10)
    x0, v0 = b.pos64(), b.vel64()
    m = b.m.astype(np.float64)
    rng = np.random.Generator(np.random.PCG64(2))
    # Target: a forward run of the initial conditions with positions perturbed by N(0, 1e-3).
    bp = b.copy()
    for f in ("x", "y", "z"):
        setattr(bp, f, (getattr(bp, f) + rng.normal(0, 1e-3, n)).astype(np.float32))
    p = L.ForceParams(G=G, eps=eps, method=L.ForceMethod.direct)
    be.upload(bp)
    be.compute_forces(p, False)
    for _ in range(steps):
        be.kick(0.5 * dt)
        be.drift(dt)
        be.compute_forces(p, False)
        be.kick(0.5 * dt)
    xstar = np.zeros((n, 3))
    xstar[be.download().id] = be.pos64().T
    be.upload(b)
    be.adjoint_forward(p, dt, steps, every)
    loss, gx, gv, gm = be.adjoint_backward(xstar)
    ux = rng.normal(0, 1, (n, 3))
    uv = rng.normal(0, 1, (n, 3))
    s = 1.0 / np.sqrt((ux * ux).sum() + (uv * uv).sum())
    ux *= s
    uv *= s
    h = 1e-5
    lp = O.loss_direct_fp64(x0 + h * ux, v0 + h * uv, m, G, eps, dt, steps, xstar)
    lm = O.loss_direct_fp64(x0 - h * ux, v0 - h * uv, m, G, eps, dt, steps, xstar)
    fd = (lp - lm) / (2 * h)
    ad = float((gx * ux).sum() + (gv * uv).sum())
    rel = abs(ad - fd) / abs(fd)
    print(f"N={n} steps={steps} every={every}: loss {loss:.9g}, directional adjoint {ad:.9g}, "
          f"FP64 central difference {fd:.9g}, rel diff {rel:.3g}")
    assert rel <= 1e-4
