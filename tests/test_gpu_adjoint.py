"""Adjoint of the KDK leapfrog on the GPU, through the C ABI.

Direct forces: against the FP64 CPU adjoint (oracle/lettuce_oracle.c) and FP64 central finite
differences of the FP64 loss (h = 1e-5). Stated tolerances: loss within 1e-6 relative of the FP64
forward; gradient arrays within 1e-4 relative (norm of the difference over the norm) of the FP64
adjoint; sampled components within 1e-4 relative of the FP64 central differences (FP32 pair
arithmetic in the forward and the VJP).

Tree forces (frozen interaction lists): against FP64 central differences of the FP64 frozen-list
loss (oracle FrozenTree: the engine's own trees of the trajectory, lists rebuilt with the walk's
opening rule, cell moments recomputed from the perturbed positions). Stated tolerances: sampled
components within 1e-3 relative (+1e-6 of the largest component), a random directional derivative
within 1e-4 relative; at theta = 0 the tree adjoint equals the direct adjoint within 1e-5."""
import numpy as np
import pytest

import lettuce_simulate_physics_gb300 as L
from gpu_util import deep_radial, traversal_stack_depth, zero_v
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


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - b) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.parametrize("vjp", ["symmetric", "pairs"])
@pytest.mark.parametrize("n,steps,every", [(256, 40, 8), (700, 64, 16), (512, 33, 32)])
def test_adjoint_matches_fp64_adjoint_and_central_differences(be, n, steps, every, vjp, monkeypatch):
    monkeypatch.setenv("LETTUCE_GB300_VJP", vjp)
    b = S.plummer(n, 2, cut=10)
    G, eps, dt = 1.0, 0.05, 1e-3
    x0, v0 = b.pos64(), b.vel64()
    m = b.m.astype(np.float64)
    rng = np.random.Generator(np.random.PCG64(n))
    xstar = x0 + rng.normal(0, 1e-2, x0.shape)
    be.upload(b)
    be.adjoint_forward(L.ForceParams(G=G, eps=eps, method=L.ForceMethod.direct), dt, steps, every)
    loss, gx, gv, gm = be.adjoint_backward(xstar)
    Lr, gxr, gvr, gmr = O.adjoint_direct_fp64(x0, v0, m, G, eps, dt, steps, xstar)
    assert abs(loss / Lr - 1) <= 1e-6, (loss, Lr)
    ex, ev, em = _rel(gx, gxr), _rel(gv, gvr), _rel(gm, gmr)
    print(f"n={n} steps={steps}: rel err gx {ex:.2e} gv {ev:.2e} gm {em:.2e}")
    assert ex <= 1e-4 and ev <= 1e-4 and em <= 1e-4
    h = 1e-5
    picks = rng.choice(n, size=6, replace=False)
    worst = 0.0
    for k, i in enumerate(picks):
        c = k % 3
        for arr, grad in ((x0, gx), (v0, gv)):
            p, q = arr.copy(), arr.copy()
            p[i, c] += h
            q[i, c] -= h
            if arr is x0:
                fd = (O.loss_direct_fp64(p, v0, m, G, eps, dt, steps, xstar)
                      - O.loss_direct_fp64(q, v0, m, G, eps, dt, steps, xstar)) / (2 * h)
            else:
                fd = (O.loss_direct_fp64(x0, p, m, G, eps, dt, steps, xstar)
                      - O.loss_direct_fp64(x0, q, m, G, eps, dt, steps, xstar)) / (2 * h)
            worst = max(worst, abs(grad[i, c] - fd) / abs(fd))
            assert abs(grad[i, c] - fd) <= 1e-4 * abs(fd) + 1e-9 * np.abs(grad).max(), (i, c, grad[i, c], fd)
        p, q = m.copy(), m.copy()
        p[i] += h * m[i]
        q[i] -= h * m[i]
        fd = (O.loss_direct_fp64(x0, v0, p, G, eps, dt, steps, xstar)
              - O.loss_direct_fp64(x0, v0, q, G, eps, dt, steps, xstar)) / (2 * h * m[i])
        worst = max(worst, abs(gm[i] - fd) / abs(fd))
        assert abs(gm[i] - fd) <= 1e-4 * abs(fd) + 1e-9 * np.abs(gm).max(), (i, gm[i], fd)
    print(f"n={n} steps={steps} {vjp}: worst sampled component vs FP64 central differences {worst:.2e}")


@pytest.mark.parametrize("eps", [0.02, 0.0])
def test_symmetric_vjp_equals_one_sided_vjp(be, eps, monkeypatch):
    """The symmetric pairwise VJP (each unordered pair once; 512-body tiles, one block per tile pair,
    here ten tiles with a partial last one) gives the one-sided kernel's gradients to FP32 rounding,
    and repeats itself bit for bit."""
    b = S.plummer(5000, 9, cut=10)
    n = len(b)
    G, dt, steps, every = 1.0, 1e-3, 5, 2
    rng = np.random.Generator(np.random.PCG64(9))
    xstar = b.pos64() + rng.normal(0, 1e-2, (n, 3))
    out = {}
    for mode in ("pairs", "symmetric", "symmetric"):
        monkeypatch.setenv("LETTUCE_GB300_VJP", mode)
        be.upload(b)
        be.adjoint_forward(L.ForceParams(G=G, eps=eps, method=L.ForceMethod.direct), dt, steps, every)
        r = be.adjoint_backward(xstar)
        if mode in out:
            assert all(np.array_equal(x, y) for x, y in zip(r[1:], out[mode][1:])), "deterministic"
        out[mode] = r
    (lp, gxp, gvp, gmp), (ls, gxs, gvs, gms) = out["pairs"], out["symmetric"]
    e = (_rel(gxs, gxp), _rel(gvs, gvp), _rel(gms, gmp))
    print(f"eps={eps}: symmetric vs one-sided gx {e[0]:.3g} gv {e[1]:.3g} gm {e[2]:.3g}")
    assert ls == lp
    tol = 2e-6 if eps > 0 else 1e-4  # unsoftened close pairs amplify FP32 rounding differences
    assert max(e) <= tol


def test_adjoint_backward_requires_forward(be):
    b = S.plummer(64, 3, cut=10)
    be.upload(b)
    with pytest.raises(L.LogicError):
        be.adjoint_backward(b.pos64())
    bad = b.copy()
    bad.id = bad.id + 5
    be.upload(bad)
    with pytest.raises(ValueError):  # the tree path indexes its adjoint state by id
        be.adjoint_forward(L.ForceParams(eps=0.05, method=L.ForceMethod.tree), 1e-3, 4, 2)


def _tree_record(be):
    """The engine's tree after a force call, as a frozen-list record for the oracle."""
    r, mo, _ = be.tree_nodes()
    box, lohi = be.tree_groups()
    return {"perm": be.download().id.astype(np.uint32), "range4": r, "moments11": mo, "glohi": lohi, "box6": box}


def _by_id(be, cols):
    ids = be.download().id
    out = np.zeros((len(ids), cols.shape[0]))
    out[ids] = cols.T
    return out


@pytest.mark.parametrize("eps", [0.03, 0.0])
def test_tree_adjoint_theta0_equals_direct_adjoint(be, eps):
    """At theta = 0 every list is all bodies: the tree VJP is the pairwise VJP (with eps = 0 both
    take the unsoftened kernels, which drop the self pair by r = 0)."""
    b = S.plummer(600, 6, cut=10)
    G, dt, steps, every = 1.0, 1e-3, 12, 4
    rng = np.random.Generator(np.random.PCG64(6))
    xstar = b.pos64() + rng.normal(0, 1e-2, (len(b), 3))
    out = []
    for method in (L.ForceMethod.direct, L.ForceMethod.tree):
        be.upload(b)
        be.adjoint_forward(L.ForceParams(G=G, eps=eps, theta=0.0, method=method), dt, steps, every)
        out.append(be.adjoint_backward(xstar))
    (ld, gxd, gvd, gmd), (lt, gxt, gvt, gmt) = out
    assert np.isfinite(gxt).all() and np.isfinite(gmt).all()
    assert abs(lt / ld - 1) <= 1e-6
    tol = 1e-5 if eps > 0 else 1e-3  # unsoftened close pairs amplify FP32 rounding differences
    assert _rel(gxt, gxd) <= tol and _rel(gvt, gvd) <= tol and _rel(gmt, gmd) <= tol


def test_deep_tree_adjoint_theta0_equals_direct_adjoint(be):
    """The VJP walk runs the forward walk's traversal, spill to the warp's global stack slice
    included: on a 1e5-body, 43-level tree whose smallest groups hold ~290 child blocks (more than
    the 256 shared entries), the theta = 0 tree adjoint must still be the pairwise adjoint. The mass
    gradient comes from the force VJP alone, so a lost or repeated subtree shows there."""
    b = deep_radial(100_000, 3, 12)
    port = O.OracleBackend("port", 0)
    port.upload(zero_v(b))
    port.build_tree(O.TREE, 0.0)
    cg = port.groups()
    h = np.maximum(np.maximum(cg["hx"], cg["hy"]), cg["hz"])
    deepest = traversal_stack_depth(port, np.argsort(h, kind="stable")[:16])
    assert (deepest > 256).sum() >= 4, deepest
    port.close()
    G, eps, dt, steps, every = 1.0, 0.03, 1e-2, 2, 2
    rng = np.random.Generator(np.random.PCG64(8))
    xstar = b.pos64() + rng.normal(0, 1e-2, (len(b), 3))
    out = []
    for method in (L.ForceMethod.direct, L.ForceMethod.tree):
        be.upload(b)
        be.adjoint_forward(L.ForceParams(G=G, eps=eps, theta=0.0, method=method), dt, steps, every)
        out.append(be.adjoint_backward(xstar))
    (ld, gxd, gvd, gmd), (lt, gxt, gvt, gmt) = out
    worst = float(np.max(np.abs(gmt - gmd) / (np.abs(gmd) + 1e-3 * np.abs(gmd).max())))
    print(f"deep tree adjoint: gm rel {_rel(gmt, gmd):.3g} (worst body {worst:.3g}), "
          f"gx rel {_rel(gxt, gxd):.3g}, gv rel {_rel(gvt, gvd):.3g}")
    assert np.isfinite(gxt).all() and np.isfinite(gmt).all()
    assert abs(lt / ld - 1) <= 1e-6
    assert _rel(gxt, gxd) <= 1e-5 and _rel(gvt, gvd) <= 1e-5 and _rel(gmt, gmd) <= 1e-5
    assert worst <= 2e-4


def _engine_with_groups(mode):
    """mode: "reference" or "merged" walk groups, or "groupN": reference groups of up to N bodies
    (N > 128 makes the walk and its VJP take several passes per group)."""
    import os
    env = {"LETTUCE_GB300_WALK_GROUPS": "reference", "LETTUCE_CUDA_GROUP": None}
    if mode.startswith("group"):
        env["LETTUCE_CUDA_GROUP"] = mode[5:]
    else:
        env["LETTUCE_GB300_WALK_GROUPS"] = mode
    old = {k: os.environ.get(k) for k in env}
    try:
        for k, v in env.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
        return L.CudaBackend(0)
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


@pytest.mark.parametrize("theta,groups", [(0.6, "reference"), (0.3, "reference"), (0.6, "merged"),
                                          (0.6, "group256")])
def test_tree_adjoint_vs_frozen_list_central_differences(be, theta, groups):
    be = _engine_with_groups(groups)
    b = S.plummer(3000, 4, cut=10)
    n = len(b)
    G, eps, dt, steps, every = 1.0, 0.02, 2e-3, 6, 2
    p = L.ForceParams(G=G, eps=eps, theta=theta, method=L.ForceMethod.tree)
    # The trajectory's trees through the plain API (the adjoint's forward runs the same kernels).
    be.upload(b)
    be.compute_forces(p, False)
    calls = [_tree_record(be)]
    for s in range(steps):
        be.kick(0.5 * dt)
        be.drift(dt)
        be.compute_forces(p, False)
        if s + 1 < steps:
            calls.append(_tree_record(be))
        be.kick(0.5 * dt)
    xT = _by_id(be, be.pos64())
    rng = np.random.Generator(np.random.PCG64(7))
    xstar = xT + rng.normal(0, 1e-2, xT.shape)
    be.upload(b)
    be.adjoint_forward(p, dt, steps, every)
    assert np.array_equal(_by_id(be, be.pos64()), xT)  # bit-identical trajectory
    loss, gx, gv, gm = be.adjoint_backward(xstar)
    x0, v0, m = b.pos64(), b.vel64(), b.m.astype(np.float64)
    fz = O.FrozenTree(n, calls)
    L0 = fz.loss(x0, v0, m, G, eps, dt, xstar)
    assert abs(loss / L0 - 1) <= 1e-5, (loss, L0)
    h = 1e-5
    worst = 0.0
    for k, i in enumerate(rng.choice(n, size=8, replace=False)):
        c = k % 3
        for arr, grad in ((x0, gx), (v0, gv)):
            pp, qq = arr.copy(), arr.copy()
            pp[i, c] += h
            qq[i, c] -= h
            args_p = (pp, v0) if arr is x0 else (x0, pp)
            args_q = (qq, v0) if arr is x0 else (x0, qq)
            fd = (fz.loss(*args_p, m, G, eps, dt, xstar) - fz.loss(*args_q, m, G, eps, dt, xstar)) / (2 * h)
            err = abs(grad[i, c] - fd) / (abs(fd) + 1e-3 * np.abs(grad).max())
            worst = max(worst, err)
            assert abs(grad[i, c] - fd) <= 1e-3 * abs(fd) + 1e-6 * np.abs(grad).max(), (i, c, grad[i, c], fd)
        pm, qm = m.copy(), m.copy()
        pm[i] += h * m[i]
        qm[i] -= h * m[i]
        fd = (fz.loss(x0, v0, pm, G, eps, dt, xstar) - fz.loss(x0, v0, qm, G, eps, dt, xstar)) / (2 * h * m[i])
        assert abs(gm[i] - fd) <= 1e-3 * abs(fd) + 1e-6 * np.abs(gm).max(), (i, gm[i], fd)
    # A random direction through every component.
    dx, dv = rng.normal(0, 1, x0.shape), rng.normal(0, 1, v0.shape)
    dm = rng.normal(0, 1, n) * m
    hh = 1e-6
    fd = (fz.loss(x0 + hh * dx, v0 + hh * dv, m + hh * dm, G, eps, dt, xstar)
          - fz.loss(x0 - hh * dx, v0 - hh * dv, m - hh * dm, G, eps, dt, xstar)) / (2 * hh)
    ad = float((gx * dx).sum() + (gv * dv).sum() + (gm * dm).sum())
    print(f"theta={theta} {groups}: directional {ad:.9e} vs FD {fd:.9e}; worst sampled {worst:.2e}")
    assert abs(ad - fd) <= 1e-4 * abs(fd), (ad, fd)
    fz.close()
    be.close()


@pytest.mark.parametrize("method", [L.ForceMethod.direct, L.ForceMethod.tree])
def test_seeded_backward_equals_the_target_loss(be, method):
    """lg_adjoint_backward_seeded with dL/dx(T) = 2 m (x(T) - x*) gives the target loss's gradients
    (the mass gradient less the loss's explicit |x(T) - x*|^2)."""
    b = S.plummer(500, 8, cut=10)
    p = L.ForceParams(G=1.0, eps=0.03, theta=0.5, method=method)
    dt, steps, every = 1e-3, 10, 4
    be.upload(b)
    be.adjoint_forward(p, dt, steps, every)
    xT = _by_id(be, be.pos64())
    rng = np.random.Generator(np.random.PCG64(9))
    xstar = xT + rng.normal(0, 1e-2, xT.shape)
    m = b.m.astype(np.float64)
    gx1, gv1, gm1 = be.adjoint_backward_seeded(2 * m[:, None] * (xT - xstar))
    be.upload(b)
    be.adjoint_forward(p, dt, steps, every)
    _, gx2, gv2, gm2 = be.adjoint_backward(xstar)
    assert np.array_equal(gx1, gx2) and np.array_equal(gv1, gv2)
    np.testing.assert_allclose(gm1 + ((xT - xstar) ** 2).sum(1), gm2, rtol=1e-12, atol=1e-14 * np.abs(gm2).max())
