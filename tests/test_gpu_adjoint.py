"""Adjoint of the KDK leapfrog (direct forces) on the GPU, through the C ABI, against the FP64 CPU
adjoint (oracle/lettuce_oracle.c) and FP64 central finite differences of the FP64 loss (h = 1e-5).

Stated tolerances: loss within 1e-6 relative of the FP64 forward; gradient arrays within 1e-4
relative (norm of the difference over the norm) of the FP64 adjoint; sampled components within
1e-4 relative of the FP64 central differences (FP32 pair arithmetic in the forward and the VJP)."""
import numpy as np
import pytest

import lettuce_simulate_physics_gb300 as L
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


@pytest.mark.parametrize("n,steps,every", [(256, 40, 8), (700, 64, 16), (512, 33, 32)])
def test_adjoint_matches_fp64_adjoint_and_central_differences(be, n, steps, every):
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
            assert abs(grad[i, c] - fd) <= 1e-4 * abs(fd) + 1e-9 * np.abs(grad).max(), (i, c, grad[i, c], fd)
        p, q = m.copy(), m.copy()
        p[i] += h * m[i]
        q[i] -= h * m[i]
        fd = (O.loss_direct_fp64(x0, v0, p, G, eps, dt, steps, xstar)
              - O.loss_direct_fp64(x0, v0, q, G, eps, dt, steps, xstar)) / (2 * h * m[i])
        assert abs(gm[i] - fd) <= 1e-4 * abs(fd) + 1e-9 * np.abs(gm).max(), (i, gm[i], fd)


def test_adjoint_backward_requires_forward(be):
    b = S.plummer(64, 3, cut=10)
    be.upload(b)
    with pytest.raises(L.LogicError):
        be.adjoint_backward(b.pos64())
    with pytest.raises(RuntimeError):
        be.adjoint_forward(L.ForceParams(eps=0.05, method=L.ForceMethod.tree), 1e-3, 4, 2)
