"""Known-answer cases of the reference's CPU-backend tests, run on the GPU engine with the
reference's own bounds:
- degenerate inputs (tests/test_cpu_backend.cpp:241-285): one body feels nothing; two unit masses
  at distance 1 have PE = -1/sqrt(1 + eps^2) and, after kick(1), |v| = 1/(1 + eps^2)^(3/2) (1e-6);
  40 coincident bodies plus one stay finite, and with eps > 0 their PE is below
  -0.99 * 40*39/2/eps;
- huge opening angles (:288-303): theta 5, 1e6, 1e30 give finite accelerations with total
  momentum change |sum m a_x| < 1;
- a far escaper with a tight clump (:305-335): relative rms <= 1e-3 at theta 0.6 and <= 1e-5 at
  theta 0 against direct summation, interactions <= 1.2 times those without the escaper, every id
  once after download."""
import math

import numpy as np
import pytest

import lettuce_simulate_physics_gb300 as L
from gpu_util import accel, params, rel_rms
from lettuce_simulate_physics_gb300 import scenarios as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def be():
    from lettuce_simulate_physics_gb300 import build as B
    B.build()
    e = L.CudaBackend(0)
    yield e
    e.close()


def bodies(rows):
    a = np.asarray(rows, np.float64)
    return L.Bodies.from_arrays(a[:, 0:3], a[:, 3:6], a[:, 6])


def kdk(be, p, dt, steps):
    be.compute_forces(p, False)
    for _ in range(steps):
        be.kick(0.5 * dt)
        be.drift(dt)
        be.compute_forces(p, False)
        be.kick(0.5 * dt)


def finite(o):
    return all(np.isfinite(getattr(o, f)).all() for f in ("x", "y", "z", "vx", "vy", "vz", "m"))


@pytest.mark.parametrize("method", [0, 1])
@pytest.mark.parametrize("eps", [0.0, 0.01])
def test_degenerate_inputs_stay_finite(be, method, eps):
    p = params(method, eps, 0.6)
    be.upload(bodies([[0.5, -1, 2, 0.1, 0, 0, 1]]))
    be.compute_forces(p, True)
    assert be.diagnostics().pe == 0
    kdk(be, p, 0.01, 3)
    o = be.download()
    assert finite(o)
    assert abs(o.vx[0] - 0.1) <= 1e-7

    be.upload(bodies([[0, 0, 0, 0, 0, 0, 1], [1, 0, 0, 0, 0, 0, 1]]))
    be.compute_forces(p, True)
    assert abs(be.diagnostics().pe - (-1 / math.sqrt(1 + eps * eps))) <= 1e-6
    be.kick(1)
    o = be.download()
    for i in range(2):
        want = (1 if o.x[i] == 0 else -1) / (1 + eps * eps) ** 1.5
        assert abs(o.vx[i] - want) <= 1e-6

    co = bodies([[0.25, 0.25, 0.25, 0, 0, 0, 1]] * 40 + [[1, 1, 1, 0, 0, 0, 1]])
    be.upload(co)
    be.compute_forces(p, True)
    be.kick(1)
    o = be.download()
    assert finite(o)
    pe = be.diagnostics().pe
    assert math.isfinite(pe)
    if eps > 0:
        assert pe < -40 * 39 / 2 / eps * 0.99


def test_huge_theta_is_finite_and_momentum_sane(be):
    b = S.plummer(5000, 6)
    m = b.m.astype(np.float64)
    for theta in (5.0, 1e6, 1e30):
        g = accel(be, b, params(1, 0.01, theta), False)
        assert np.isfinite(g.a).all()
        assert abs(float((m * g.a[0]).sum())) < 1.0


def test_far_escaper_keeps_the_tree_accurate_and_the_walk_small(be):
    b = S.plummer(20000, 7)
    for i in range(60):
        d = np.float32(0.0) if i < 20 else np.float32(1e-6) * np.float32(i % 7 - 3)
        b.x[i] = np.float32(0.3) + d
        b.y[i] = np.float32(0.3) - np.float32(0.5) * d
        b.z[i] = np.float32(0.3) + np.float32(0.25) * d
    be.upload(b)
    be.compute_forces(params(1, 0.01, 0.6), False)
    base = be.times().interactions
    f = b.copy()
    f.x[100] = np.float32(1e8)
    ad = accel(be, f, params(0, 0.01), False).a
    g6 = accel(be, f, params(1, 0.01, 0.6), False)
    e6 = rel_rms(g6.a, ad)
    esc = g6.times.interactions
    e0 = rel_rms(accel(be, f, params(1, 0.01, 0.0), False).a, ad)
    print(f"escaper: rel rms theta 0.6 {e6:.3g}, theta 0 {e0:.3g}; interactions {esc} vs {base} without")
    assert e6 <= 1e-3
    assert e0 <= 1e-5
    assert esc <= 1.2 * base
    o = be.download()
    assert np.array_equal(np.sort(o.id), np.arange(len(f), dtype=np.uint32))
    assert finite(o)
