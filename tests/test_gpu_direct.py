"""Direct summation, integration and diagnostics on the GPU, through the C ABI, against the
reference's golden vectors and the FP64 oracle (shapes of tests/test_cuda_backend.cpp:172-378).

Tolerances (stated per test): direct accelerations within 1e-5 relative rms and 1e-4 per body of
the reference's own direct forces and of the FP64 direct sum."""
import math

import numpy as np
import pytest

import lettuce_simulate_physics_gb300 as L
from golden_io import Golden, by_id as g_by_id, names
from gpu_util import accel, by_id, params, per_body_rel, rel_rms
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


def test_name_and_compiled_flag(be):
    assert L.cuda_compiled()
    assert be.name().startswith("cuda: ")
    print(be.name())


def test_direct_vs_fp64_and_reference_4096(be):
    g = Golden("direct_plummer4096")
    b = g.inputs()
    eps = g.param("eps")
    exact = O.direct_fp64(b, 1.0, eps)
    ref_pe = 0.5 * float((b.m.astype(np.float64) * exact[3]).sum())
    g0 = accel(be, b, params(0, eps), False)
    assert rel_rms(g0.a, by_id(b.id, exact[:3])) <= 1e-5
    assert not g0.diag.has_pe
    g1 = accel(be, b, params(0, eps), True)
    e1 = rel_rms(g1.a, by_id(b.id, exact[:3]))
    assert e1 <= 1e-5
    assert g1.diag.has_pe
    assert abs(g1.diag.pe / ref_pe - 1) <= 1e-5
    assert abs(be.exact_potential_energy(1.0, eps) / ref_pe - 1) <= 1e-9
    assert g1.times.interactions == 4096 * 4095
    # Against the reference's own direct forces: rel rms 1e-5, every body within 1e-4.
    ref = g.case("pot")
    ar = g_by_id(ref["order_id"], ref["acc"])[:3].astype(np.float64)
    assert rel_rms(g1.a, ar) <= 1e-5
    assert per_body_rel(g1.a, ar).max() <= 1e-4


@pytest.mark.parametrize("name", names("small_"))
def test_small_and_odd_n_direct_and_tree_theta0(be, name):
    g = Golden(name)
    b = g.inputs()
    n = len(b)
    eps = g.param("eps")
    exact = O.direct_fp64(b, 1.0, eps)
    ref_pe = 0.5 * float((b.m.astype(np.float64) * exact[3]).sum())
    for m in (0, 1):
        got = accel(be, b, params(m, eps, 0.0), True)
        assert np.isfinite(got.a).all()
        if n == 1:
            assert (got.a == 0).all()
            assert got.diag.pe == 0
            continue
        assert rel_rms(got.a, by_id(b.id, exact[:3])) <= 1e-5, m
        assert abs(got.diag.pe / ref_pe - 1) <= 1e-5
        assert got.times.interactions == n * (n - 1)


def test_kick_drift_diagnostics_vs_reference_golden(be):
    g = Golden("kdk_plummer2000")
    b = g.inputs()
    ref = g.case("out")
    G, eps, dt = g.param("G"), g.param("eps"), g.param("dt")
    p = params(0, eps)
    be.upload(b)
    be.compute_forces(p, True)
    be.kick(dt)
    be.drift(dt)
    be.compute_forces(p, True)
    be.kick(dt)
    d = be.diagnostics()
    out = be.download()
    r = np.sqrt(b.x.astype(np.float64) ** 2 + b.y.astype(np.float64) ** 2 + b.z.astype(np.float64) ** 2)
    v = np.sqrt(b.vx.astype(np.float64) ** 2 + b.vy.astype(np.float64) ** 2 + b.vz.astype(np.float64) ** 2)
    m = b.m.astype(np.float64)
    pscale, lscale, cscale = (m * v).sum(), (m * r * v).sum(), (m * r).sum()
    tol = 1e-5
    rd = ref["diag"]
    assert abs(d.mass - rd[0]) <= tol * rd[0]
    assert abs(d.ke - rd[1]) <= tol * rd[1]
    assert d.has_pe
    assert abs(d.pe - rd[2]) <= tol * abs(rd[2])
    for k, val in enumerate((d.px, d.py, d.pz)):
        assert abs(val - rd[3 + k]) <= tol * pscale
    for k, val in enumerate((d.lx, d.ly, d.lz)):
        assert abs(val - rd[6 + k]) <= tol * lscale
    for k, val in enumerate((d.cx, d.cy, d.cz)):
        assert abs(val - rd[9 + k]) <= tol * cscale
    at = np.empty(len(b), np.int64)
    at[ref["id"]] = np.arange(len(b))
    j = at[out.id]

    def close(u, w):
        return np.abs(u.astype(np.float64) - w) <= tol * (np.abs(w.astype(np.float64)) + 1e-2)

    ok = close(out.x, ref["x"][j]) & close(out.y, ref["y"][j]) & close(out.z, ref["z"][j])
    ok &= close(out.vx, ref["vx"][j]) & close(out.vy, ref["vy"][j]) & close(out.vz, ref["vz"][j])
    assert ok.all()


@pytest.mark.parametrize("method", [0, 1])
def test_two_body_circular_orbit_returns_after_one_period(be, method):
    b = L.Bodies.from_arrays(np.array([[0.5, 0, 0], [-0.5, 0, 0]]), np.array([[0, 0.5, 0], [0, -0.5, 0]]),
                             np.array([0.5, 0.5]))
    p = params(method, 0.0)
    steps = 1000
    dt = 2 * math.pi / steps
    be.upload(b)
    be.compute_forces(p, True)
    d0 = be.diagnostics()
    for _ in range(steps):
        be.kick(dt / 2)
        be.drift(dt)
        be.compute_forces(p, True)
        be.kick(dt / 2)
    d1 = be.diagnostics()
    out = be.download()
    for i in range(2):
        k = int(out.id[i])
        dist = math.hypot(out.x[i] - b.x[k], out.y[i] - b.y[k], out.z[i] - b.z[k])
        assert dist <= 1e-3
    assert abs((d1.ke + d1.pe) / (d0.ke + d0.pe) - 1) <= 1e-4


def test_direct_interactions_costs_and_bounds(be):
    b = S.cube(3000, 21)
    be.upload(b)
    be.compute_forces(params(0, 0.05), False)
    ok, cost = be.body_costs()
    assert ok and len(cost) == 3000
    assert float(cost.astype(np.float64).sum()) == be.times().interactions
    box = be.local_bounds()
    out = be.download()
    assert box.lo == (float(out.x.min()), float(out.y.min()), float(out.z.min()))
    assert box.hi == (float(out.x.max()), float(out.y.max()), float(out.z.max()))


def test_eps_zero_coincident_bodies_stay_finite(be):
    b = S.cube(500, 3)
    b.x[:10] = 0.125
    b.y[:10] = 0.25
    b.z[:10] = -0.5
    got = accel(be, b, params(0, 0.0), True)
    assert np.isfinite(got.a).all()
    assert np.isfinite(got.diag.pe)


def test_state_errors_and_empty_and_single(be):
    be.upload(L.Bodies.empty(0))
    be.compute_forces(params(1, 0.01), True)
    assert be.download().size() == 0
    be.upload(S.cube(1, 1))
    be.compute_forces(params(1, 0.01), True)
    assert be.diagnostics().pe == 0
    with pytest.raises(TypeError):
        be.compute_forces_with(params(0, 0.01), False, remote=[object()])
    # A remote tree whose links leave it is rejected before anything reaches the device.
    bad = L.LetTree(np.zeros(1, L.backend.LET_NODE_DTYPE))
    bad.nodes["first_child"] = 5
    bad.nodes["child_count"] = 2
    with pytest.raises(ValueError):
        be.compute_forces_with(params(0, 0.01), False, remote=[bad])


def test_download_into_page_locked_bodies(be):
    b = S.plummer(3000, 21, cut=20)
    be.upload(b)
    be.compute_forces(params(1, 0.01), False)
    be.kick(1e-3)
    be.drift(1e-3)
    want = be.download()
    pin = L.backend.PinnedBodies(len(b))
    try:
        got = be.download(pin.bodies)
        assert got is pin.bodies
        for f in ("x", "y", "z", "vx", "vy", "vz", "m", "id"):
            assert np.array_equal(getattr(got, f), getattr(want, f)), f
        short = L.Bodies.empty(len(b) - 1)
        with pytest.raises(ValueError):
            be.download(short)
    finally:
        pin.free()


def test_bounded_waits_report_timeout_and_engine_stays_usable(be):
    """Failure detection without a GPU fault: waits that nothing satisfies (an mbarrier no one
    arrives on, a flag no one sets) give up after their poll limit, the host reports "device wait
    timed out", the error word is cleared and the next force call is unaffected."""
    b = S.plummer(2000, 41)
    p = params(1, 0.01)
    be.upload(b)
    be.compute_forces(p, True)
    a0, pe0 = be.accel(), be.diagnostics().pe
    with pytest.raises(RuntimeError, match="device wait timed out"):
        be.probe_wait_timeout(2048)
    be.upload(b)
    be.compute_forces(p, True)
    assert np.array_equal(be.accel(), a0) and be.diagnostics().pe == pe0
    with pytest.raises(ValueError):
        be.probe_wait_timeout(0)
