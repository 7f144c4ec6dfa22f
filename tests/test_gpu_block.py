"""Block (hierarchical) time steps on the GPU (lg_block_step) against the FP64 oracle of the same
scheme (oracle/lettuce_oracle.c or_block_direct_fp64), and the plain leapfrog as its one-level case.

Stated tolerances: direct forces, 3 steps of 16 substeps: levels equal to the oracle's for >= 99.5%
of the bodies and positions within 1e-5 (relative to the system size) of the FP64 trajectory;
max_level 0: bit-identical to the plain kick-drift-kick steps; tree at theta 0 within 1e-5 of the
direct block steps; energy drift of a tree run within 1e-4."""
import numpy as np
import pytest

import lettuce_simulate_physics_gb300 as L
from gpu_util import params
from lettuce_simulate_physics_gb300 import scenarios as S
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def be():
    from lettuce_simulate_physics_gb300 import build as B
    B.build()
    be = L.CudaBackend(0)
    yield be
    be.close()


def state_by_id(be):
    out = be.download()
    n = len(out)
    x = np.zeros((n, 3))
    x[out.id] = be.pos64().T
    v = np.zeros((n, 3))
    v[out.id] = np.stack([out.vx, out.vy, out.vz], 1)
    lv = np.zeros(n, np.uint8)
    lv[out.id] = be.block_levels()
    return x, v, lv


def test_block_steps_match_fp64_oracle(be):
    b = S.plummer(600, 2, cut=10)
    G, eps, dt, K, eta, steps = 1.0, 0.01, 1e-2, 4, 0.05, 3
    be.upload(b)
    be.block_step(params(0, eps), dt, K, eta, steps)
    x, v, lv = state_by_id(be)
    xr, vr, lr = O.block_direct_fp64(b.pos64(), b.vel64(), b.m.astype(np.float64), G, eps, dt, K, eta, steps)
    same = float((lv == lr).mean())
    print(f"levels {np.bincount(lr, minlength=K + 1)}, equal {same:.4f}")
    assert same >= 0.995
    assert len(set(lr.tolist())) >= 2  # the run really uses several levels
    ok = lv == lr
    scale = np.abs(xr).max()
    assert np.abs(x[ok] - xr[ok]).max() <= 1e-5 * scale


def test_level_zero_is_the_plain_leapfrog(be):
    b = S.plummer(2000, 3, cut=20)
    p = params(0, 0.02)
    dt = 1e-3
    be.upload(b)
    be.block_step(p, dt, 0, 0.05, 5)
    xa, va, _ = state_by_id(be)
    be.upload(b)
    be.compute_forces(p, False)
    for _ in range(5):
        be.kick(0.5 * dt)
        be.drift(dt)
        be.compute_forces(p, False)
        be.kick(0.5 * dt)
    out = be.download()
    xb = np.zeros_like(xa)
    xb[out.id] = be.pos64().T
    vb = np.zeros_like(va)
    vb[out.id] = np.stack([out.vx, out.vy, out.vz], 1)
    assert np.array_equal(xa, xb) and np.array_equal(va, vb)


def test_tree_theta0_matches_direct_block_steps(be):
    b = S.plummer(1500, 4, cut=10)
    dt, K, eta, steps = 1e-2, 3, 0.05, 2
    be.upload(b)
    be.block_step(params(0, 0.01), dt, K, eta, steps)
    xd, _, ld = state_by_id(be)
    be.upload(b)
    be.block_step(params(1, 0.01, 0.0), dt, K, eta, steps)
    xt, _, lt = state_by_id(be)
    assert float((ld == lt).mean()) >= 0.995
    ok = ld == lt
    assert np.abs(xd[ok] - xt[ok]).max() <= 1e-5 * np.abs(xd).max()


def test_tree_block_steps_conserve_energy_and_skip_work(be):
    b = S.plummer(20000, 5, cut=10)
    p = params(1, 0.01, 0.6)
    dt, K, eta = 1e-2, 4, 0.05
    be.upload(b)
    be.compute_forces(p, True)
    e0 = be.diagnostics()
    E0 = e0.ke + e0.pe
    be.block_step(p, dt, K, eta, 4)
    lv = be.block_levels()
    assert len(np.unique(lv)) >= 2
    be.compute_forces(p, True)
    e1 = be.diagnostics()
    E1 = e1.ke + e1.pe
    print(f"levels {np.bincount(lv, minlength=K + 1)}, dE/E {abs(E1 / E0 - 1):.2e}")
    assert abs(E1 / E0 - 1) <= 1e-4
