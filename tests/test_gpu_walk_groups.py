"""The engine's packed walk groups (LETTUCE_GB300_WALK_GROUPS=merged): consecutive sibling groups of
the reference's rule packed into groups of up to 128 bodies. The lists are exact-rule lists for
the larger boxes, so forces stay within the method's accuracy and differ from the reference-group
forces only at the approximation level.

Stated tolerances (theta 0.6, Plummer and disk): relative rms vs the FP64 direct sum <= 1e-3;
per-body median relative difference from the reference-group forces <= 3e-4; theta 0 exact
pair counts N(N-1); costs sum to the interaction count; interaction counts at least the
reference-group counts (larger boxes open more)."""
import os

import numpy as np
import pytest

import lettuce_simulate_physics_gb300 as L
from gpu_util import accel, params, per_body_rel, rel_rms
from lettuce_simulate_physics_gb300 import scenarios as S
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def engine(mode):
    old = os.environ.get("LETTUCE_GB300_WALK_GROUPS")
    os.environ["LETTUCE_GB300_WALK_GROUPS"] = mode
    try:
        from lettuce_simulate_physics_gb300 import build as B
        B.build()
        return L.CudaBackend(0)
    finally:
        if old is None:
            os.environ.pop("LETTUCE_GB300_WALK_GROUPS", None)
        else:
            os.environ["LETTUCE_GB300_WALK_GROUPS"] = old


@pytest.fixture(scope="module")
def pair():
    m, r = engine("merged"), engine("reference")
    yield m, r
    m.close()
    r.close()


@pytest.mark.parametrize("kind", ["plummer", "disk"])
def test_packed_groups_accuracy(pair, kind):
    m, r = pair
    assert m.name().endswith("(packed)") and r.name().endswith("(reference groups)")
    b = S.plummer(30000, 3, cut=20) if kind == "plummer" else S.disk(30000, 4)
    eps = 0.01 if kind == "plummer" else 0.005
    ref = O.direct_fp64(b, 1.0, eps)
    p = params(1, eps, 0.6)
    gm = accel(m, b, p, True)
    gr = accel(r, b, p, True)
    assert rel_rms(gm.a, ref[:3]) <= 1e-3
    assert np.median(per_body_rel(gm.a, gr.a)) <= 3e-4
    assert gm.times.interactions >= gr.times.interactions
    ok, c = m.body_costs()
    assert ok and float(c.astype(np.float64).sum()) == float(gm.times.interactions)
    ngr = r.tree_counts()["groups"]
    ngm = m.tree_counts()["groups"]
    assert ngm < ngr
    box, lohi = m.tree_groups()
    assert len(lohi) == ngm and int(lohi[0][0]) == 0 and int(lohi[-1][1]) == len(b)
    assert np.all(lohi[1:, 0] == lohi[:-1, 1]) and np.all(lohi[:, 1] - lohi[:, 0] <= 128)


def test_packed_groups_theta0_counts(pair):
    m, _ = pair
    b = S.cube(3000, 9)
    g = accel(m, b, params(1, 0.05, 0.0), True)
    assert g.times.interactions == 3000 * 2999
