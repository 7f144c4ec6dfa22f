"""Density render on the GPU (lg_render) against the reference's own render_image
(src/render.cpp:83-224) on the same bodies: golden images from the reference (tests/golden/render_*).

Stated tolerance: the fitted extent within 1e-6 relative; RGB bytes equal in >= 99% of the pixels
and within 2 everywhere (the engine sums each pixel's mass exactly in fixed point, the reference in
float in body order, so a colour can round the other way at a byte boundary)."""
import numpy as np
import pytest

import lettuce_simulate_physics_gb300 as L
from golden_io import Golden, names

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def be():
    from lettuce_simulate_physics_gb300 import build as B
    B.build()
    be = L.CudaBackend(0)
    yield be
    be.close()


@pytest.mark.parametrize("name", names("render_"))
def test_render_matches_reference(be, name):
    g = Golden(name)
    be.upload(g.inputs())
    for c in g.cases():
        ref = g.case(c)
        rgb, ext = be.render(int(ref["width"]), int(ref["height"]), str(ref["view"]), float(ref["extent_in"]),
                             "speed" if int(ref["color"]) == 1 else "density")
        assert abs(ext / float(ref["extent"]) - 1) <= 1e-6, (c, ext, float(ref["extent"]))
        d = np.abs(rgb.astype(np.int32) - ref["rgb"].astype(np.int32))
        same = float((d == 0).all(-1).mean())
        print(f"{name}/{c}: {same:.4%} pixels equal, max diff {d.max()}")
        assert same >= 0.99 and d.max() <= 2, (c, same, d.max())


def test_render_rejects_bad_views_and_sizes(be):
    be.upload(L.Bodies.empty(0))
    rgb, ext = be.render(16, 8)
    assert rgb.shape == (8, 16, 3) and not rgb.any() and ext == 1.0
    with pytest.raises(ValueError):
        be.render(16, 16, view="sideways")
    with pytest.raises(ValueError):
        be.render(0, 16)


def test_non_finite_bodies_are_skipped(be):
    """tests/test_render.cpp:83-105: non-finite bodies do not poison the frame."""
    t = np.arange(200) * 0.3
    pos = np.stack([np.cos(t), np.sin(t), np.zeros(200)], 1)
    clean = L.Bodies.from_arrays(pos, np.zeros((200, 3)), np.ones(200))
    be.upload(clean)
    rgb0, ext0 = be.render(64, 64)
    bad_pos = np.array([[np.nan, 0, 0], [0, np.inf, 0], [0, 0, 0]])
    bad_vel = np.array([[0, 0, 0], [0, 0, 0], [np.nan, 0, 0]])
    dirty = clean.append(L.Bodies.from_arrays(bad_pos, bad_vel, np.ones(3)))
    be.upload(dirty)
    rgb1, ext1 = be.render(64, 64)
    assert abs(ext1 - ext0) <= 0.01
    assert int((rgb1 > 40).sum()) > 50
    _, ext_speed = be.render(64, 64, color="speed")
    assert ext_speed > 0
