"""Batched ensembles on the GPU (lg_ensemble_*): many independent systems in one forest tree and
one batched direct launch give the same results as running each system alone through the plain
engine, bit for bit, for forces and for whole step sequences, with and without graph capture; the
recovery path for sync-free tree builds; per-system energies; the autotuner and its cache.

Bit-exactness holds because each system's tree in the forest equals its single-system tree
(same frame, keys, topology and moments), the walk visits the same lists, and the batched direct
kernel does each system's sums with the same tiles as the plain kernel without split-j (set with
LETTUCE_GB300_DIRECT="ipt,1,tile" for the plain engine). Accuracy against the FP64 direct sum:
relative rms <= 1e-5 for direct systems and <= 3e-3 for tree systems at theta 0.5."""
import os

import numpy as np
import pytest

import lettuce_simulate_physics_gb300 as L
from gpu_util import rel_rms
from lettuce_simulate_physics_gb300 import scenarios as S
from lettuce_simulate_physics_gb300.ensemble import Ensemble
from oracle import oracle as O

pytestmark = pytest.mark.gpu

# Mixed sizes: three direct systems (one per size class) and four tree systems.
SIZES = [1500, 20000, 3000, 9000, 6000, 33000, 12000]
DIRECT_MAX = 8192
DT = 1e-3


@pytest.fixture(scope="module")
def workload():
    from lettuce_simulate_physics_gb300 import build as B
    B.build()
    return S.ensemble(sizes=SIZES, direct_max=DIRECT_MAX, theta=0.5)


def env(**kv):
    class _Env:
        def __enter__(self):
            self.old = {k: os.environ.get(k) for k in kv}
            for k, v in kv.items():
                if v is None:
                    os.environ.pop(k, None)
                else:
                    os.environ[k] = v

        def __exit__(self, *exc):
            for k, v in self.old.items():
                if v is None:
                    os.environ.pop(k, None)
                else:
                    os.environ[k] = v
    return _Env()


def offsets(counts):
    return np.concatenate([[0], np.cumsum(np.asarray(counts, np.int64))])


def system_bodies(b, lo, hi):
    s = L.Bodies(b.x[lo:hi], b.y[lo:hi], b.z[lo:hi], b.vx[lo:hi], b.vy[lo:hi], b.vz[lo:hi], b.m[lo:hi],
                 b.id[lo:hi] - lo)
    return s


def ensemble_from(workload):
    b, counts, eps, theta, methods = workload
    en = Ensemble(0)
    en.upload(b, counts, eps, theta, methods)
    return en


def plain_engine(k, workload, tuning):
    """A plain engine for system k; direct systems without split-j and with the ensemble's i-bodies
    per thread and j-tile, so the sums are formed in the same order."""
    b, counts, eps, theta, methods = workload
    n = int(counts[k])
    cls = 0 if n < 2048 else (1 if n < 4096 else 2)
    with env(LETTUCE_GB300_DIRECT=f"{tuning.direct_ipt[cls]},1,{tuning.direct_tile[cls]}",
             LETTUCE_CUDA_GROUP=str(tuning.walk_group)):
        return L.CudaBackend(0)


def plain_params(k, workload):
    b, counts, eps, theta, methods = workload
    m = L.ForceMethod.tree if methods[k] == 1 else L.ForceMethod.direct
    return L.ForceParams(G=1.0, eps=float(eps[k]), theta=float(theta[k]), method=m)


def by_local_id(ids, cols):
    out = np.zeros_like(cols)
    out[..., ids] = cols
    return out


def test_forces_bit_exact_vs_plain_engine(workload):
    b, counts, eps, theta, methods = workload
    off = offsets(counts)
    en = ensemble_from(workload)
    en.energy()  # a force phase with potentials
    a = en.accel()
    got = en.download()
    tun = en.tuning()
    for k in range(len(counts)):
        lo, hi = int(off[k]), int(off[k + 1])
        ids = got.id[lo:hi] - lo
        ga = by_local_id(ids, a[:, lo:hi])
        be = plain_engine(k, workload, tun)
        be.upload(system_bodies(b, lo, hi))
        be.compute_forces(plain_params(k, workload), True)
        ra = be.accel()
        ro = be.download()
        ra = by_local_id(ro.id, ra)
        be.close()
        assert np.array_equal(ga.view(np.uint32), ra.view(np.uint32)), f"system {k} (N={hi - lo}, method {methods[k]})"


def test_forces_vs_fp64_direct(workload):
    b, counts, eps, theta, methods = workload
    off = offsets(counts)
    en = ensemble_from(workload)
    en.energy()
    a = en.accel()
    got = en.download()
    for k in (0, 1, 2, 3):
        lo, hi = int(off[k]), int(off[k + 1])
        ids = got.id[lo:hi] - lo
        ga = by_local_id(ids, a[:3, lo:hi]).astype(np.float64)
        sb = system_bodies(b, lo, hi)
        ref = O.direct_fp64(sb, 1.0, float(eps[k]))[:3]
        tol = 1e-5 if methods[k] == 0 else 3e-3
        assert rel_rms(ga, ref) <= tol, (k, rel_rms(ga, ref))


@pytest.mark.parametrize("use_graph", [True, False])
def test_steps_bit_exact_vs_plain_engine(workload, use_graph):
    b, counts, eps, theta, methods = workload
    off = offsets(counts)
    steps = 6
    en = ensemble_from(workload)
    en.run(DT, steps, use_graph=use_graph)
    st = en.stats()
    assert st.used_graph == use_graph
    assert st.recoveries == 0
    got = en.download()
    tun = en.tuning()
    for k in range(len(counts)):
        lo, hi = int(off[k]), int(off[k + 1])
        be = plain_engine(k, workload, tun)
        be.upload(system_bodies(b, lo, hi))
        p = plain_params(k, workload)
        be.compute_forces(p, False)
        for _ in range(steps):
            be.kick(0.5 * DT)
            be.drift(DT)
            be.compute_forces(p, False)
            be.kick(0.5 * DT)
        ro = be.download()
        be.close()
        ids = got.id[lo:hi] - lo
        for f in ("x", "y", "z", "vx", "vy", "vz"):
            mine = by_local_id(ids, getattr(got, f)[lo:hi])
            ref = by_local_id(ro.id, getattr(ro, f))
            assert np.array_equal(mine.view(np.uint32), ref.view(np.uint32)), (k, f)


def test_graph_replay_matches_eager(workload):
    en_g = ensemble_from(workload)
    en_e = ensemble_from(workload)
    for _ in range(2):  # the second graph run replays the captured graph
        en_g.run(DT, 4, use_graph=True)
        en_e.run(DT, 4, use_graph=False)
    assert en_g.stats().captures == 1
    g, e = en_g.download(), en_e.download()
    for f in ("x", "y", "z", "vx", "vy", "vz", "id"):
        assert np.array_equal(getattr(g, f), getattr(e, f)), f


def converging_workload(G):
    """Three systems (direct, tree, tree); in the first tree system 40 bodies have dyadic offsets
    and velocities that bring them onto one point after a drift of 1 (exact in FP64)."""
    b, counts, eps, theta, methods = S.ensemble(sizes=[3000, 20000, 12000], direct_max=DIRECT_MAX, theta=0.5)
    lo = int(counts[0])
    rng = np.random.Generator(np.random.PCG64(3))
    v = rng.integers(-64, 64, (40, 3)).astype(np.float64) / 1024.0
    p0 = np.array([0.5, 0.25, -0.125])
    for c, (pf, vf) in enumerate((("x", "vx"), ("y", "vy"), ("z", "vz"))):
        getattr(b, pf)[lo:lo + 40] = p0[c] - v[:, c]
        getattr(b, vf)[lo:lo + 40] = v[:, c]
    return b, counts, eps, theta, methods


def test_recovery_after_sync_free_miss():
    """A step whose drift makes 40 bodies coincide needs a key restart that the sync-free build
    assumed away: the device-side check flags it and the run is redone from its saved state with
    checked builds. With G = 0 the exact result is x + v dt."""
    b, counts, eps, theta, methods = converging_workload(0.0)
    en = Ensemble(0)
    en.upload(b, counts, eps, theta, methods, G=0.0)
    en.run(1.0, 1, use_graph=True)
    st = en.stats()
    assert st.recoveries == 1
    got = en.download()
    for pf, vf in (("x", "vx"), ("y", "vy"), ("z", "vz")):
        want = (getattr(b, pf).astype(np.float64) + getattr(b, vf).astype(np.float64)).astype(np.float32)
        assert np.array_equal(getattr(got, pf), want[got.id]), pf
    lo = int(counts[0])
    sel = (got.id >= lo) & (got.id < lo + 40)
    assert np.all(got.x[sel] == np.float32(0.5)) and np.all(got.z[sel] == np.float32(-0.125))


def test_forest_key_restarts_bit_exact():
    """A tree system holding 40 coincident bodies needs key restarts in the forest as in a plain
    engine: forces agree bit for bit."""
    b, counts, eps, theta, methods = converging_workload(1.0)
    lo = int(counts[0])
    b.x[lo:lo + 40], b.y[lo:lo + 40], b.z[lo:lo + 40] = np.float32(0.5), np.float32(0.25), np.float32(-0.125)
    wl = (b, counts, eps, theta, methods)
    en = ensemble_from(wl)
    en.energy()
    a = en.accel()
    got = en.download()
    off = offsets(counts)
    tun = en.tuning()
    for k in range(len(counts)):
        s0, s1 = int(off[k]), int(off[k + 1])
        ga = by_local_id(got.id[s0:s1] - s0, a[:, s0:s1])
        be = plain_engine(k, wl, tun)
        be.upload(system_bodies(b, s0, s1))
        be.compute_forces(plain_params(k, wl), True)
        ra = by_local_id(be.download().id, be.accel())
        be.close()
        assert np.array_equal(ga.view(np.uint32), ra.view(np.uint32)), k


def test_forest_nested_key_restarts_bit_exact():
    """A tree system whose bodies sit at radii log-uniform over 30 decades needs key restarts
    within key restarts (a 101-level tree) in the forest as in a plain engine: forces agree bit
    for bit, and the other systems are untouched by its frames."""
    from gpu_util import deep_radial
    b, counts, eps, theta, methods = S.ensemble(sizes=[3000, 20000, 12000], direct_max=DIRECT_MAX, theta=0.5)
    lo, n1 = int(counts[0]), int(counts[1])
    d = deep_radial(n1, 5, 30)
    b.x[lo:lo + n1], b.y[lo:lo + n1], b.z[lo:lo + n1] = d.x, d.y, d.z
    wl = (b, counts, eps, theta, methods)
    en = ensemble_from(wl)
    en.energy()
    a = en.accel()
    got = en.download()
    off = offsets(counts)
    tun = en.tuning()
    for k in range(len(counts)):
        s0, s1 = int(off[k]), int(off[k + 1])
        ga = by_local_id(got.id[s0:s1] - s0, a[:, s0:s1])
        be = plain_engine(k, wl, tun)
        be.upload(system_bodies(b, s0, s1))
        be.compute_forces(plain_params(k, wl), True)
        if k == 1:
            assert be.tree_counts()["max_depth"] > 4 * 21
        ra = by_local_id(be.download().id, be.accel())
        be.close()
        assert np.array_equal(ga.view(np.uint32), ra.view(np.uint32)), k


def test_energy_per_system(workload):
    b, counts, eps, theta, methods = workload
    en = ensemble_from(workload)
    e0, ke0, pe0 = en.energy()
    assert np.all(ke0 > 0) and np.all(pe0 < 0)
    # Plummer clusters in Henon units: E close to -1/4 (softened, truncated: within 10 %).
    assert np.all(np.abs(e0 + 0.25) < 0.025), e0
    en.run(DT, 20, use_graph=True)
    e1, _, _ = en.energy()
    rel = np.abs((e1 - e0) / e0)
    assert np.all(rel < 5e-4), rel


def test_autotuner_and_cache(workload, tmp_path):
    cache = str(tmp_path / "tune.txt")
    with env(LETTUCE_GB300_TUNE_CACHE=cache):
        en = ensemble_from(workload)
        t = en.tune()
        assert t.tuned and all(v in (1, 2, 4) for v in t.direct_ipt) and t.walk_group in (64, 96, 128)
        assert all(v in (128, 256) for v in t.direct_tile)
        assert os.path.exists(cache)
        en2 = ensemble_from(workload)
        t2 = en2.tune()  # loaded from the cache
        assert t2 == t
        # Tuned results stay correct.
        en2.run(DT, 2, use_graph=True)
        e, _, _ = en2.energy()
        assert np.all(np.isfinite(e))
    en.set_tuning((2, 2, 2), 96, (128, 256, 128))
    assert en.tuning().direct_ipt == (2, 2, 2) and en.tuning().walk_group == 96
    assert en.tuning().direct_tile == (128, 256, 128)
    with pytest.raises(ValueError):
        en.set_tuning((8, 2, 2), 96, (128, 256, 256))  # 128-body tiles are built for 1, 2 or 4 i-bodies


def test_tile128_forces_bit_exact_vs_plain_engine(workload):
    """With 128-body j-tiles in every direct class the batched kernel still forms each system's sums
    as the plain kernel does with the same shape."""
    b, counts, eps, theta, methods = workload
    off = offsets(counts)
    en = ensemble_from(workload)
    en.set_tuning((1, 2, 4), 128, (128, 128, 128))
    en.energy()
    a = en.accel()
    got = en.download()
    tun = en.tuning()
    for k in range(len(counts)):
        if methods[k] != 0:
            continue
        lo, hi = int(off[k]), int(off[k + 1])
        ga = by_local_id(got.id[lo:hi] - lo, a[:, lo:hi])
        be = plain_engine(k, workload, tun)
        be.upload(system_bodies(b, lo, hi))
        be.compute_forces(plain_params(k, workload), True)
        ra = by_local_id(be.download().id, be.accel())
        be.close()
        assert np.array_equal(ga.view(np.uint32), ra.view(np.uint32)), k


def test_upload_rejects_bad_tables(workload):
    b, counts, eps, theta, methods = workload
    en = Ensemble(0)
    bad = eps.copy()
    bad[0] = 0.0
    with pytest.raises(ValueError):
        en.upload(b, counts, bad, theta, methods)
    badm = methods.copy()
    badm[0] = 7
    with pytest.raises(ValueError):
        en.upload(b, counts, eps, theta, badm)
    with pytest.raises(ValueError):
        en.upload(b, counts[:-1], eps[:-1], theta[:-1], methods[:-1])
