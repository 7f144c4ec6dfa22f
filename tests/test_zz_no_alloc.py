"""lg_direct_forces_noalloc, the direct-force entry point that allocates no device memory.

It exists for callers that cannot allocate device memory when they need forces (a code that owns
its device memory through a fixed arena, or a stepping loop that must avoid cudaMalloc's implicit
synchronisation). The test calls it through the C ABI on caller-owned device buffers and checks its
accelerations and potentials against the engine's regular direct path (lg_compute_forces), with
the direct tolerance used elsewhere (1e-5 relative rms), on two calls in a row, so the second call
runs on scratch that still holds the first call's partial sums. Further cases: positions passed as
FP64 high and low parts (against the engine holding the same FP64 positions, 1e-7), a forced
split-j shape whose partial sums exceed the static array (the call uses fewer slices), and pointers
the call must reject on the host before it enqueues any work (misaligned, or host memory).

This file is named to be collected last: pytest runs it after every other test file.
"""
import ctypes as C

import numpy as np
import pytest

import lettuce_simulate_physics_gb300 as L
from lettuce_simulate_physics_gb300 import scenarios as S

pytestmark = pytest.mark.gpu


def _rel_rms(a, ref):
    a = np.asarray(a, np.float64)
    ref = np.asarray(ref, np.float64)
    return float(np.sqrt(((a - ref) ** 2).sum() / (ref ** 2).sum()))


@pytest.mark.parametrize("n,seed", [(4096, 31), (200_000, 32)])
def test_noalloc_direct_matches_engine_direct_twice(n, seed):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("CUDA device not visible to torch")
    from lettuce_simulate_physics_gb300 import backend as Bk
    from lettuce_simulate_physics_gb300 import build as B
    B.build()
    lib = Bk._lib()
    fn = lib.lg_direct_forces_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_int, C.c_void_p, C.c_void_p]

    b = S.plummer(n, seed, cut=20)
    eps = 0.01
    be = L.CudaBackend(0)
    be.upload(b)
    be.compute_forces(L.ForceParams(G=1.0, eps=eps, method=L.ForceMethod.direct), True)
    ref = be.accel()  # upload order: the direct path does not reorder bodies
    assert np.array_equal(be.download().id, b.id)
    be.close()

    dev = torch.device("cuda", 0)
    posm = torch.from_numpy(np.stack([b.x, b.y, b.z, b.m], 1).astype(np.float32)).to(dev)
    poslo = torch.zeros((n, 4), dtype=torch.float32, device=dev)
    acc = torch.empty((n, 4), dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    for call in range(2):
        acc.fill_(float("nan"))
        torch.cuda.synchronize(dev)
        status = fn(posm.data_ptr(), poslo.data_ptr(), n, 1.0, eps, 1, acc.data_ptr(), stream)
        assert status == 0, Bk.last_error()
        got = acc.cpu().numpy().T
        assert np.isfinite(got).all(), f"call {call}"
        assert _rel_rms(got[:3], ref[:3]) <= 1e-5, f"call {call}"
        assert _rel_rms(got[3], ref[3]) <= 1e-5, f"call {call}"


def _fn():
    from lettuce_simulate_physics_gb300 import backend as Bk
    from lettuce_simulate_physics_gb300 import build as B
    B.build()
    fn = Bk._lib().lg_direct_forces_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_int, C.c_void_p, C.c_void_p]
    return fn


def test_noalloc_fp64_split_positions_match_engine():
    torch = pytest.importorskip("torch")
    from lettuce_simulate_physics_gb300 import backend as Bk
    fn = _fn()
    n, eps = 20000, 0.01
    b = S.plummer(n, 33, cut=20)
    rng = np.random.Generator(np.random.PCG64(33))
    # FP64 positions with low parts that a float cannot hold.
    pos = np.stack([b.x, b.y, b.z], 1).astype(np.float64) + rng.uniform(-1e-8, 1e-8, (n, 3))
    be = L.CudaBackend(0)
    be.upload64(b, pos)
    be.compute_forces(L.ForceParams(G=1.0, eps=eps, method=L.ForceMethod.direct), True)
    ref = be.accel()
    assert np.array_equal(be.download().id, b.id)
    be.close()
    hi = pos.astype(np.float32)
    lo = (pos - hi.astype(np.float64)).astype(np.float32)
    dev = torch.device("cuda", 0)
    posm = torch.from_numpy(np.concatenate([hi, b.m[:, None]], 1).astype(np.float32)).to(dev)
    poslo = torch.from_numpy(np.concatenate([lo, np.zeros((n, 1), np.float32)], 1)).to(dev)
    acc = torch.full((n, 4), float("nan"), dtype=torch.float32, device=dev)
    torch.cuda.synchronize(dev)
    status = fn(posm.data_ptr(), poslo.data_ptr(), n, 1.0, eps, 1, acc.data_ptr(),
                torch.cuda.current_stream(dev).cuda_stream)
    assert status == 0, Bk.last_error()
    got = acc.cpu().numpy().T
    assert _rel_rms(got[:3], ref[:3]) <= 1e-7
    assert _rel_rms(got[3], ref[3]) <= 1e-7


def test_noalloc_caps_split_j_to_its_scratch(monkeypatch):
    """64 slices of 65536 bodies need 4M partial sums; the static array holds 1M, so the call runs
    16 slices instead, with the same forces."""
    torch = pytest.importorskip("torch")
    from lettuce_simulate_physics_gb300 import backend as Bk
    fn = _fn()
    n, eps = 65536, 0.01
    b = S.plummer(n, 34, cut=20)
    be = L.CudaBackend(0)
    be.upload(b)
    be.compute_forces(L.ForceParams(G=1.0, eps=eps, method=L.ForceMethod.direct), True)
    ref = be.accel()
    be.close()
    dev = torch.device("cuda", 0)
    posm = torch.from_numpy(np.stack([b.x, b.y, b.z, b.m], 1).astype(np.float32)).to(dev)
    poslo = torch.zeros((n, 4), dtype=torch.float32, device=dev)
    acc = torch.full((n, 4), float("nan"), dtype=torch.float32, device=dev)
    torch.cuda.synchronize(dev)
    monkeypatch.setenv("LETTUCE_GB300_DIRECT", "4,64")
    status = fn(posm.data_ptr(), poslo.data_ptr(), n, 1.0, eps, 1, acc.data_ptr(),
                torch.cuda.current_stream(dev).cuda_stream)
    assert status == 0, Bk.last_error()
    got = acc.cpu().numpy().T
    assert np.isfinite(got).all()
    assert _rel_rms(got[:3], ref[:3]) <= 1e-5
    assert _rel_rms(got[3], ref[3]) <= 1e-5


def test_noalloc_rejects_misaligned_and_host_pointers():
    """Rejected on the host: the call returns LG_ERR_ARG before it enqueues any work."""
    torch = pytest.importorskip("torch")
    from lettuce_simulate_physics_gb300 import backend as Bk
    fn = _fn()
    n = 1024
    dev = torch.device("cuda", 0)
    buf = torch.zeros((n + 1, 4), dtype=torch.float32, device=dev)
    acc = torch.zeros((n, 4), dtype=torch.float32, device=dev)
    status = fn(buf.data_ptr() + 4, buf.data_ptr(), n, 1.0, 0.01, 0, acc.data_ptr(), None)
    assert status == 3 and "aligned" in Bk.last_error()
    host = np.zeros((n, 4), np.float32)
    status = fn(buf.data_ptr(), buf.data_ptr(), n, 1.0, 0.01, 0, host.ctypes.data, None)
    assert status == 3 and "device memory" in Bk.last_error()
    assert np.all(host == 0)


def test_noalloc_rejects_sizes_beyond_its_scratch():
    from lettuce_simulate_physics_gb300 import backend as Bk
    lib = Bk._lib()
    fn = lib.lg_direct_forces_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_int, C.c_void_p, C.c_void_p]
    status = fn(None, None, (1 << 20) + 1, 1.0, 0.01, 0, None, None)
    assert status == 3
    assert "outside" in Bk.last_error()
