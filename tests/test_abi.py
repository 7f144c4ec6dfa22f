"""The C-ABI library: it builds, loads and exports every entry point include/*.h declares; host-side
logic that needs no device. CPU only."""
import glob
import os
import re

import numpy as np
import pytest

import lettuce_simulate_physics_gb300 as L
from lettuce_simulate_physics_gb300 import build as B

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    B.build()
    from lettuce_simulate_physics_gb300 import backend
    return backend._lib()


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"\b(lg_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_symbols()
    for must in ("lg_create", "lg_upload", "lg_download", "lg_compute_forces", "lg_kick", "lg_drift",
                 "lg_diagnostics", "lg_exact_potential_energy", "lg_times", "lg_local_bounds", "lg_build_tree",
                 "lg_compute_forces_with", "lg_memory_need", "lg_device_memory", "lg_body_costs"):
        assert must in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_compiled_flag_and_device_count(lib):
    assert L.cuda_compiled()
    assert L.cuda_device_count() >= 0


def test_factory_without_device_returns_reason():
    if L.cuda_device_count() > 0:
        pytest.skip("a device is present")
    be, why = L.make_cuda_backend(0)
    assert be is None and why


def test_memory_need_grows_with_n_and_tree():
    d1 = L.CudaBackend.memory_need(1000, L.ForceMethod.direct).device
    d2 = L.CudaBackend.memory_need(1_000_000, L.ForceMethod.direct).device
    t2 = L.CudaBackend.memory_need(1_000_000, L.ForceMethod.tree).device
    assert d2 > d1 and t2 > d2


def test_null_engine_is_an_argument_error(lib):
    import ctypes as C
    n = C.c_size_t()
    assert lib.lg_size(None, C.byref(n)) == 3
    assert "null engine" in L.backend.last_error()


def test_bodies_validation():
    with pytest.raises(ValueError):
        L.Bodies(np.zeros(3), np.zeros(2), np.zeros(3), np.zeros(3), np.zeros(3), np.zeros(3), np.zeros(3),
                 np.zeros(3, np.uint32))
