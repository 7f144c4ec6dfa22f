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


def _write_sidecar(path, n, step, ids, lo):
    with open(path, "wb") as f:
        f.write(b"LGF64LO1")
        f.write(np.array([n, step, 0], np.uint64).tobytes())
        pad = np.zeros((n + 1) & ~1, np.uint32)
        pad[:n] = ids
        f.write(pad.tobytes())
        f.write(np.ascontiguousarray(lo, np.float64).tobytes())


def test_fp64_sidecar_reader(lib, tmp_path):
    """The sidecar restores FP64 positions from a float snapshot bit for bit (host-only reader)."""
    from lettuce_simulate_physics_gb300.backend import read_fp64_sidecar
    rng = np.random.Generator(np.random.PCG64(5))
    n = 1001
    pos = rng.normal(0, 3, (n, 3))
    ids = rng.permutation(n).astype(np.uint32)
    f32 = pos.astype(np.float32)
    lo = (pos - f32.astype(np.float64)).T  # (3, n) exact
    path = str(tmp_path / "s.f64lo")
    _write_sidecar(path, n, 77, ids, lo)
    b = L.Bodies(f32[:, 0], f32[:, 1], f32[:, 2], np.zeros(n), np.zeros(n), np.zeros(n), np.ones(n), ids)
    got, step = read_fp64_sidecar(path, b)
    assert step == 77 and np.array_equal(got, pos)
    bad = b.copy()
    bad.id = bad.id[::-1].copy()
    with pytest.raises(RuntimeError):
        read_fp64_sidecar(path, bad)
    with pytest.raises(RuntimeError):
        read_fp64_sidecar(path, b.subset(np.arange(n - 1)))


# ctypes mirrors of the header's structs (backend.py) against the C compiler's layout.
_MIRRORS = {
    "lg_force_params": ("_CForceParams", ["G", "eps", "theta", "method"]),
    "lg_diag": ("_CDiag", ["mass", "ke", "pe", "has_pe", "px", "lz", "cz"]),
    "lg_phase_times": ("_CTimes", ["force_ms", "walk_ms", "interactions", "comm_ms", "balance_ms"]),
    "lg_memory_estimate": ("_CMem", ["device", "host"]),
    "lg_let_tree": ("_CLetTree", ["nodes", "nnodes", "bx", "bm", "nbodies"]),
    "lg_render_options": ("_CRenderOptions", ["width", "height", "view", "extent", "color"]),
    "lg_ensemble_stats": ("_CEnsStats", ["run_ms", "steps", "recoveries", "n", "n_direct", "launches_per_step",
                                         "last_interactions"]),
    "lg_ensemble_tuning": ("_CEnsTuning", ["direct_ipt", "walk_group", "tuned", "direct_tile"]),
}


def test_ctypes_mirrors_match_the_header_layout(tmp_path):
    """Every struct the Python bindings pass through the C ABI has the header's size and field
    offsets (a C program built with the system compiler prints them)."""
    import shutil
    import subprocess
    import ctypes as C
    from lettuce_simulate_physics_gb300 import backend
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "lettuce_gb300.h"', "int main(void) {"]
    for ctype, (_, fields) in _MIRRORS.items():
        lines.append(f'  printf("{ctype} size %zu\\n", sizeof({ctype}));')
        for f in fields:
            lines.append(f'  printf("{ctype} {f} %zu\\n", offsetof({ctype}, {f}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = {}
    for ln in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines():
        t, f, v = ln.split()
        got[(t, f)] = int(v)
    for ctype, (mirror, fields) in _MIRRORS.items():
        m = getattr(backend, mirror)
        assert C.sizeof(m) == got[(ctype, "size")], ctype
        for f in fields:
            assert getattr(m, f).offset == got[(ctype, f)], (ctype, f)
