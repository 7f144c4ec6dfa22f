"""The drop-in boundary from the reference's side: the reference's own drivers and test binary
link against the C++ Backend adapter (integration/gb300_backend.cpp) and the engine library in
place of src/cuda_backend.cu. CPU only; needs the reference sources (LETTUCE_REF, or the staged copy
made by baseline/stage.py; skipped where absent). Without a device the reference's CUDA tests SKIP
through make_cuda_backend returning nullptr with a reason, which this checks too. The same binaries
run on the GPU in tests/test_gpu_reference_suite.py."""
import os
import subprocess

import pytest

from baseline.stage import staged_root
from lettuce_simulate_physics_gb300 import build as B

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = staged_root()
INTEG = os.path.join(ROOT, "lettuce_simulate_physics_gb300", "integration")

pytestmark = pytest.mark.skipif(REF is None, reason="reference sources not present")


@pytest.fixture(scope="module")
def binaries():
    B.build()
    r = subprocess.run(["make", "-s", "-j8", "-C", INTEG, f"REF={REF}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return os.path.join(INTEG, "_build")


def test_reference_test_binary_runs_against_the_adapter(binaries):
    r = subprocess.run([os.path.join(binaries, "lettuce-tests")], cwd=REF, capture_output=True, text=True,
                       timeout=900)
    tail = (r.stdout + r.stderr)[-2000:]
    assert r.returncode == 0, tail
    assert " 0 failed" in tail, tail


def test_reference_bench_drives_the_factory(binaries):
    r = subprocess.run([os.path.join(binaries, "lettuce-bench"), "n=2000", "backend=cpu,cuda", "steps=1",
                        "method=direct"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert "cpu     direct" in r.stdout
    # With a device the engine runs; without one the factory reports why.
    assert ("cuda    direct" in r.stdout) or ("# cuda skipped:" in r.stdout)
