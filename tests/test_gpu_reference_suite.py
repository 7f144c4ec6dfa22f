"""The reference's own CUDA test suite and benchmark driver, run on the GPU against this engine.

The reference's test binary (its tests/*.cpp with tests/test_main.cpp) and lettuce-bench are built
from the reference's sources (LETTUCE_REF, or the staged copy made by baseline/stage.py) and linked
against the C++ Backend adapter (integration/gb300_backend.cpp) in place of src/cuda_backend.cu.
Every "cuda: " case of tests/test_cuda_backend.cpp:173-595 and every "cuda let: " case of
tests/test_cuda_let.cpp:152-354 must run (not skip) and pass, with the reference's own tolerances.
"""
import os
import re
import subprocess

import pytest

from baseline.stage import staged_root
from lettuce_simulate_physics_gb300 import build as B

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(staged_root() is None, reason="reference sources not present")]

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INTEG = os.path.join(ROOT, "lettuce_simulate_physics_gb300", "integration")


@pytest.fixture(scope="module")
def binaries():
    B.build()
    ref = staged_root()
    jobs = str(max(2, min(16, os.cpu_count() or 2)))
    r = subprocess.run(["make", "-s", f"-j{jobs}", "-C", INTEG, f"REF={ref}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return os.path.join(INTEG, "_build"), ref


def test_reference_cuda_suite_runs_and_passes(binaries):
    out, ref = binaries
    r = subprocess.run([os.path.join(out, "lettuce-tests"), "cuda"], cwd=ref, capture_output=True, text=True,
                       timeout=1500)
    log = r.stdout + r.stderr
    print(log[-6000:])
    assert r.returncode == 0, log[-4000:]
    m = re.search(r"(\d+) run, (\d+) failed, (\d+) skipped", log)
    assert m, log[-2000:]
    ran, failed, skipped = map(int, m.groups())
    names = re.findall(r"\[ RUN  \] (.*)", log)
    ok = re.findall(r"\[  OK  \] (.*)", log)
    assert failed == 0 and skipped == 0, log[-4000:]
    assert sum(n.startswith("cuda: ") for n in names) == 15, names
    assert sum(n.startswith("cuda let: ") for n in names) == 5, names
    assert ran == len(names) == len(ok) == 20


def test_reference_bench_runs_the_engine(binaries):
    out, ref = binaries
    r = subprocess.run([os.path.join(out, "lettuce-bench"), "backend=cuda", "method=tree", "n=1000000", "steps=3"],
                       cwd=ref, capture_output=True, text=True, timeout=600)
    print(r.stdout)
    assert r.returncode == 0, r.stderr[-3000:]
    assert "# cuda: " in r.stdout, r.stdout
    row = [ln for ln in r.stdout.splitlines() if re.match(r"cuda\s+tree\s+1000000\s", ln)]
    assert row, r.stdout
    force_ms = float(row[0].split()[3])
    assert force_ms > 0
