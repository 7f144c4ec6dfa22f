import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

# Parity with the reference's interaction lists needs its walk groups (the engine's default);
# tests/test_gpu_walk_groups.py covers the packed-groups option.
os.environ.setdefault("LETTUCE_GB300_WALK_GROUPS", "reference")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def _oracle_built():
    """Builds the CPU oracle (and, where the reference sources exist, the reference library)."""
    from oracle import oracle as O
    O.build()
    yield
