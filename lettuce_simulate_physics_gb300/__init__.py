"""GB300-native force-and-integrate engine for lettuce (NotMaxwell/lettuce_simulate_physics).

The engine is a shared library with a C ABI (include/lettuce_gb300.h) over hand-written sm_103a
CUDA kernels (csrc/). ``backend`` exposes it with the reference's Backend interface; ``scenarios``
holds the seeded workloads; ``build`` compiles the library in-tree with nvcc.
"""
from .bodies import Bodies  # noqa: F401
from .backend import (  # noqa: F401
    Box3, CudaBackend, Diag, ForceMethod, ForceParams, LetTree, LogicError, MemoryNeed, PhaseTimes, UnavailableError,
    cuda_compiled, cuda_device_count, library_path, make_cuda_backend,
)
