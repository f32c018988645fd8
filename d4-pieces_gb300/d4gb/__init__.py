"""d4gb -- Python host bindings of the GB300 row-by-row polyomino tiling engine.

The engine itself is native (``d4-pieces_gb300/csrc``: CUDA kernels for
sm_103a + a C++ runtime behind the C ABI in ``include/d4e.h``).  This package
loads ``libd4e.so`` through ctypes and provides the seeded workload
generators.  Importing :mod:`d4gb.engine` fails loudly when the library has
not been built: there is no CPU fallback.
"""
from .problem import (  # noqa: F401
    FULL_D4,
    ROTATIONS,
    Problem,
    batched_mix,
    canonical,
    pentomino_ring,
    single_large,
    transform,
)
