"""GB300 engine for the CVF bulk-water lattice model (drop-in for SOURCE/gpu_water3D).

The compute path is the CUDA library ``_build/libcvf_gb300.so`` behind the C ABI declared in
``include/cvf.h``; this package only loads it (``abi``) and wraps it for Python callers
(``engine``). There is no CPU fallback: if the library is missing, loading fails loudly.
"""
from .abi import lib, CvfError  # noqa: F401
from .engine import Lattice, Params  # noqa: F401
