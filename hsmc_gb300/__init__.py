"""hsmc_gb300: GB300-native (sm_103a) engine for the local-move hard-sphere
Monte Carlo path of HSMC.

The product is the C ABI in ``include/hsmc_gpu.h`` implemented by
``libhsmc_gpu.so`` (CUDA sources in ``csrc/``) and the drop-in host program
built from ``host/``.  This Python package is a thin ctypes front-end over the
same ABI, for tests, analysis and benchmarks.
"""
from .system import HardSphereSystem, HsmcError, box_from_lattice, compress_to, lattice_config  # noqa: F401
from . import _native  # noqa: F401

__all__ = ["HardSphereSystem", "HsmcError", "box_from_lattice", "compress_to", "lattice_config"]
