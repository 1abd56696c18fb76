"""GB300-native single-level incompressible advance (Kynema-SGF hot path).

The compute path is the CUDA library ``_build/libks.so`` (C ABI declared in
``include/ks.h``).  This module loads it with ctypes and exposes the
reference's ``incflo`` operator surface as :class:`Incflo`.  There is no CPU
fallback: if the library is missing or no CUDA device is visible, the calls
raise.
"""
from .incflo import Incflo, KsError, library_path, load_library, build_library, fma_peak, checkpoint_cost, FIELDS, write_plotfile_host

__all__ = ["Incflo", "KsError", "library_path", "load_library", "build_library", "fma_peak", "checkpoint_cost", "FIELDS",
           "write_plotfile_host"]
