"""GB300-native drop-in for the NDSPMHD per-step SPH hot path.

The product is ``_lib/libndsph_gpu.so`` (C-ABI in ``include/ndsph.h``, built
by ``ndspmhd_gb300.build``).  ``ndspmhd_gb300.gpu`` binds it from Python;
``ndspmhd_gb300.configs`` generates the workloads' particle sets.
"""
from . import configs  # noqa: F401

__all__ = ["configs"]
