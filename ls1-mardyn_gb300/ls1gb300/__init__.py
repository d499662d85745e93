"""GB300-native short-range molecular dynamics for ls1-MarDyn's LinkedCells +
VectorizedCellProcessor + Leapfrog path (host side).

The compute path is the CUDA library ``libls1gb300.so`` behind the C ABI in
``include/ls1gb300.h``; this package holds the phase-space I/O, the ctypes
binding and the Python mirror of the reference's container/integrator calls.
"""
from . import abi, phasespace  # noqa: F401

__all__ = ["abi", "phasespace", "engine"]
