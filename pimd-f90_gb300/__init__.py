"""GB300-native force engine and ring-polymer propagator for PIMD-F90's hot path.

The compute path is libpimd_gb300.so (CUDA for sm_103a behind a C ABI declared in
include/pimd_gb300.h); this package holds its build step, the ctypes host mirror of the
reference's interfaces, the reference's configuration/checkpoint file formats (state_io) and the
synthetic water-box generator used by the benchmark.
"""
from . import build_lib, engine, state_io, waterbox  # noqa: F401
from .engine import ForceEngine, PimdError, load  # noqa: F401
