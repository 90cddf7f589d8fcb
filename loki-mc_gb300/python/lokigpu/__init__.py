"""Python front end of the GB300 electron Monte Carlo backend (libloki_gpu.so).

The compute path is the CUDA library behind the C ABI in include/loki_gpu.h;
this package only binds it (ctypes), mirrors the reference engine's
interface (BoltzmannMC: construct from a mixture and working conditions,
``solve()``, result members) and generates the synthetic workloads.
"""
from .capi import LokiGpuError, library_path, load  # noqa: F401
from .engine import BoltzmannMC  # noqa: F401
