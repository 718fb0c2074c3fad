"""rampack_gb300: GB300-native (sm_103a) hard-particle Monte Carlo move-and-overlap engine.

The product is the CUDA library behind the C ABI in include/rampack_gb300.h; this
package holds its sources (csrc/), the build recipe (build.py), a Python mirror of
the reference's Packing interface over the ABI (packing.py) and the benchmark
systems' initial configurations (workloads.py).
"""
from . import workloads  # noqa: F401

__all__ = ["workloads", "GpuPacking"]


def __getattr__(name):
    if name == "GpuPacking":
        from .packing import GpuPacking
        return GpuPacking
    raise AttributeError(name)
