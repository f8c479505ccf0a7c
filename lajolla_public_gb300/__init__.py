"""lajolla_public_gb300: lajolla's rendering hot path on one GB300 (sm_103a).

  abi      ctypes mirror of include/lj_gpu.h
  scenes   flat scene description + seeded generators + Mitsuba XML writer
  gpu      binding of liblj_gpu.so (Context, GpuScene); no CPU fallback
  build    in-tree nvcc build of liblj_gpu.so
"""
from . import abi, scenes  # noqa: F401

__all__ = ["abi", "scenes", "gpu", "build"]
