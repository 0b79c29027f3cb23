"""GB300-native Helmholtz/Poisson solve path for Nek5000.

The compute path is libnekgpu.so (hand-written CUDA for sm_103a behind the C
ABI of include/nekgpu.h and include/nekmesh.h).  This package holds its
sources (csrc/), the build recipe (build.py), a ctypes binding (_capi.py), a
front end with the reference's routine names (solver.py), a synthetic box
mesher (mesh.py) and the .re2 / .co2 mesh ingestion front end (meshio.py).
"""
from .solver import NekGpu, NekGpuBatch  # noqa: F401

__all__ = ["NekGpu", "NekGpuBatch"]
