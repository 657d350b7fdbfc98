"""GB300-native H(curl) curl-curl + mass operator and solver (Hephaestus hot path).

The compute path is the CUDA library behind include/hcurl_op.h; this package
holds the ctypes binding, the host mirror of the reference's operator/solver
interface, and synthetic-workload generators.
"""
from . import meshes  # noqa: F401
from ._native import HcError, NativeUnavailable  # noqa: F401
from .operator import (CurlCurlKernel, GpuComplexCOCGSolver, GpuHCurlPCGSolver, HCurlForm,  # noqa: F401
                       HCurlOperator, VectorFEMassKernel)
