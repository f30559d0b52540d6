"""GB300-native hierarchical matrices (the hot path of HierarchicalMatrices.jl).

Public names follow the Julia module (src/HierarchicalMatrices.jl:22-26 and
examples/Kernel.jl): ``BLOCKRANK``, ``BLOCKSIZE``, ``indsplit``,
``KernelMatrix``, the example kernels and ``mul_`` (Julia's ``mul!``).
All products run CUDA kernels compiled for sm_103a in libhmgpu.so.
"""
from ._lib import HMError, Plan
from .kernelmatrix import (BLOCKRANK, BLOCKSIZE, KERNELS, KernelMatrix, KernelMatrixBatch, cauchykernel,
                           coulombkernel, coulombprimekernel, indsplit, logkernel, mul_)

__all__ = [
    "BLOCKRANK", "BLOCKSIZE", "HMError", "KERNELS", "KernelMatrix", "KernelMatrixBatch", "Plan", "cauchykernel",
    "coulombkernel", "coulombprimekernel", "indsplit", "logkernel", "mul_",
]
