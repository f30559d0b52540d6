"""GB300-native hierarchical matrices (the hot path of HierarchicalMatrices.jl).

Public names follow the Julia module (src/HierarchicalMatrices.jl:22-26 and
examples/Kernel.jl): ``BLOCKRANK``, ``BLOCKSIZE``, ``Block``, ``hierarchical``
(the @hierarchical macro), ``HierarchicalMatrix``, ``LowRankMatrix``,
``BarycentricMatrix2D``, ``KernelMatrix``, ``indsplit``, the example kernels
and ``mul_`` (Julia's ``mul!``), the low-rank and blockwise arithmetic and
``hierarchicalcholesky`` / ``solvetransposed`` (src/LowRankMatrix.jl,
src/algebra.jl, src/cholesky.jl).  All products and block arithmetic run CUDA
kernels compiled for sm_103a in libhmgpu.so.
"""
from ._lib import DeviceWaitTimeout, HMError, Plan
from .hierarchical import (AbstractHierarchical, Adjoint, BarycentricMatrix2D, Block, EvenBarycentricMatrix,
                           HierarchicalMatrix, LowRankMatrix, Transpose, adjoint, hierarchical, mul_, transpose)
from .algebra import (Diagonal, getrank, hierarchicalcholesky, lrzeros, solvetransposed, svdtrunc, times,
                      todense)
from .kernelmatrix import (BLOCKRANK, BLOCKSIZE, KERNELS, KernelMatrix, KernelMatrixBatch, cauchykernel,
                           coulombkernel, coulombprimekernel, indsplit, logkernel)

__all__ = [
    "AbstractHierarchical", "Adjoint", "BLOCKRANK", "BLOCKSIZE", "BarycentricMatrix2D", "Block", "DeviceWaitTimeout",
    "Diagonal",
    "EvenBarycentricMatrix", "HMError", "getrank", "hierarchicalcholesky", "lrzeros", "solvetransposed", "svdtrunc",
    "times", "todense",
    "HierarchicalMatrix", "KERNELS", "KernelMatrix", "KernelMatrixBatch", "LowRankMatrix", "Plan", "Transpose",
    "adjoint", "cauchykernel", "coulombkernel", "coulombprimekernel", "hierarchical", "indsplit", "logkernel",
    "mul_", "transpose",
]
