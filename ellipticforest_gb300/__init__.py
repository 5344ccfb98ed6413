"""GB300-native quadtree-adaptive HPS solver (drop-in for EllipticForest's HPS path).

The numerical work runs in ``libellipticforest_gb300.so`` (CUDA, sm_103a) behind the C ABI of
``include/ellipticforest_gb300.h``; this package is a thin Python mirror of the reference's API.
"""
from .hps import (FISHPACK90, FivePointStencil, FiniteVolumeGrid, FiniteVolumeNodeFactory,
                  FiniteVolumePatch, FiniteVolumeSolver, HPSAlgorithm, Mesh, Server, XDIM, YDIM)

__all__ = ["FISHPACK90", "FivePointStencil", "FiniteVolumeGrid", "FiniteVolumeNodeFactory",
           "FiniteVolumePatch", "FiniteVolumeSolver", "HPSAlgorithm", "Mesh", "Server", "XDIM", "YDIM"]
