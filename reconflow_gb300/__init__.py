"""GB300-native (sm_103a) Reconflow: simultaneous optical flow and depth.

The solver runs as hand-written CUDA kernels behind a C ABI
(``include/reconflow_gb300.h``); this package holds the host-side mirror of
the reference's ``CudaFlow`` / ``ReconFlow`` / ``CameraPose`` class surface, the in-tree build
of the CUDA library and the seeded synthetic scene generator.
"""
from ._native import RfError, load  # noqa: F401
from .pose import CameraPose  # noqa: F401
from .reconflow import CudaFlow, ReconFlow, ReconFlowBatch  # noqa: F401

__all__ = ["CameraPose", "CudaFlow", "ReconFlow", "ReconFlowBatch", "RfError", "load"]
