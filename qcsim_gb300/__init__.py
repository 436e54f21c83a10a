"""GB300 statevector engine for QCSim's QubitRegister hot path.

The engine is libqcs_gpu.so (CUDA, sm_103a) behind the C ABI of include/qcs_gpu.h.  This package holds
the host-side mirror of the reference interface (QubitRegister, the QC::Gates classes, the QFT and
one-qubit-transform sub-algorithms), the seeded workload generators and the build recipe.
"""
from . import gates
from ._lib import EngineUnavailable, QcsError
from .register import QubitRegister

__all__ = ["QubitRegister", "gates", "EngineUnavailable", "QcsError"]
