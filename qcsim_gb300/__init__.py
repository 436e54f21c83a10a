"""GB300 statevector engine for QCSim's QubitRegister hot path.

The engine is libqcs_gpu.so (CUDA, sm_103a) behind the C ABI of include/qcs_gpu.h.  This package holds
the host-side mirror of the reference interface (QubitRegister, the QC::Gates classes, the QFT and
one-qubit-transform sub-algorithms), the seeded workload generators and the build recipe.

Modules:
  register     QubitRegister, the mirror of QC::QubitRegister<> over the C ABI
  gates        QCSim's gate classes (matrices and trait answers) and the gate records the engine takes
  subalgo      QuantumAlgorithm, QFT / IQFT, the one-qubit transforms, the N-qubit operator gates
  schrodinger  the split-operator Schrodinger simulation (its Trotter steps in one engine call)
  qaoa         many QAOA instances batched in one persistent launch
  costmodel    the learned fusion cost model
  circuits     seeded workload generators (layered circuits, QFT gate lists, QAOA instances)
  replicas     dealing work to ranks and gathering results

QCSim's own algorithm classes run unchanged in C++ on the drop-in QubitRegister.h of qcsim_gb300/cpp.
"""
from . import gates
from ._lib import EngineUnavailable, QcsError
from .register import QubitRegister

__all__ = ["QubitRegister", "gates", "EngineUnavailable", "QcsError"]
