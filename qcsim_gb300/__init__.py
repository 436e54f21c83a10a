"""GB300 statevector engine for QCSim's QubitRegister hot path.

The engine is libqcs_gpu.so (CUDA, sm_103a) behind the C ABI of include/qcs_gpu.h.  This package holds
the host-side mirror of the reference interface (QubitRegister, the QC::Gates classes, the QFT and
one-qubit-transform sub-algorithms), the seeded workload generators and the build recipe.

Mirrors of QCSim's algorithm classes over the engine, by module:
  algorithms         QuantumAlgorithm, QFT, phase estimation, Grover, Bernstein-Vazirani, Deutsch-Jozsa, Simon,
                     the adders, the error-correction codes, Shor's factoring
  vqe                VQE with Pauli-string terms and its Nelder-Mead search
  ising              IsingModel and the QAOA sub-algorithm with its optimiser (one register)
  qaoa               many QAOA instances batched in one persistent launch
  counting           quantum counting and the n-controlled NOT with ancillas
  teleportation      cat entangler / disentangler, Bell states, teleportation, entanglement swapping,
                     superdense coding
  measurement_basis  basis changes, the CHSH check, BB84
  distributed        distributed and teleported CNOTs
  paradoxes          quantum eraser, Hardy's paradox, the Elitzur-Vaidman bomb, coin flipping
  oracles            gate-built oracles and the Deutsch-Jozsa, Bernstein-Vazirani and Simon variants on them
  qml                q-means clustering with swap-test overlaps
  pauli_simulation   Trotter evolution under a sum of Pauli strings
  schrodinger        the split-operator Schrodinger simulation
  costmodel          the learned fusion cost model
"""
from . import gates
from ._lib import EngineUnavailable, QcsError
from .register import QubitRegister

__all__ = ["QubitRegister", "gates", "EngineUnavailable", "QcsError"]
