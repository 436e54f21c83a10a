"""QCSim's Pauli-Hamiltonian simulation over the engine: PauliString::PauliString (PauliString.h:5-43) and
QuantumSimulation::PauliZStringSimulation / PauliStringSimulation / PauliDecomposedHamiltonianSimulation
(PauliStringSimulation.h:14-219).

exp(-i c t P) for a Pauli string P is a basis change to Z on every X / Y qubit (H, or the Hy gate), a CNOT
ladder that gathers the parity on the last qubit, RZ(2 c t), the ladder back and the basis change back.
Execute applies the first-order Trotter product of all terms over the steps.  The whole evolution (steps x
terms x ~4n gates) goes to the engine as one gate list, which the pass planner packs into shared-memory
passes.  getEvolutionOperator is the exact exp(-i t H) on the host (scipy's expm; the reference uses Eigen's
MatrixFunctions), for checks.
"""
from __future__ import annotations

import enum

import numpy as np

from . import gates as G
from .algorithms import QuantumAlgorithm


class PauliOp(enum.IntEnum):
    """PauliString::PauliString::PauliOp (PauliString.h:8-13)"""
    opZ = 0
    opX = 1
    opY = 2


class PauliString:
    """PauliString::PauliString (PauliString.h:5-43): one Pauli operator per qubit (Z by default) and a
    coefficient"""

    PauliOp = PauliOp

    def __init__(self, nrQubits: int = 2):
        self.ops = [PauliOp.opZ] * nrQubits
        self.coeff = 1.0

    def setOperatorForQubit(self, qubit: int, op) -> None:
        if qubit < len(self.ops):
            self.ops[qubit] = PauliOp(op)

    def getOperatorForQubit(self, qubit: int) -> PauliOp:
        return self.ops[qubit] if qubit < len(self.ops) else PauliOp.opZ

    def getCoefficient(self) -> float:
        return self.coeff

    def setCoefficient(self, c: float) -> None:
        self.coeff = float(c)


class PauliZStringSimulation:
    """QuantumSimulation::PauliZStringSimulation (PauliStringSimulation.h:14-49): exp(-i t Z...Z) by a CNOT ladder
    onto the last qubit, RZ(2t) there and the ladder back"""

    def __init__(self, t: float = 0.0):
        self.cnot = G.CNOTGate()
        self.setTimeInterval(t)

    def setTimeInterval(self, t: float) -> None:
        self.rz = G.RzGate(2.0 * t)

    def gates(self, nrQubits: int) -> list[tuple]:
        last = nrQubits - 1
        return ([(self.cnot, q + 1, q) for q in range(last)] + [(self.rz, last)] +
                [(self.cnot, q, q - 1) for q in range(last, 0, -1)])

    def Execute(self, reg) -> int:
        reg.ApplyGates(self.gates(reg.getNrQubits()))
        return 0


class PauliStringSimulation(PauliZStringSimulation):
    """QuantumSimulation::PauliStringSimulation (PauliStringSimulation.h:51-103): the Z-string evolution inside a
    basis change, H on X qubits and the Hy gate on Y qubits (MeasurementBasis, Utils.h:62-130)"""

    def __init__(self, t: float = 0.0, N: int = 3):
        super().__init__(t)
        self.pauliString = PauliString(N)
        self.hadamard = G.HadamardGate()
        self.hy = G.HyGate()

    def setOperatorForQubit(self, qubit: int, op) -> None:
        self.pauliString.setOperatorForQubit(qubit, op)

    def getOperatorForQubit(self, qubit: int) -> PauliOp:
        return self.pauliString.getOperatorForQubit(qubit)

    def getCoefficient(self) -> float:
        return self.pauliString.getCoefficient()

    def setCoefficient(self, c: float) -> None:
        self.pauliString.setCoefficient(c)

    def gates(self, nrQubits: int) -> list[tuple]:
        change = []
        for q in range(nrQubits):
            op = self.getOperatorForQubit(q)
            if op == PauliOp.opX:
                change.append((self.hadamard, q))
            elif op == PauliOp.opY:
                change.append((self.hy, q))
        # H and Hy are their own inverses, so the change back repeats them (PauliStringSimulation.h:70-86)
        return change + super().gates(nrQubits) + change

    def copy(self) -> "PauliStringSimulation":
        t = PauliStringSimulation(0.0, len(self.pauliString.ops))
        t.pauliString.ops = list(self.pauliString.ops)
        t.pauliString.coeff = self.pauliString.coeff
        return t


_PAULI = {PauliOp.opX: np.array([[0, 1], [1, 0]], dtype=np.complex128),
          PauliOp.opY: np.array([[0, -1j], [1j, 0]], dtype=np.complex128),
          PauliOp.opZ: np.array([[1, 0], [0, -1]], dtype=np.complex128)}


class PauliDecomposedHamiltonianSimulation(QuantumAlgorithm):
    """QuantumSimulation::PauliDecomposedHamiltonianSimulation (PauliStringSimulation.h:105-219): H = sum_k c_k P_k
    evolved for simTime in nrSteps first-order Trotter steps"""

    def __init__(self, N: int = 3, t: float = 0.0, nrSteps: int = 1, addSeed: bool = False, **kw):
        super().__init__(N, int(addSeed), **kw)
        self.simTime = t
        self.steps = nrSteps
        self.terms: list[PauliStringSimulation] = []

    def AddTerm(self, coeff: float, term: PauliStringSimulation) -> None:
        """a copy of the term with the coefficient (the reference stores the term by value)"""
        t = term.copy()
        t.setCoefficient(coeff)
        self.terms.append(t)

    def Clear(self) -> None:  # type: ignore[override]
        """removes the terms (PauliStringSimulation.h:123-126; it hides the register's Clear as in the reference)"""
        self.terms = []

    def Execute(self) -> int:
        deltat = self.simTime / self.steps
        n = self.getNrQubits()
        step = []
        for term in self.terms:
            term.setTimeInterval(deltat * term.getCoefficient())
            step += term.gates(n)
        self.ApplyGates(step * self.steps)
        return 0

    def setSimulationTime(self, t: float) -> None:
        self.simTime = t

    def getSimulationTime(self) -> float:
        return self.simTime

    def setNrSteps(self, nrSteps: int) -> None:
        self.steps = nrSteps

    def getNrSteps(self) -> int:
        return self.steps

    def getEvolutionOperator(self, t: float) -> np.ndarray:
        """exp(-i t H) with H built from Kronecker products, qubit 0 rightmost (PauliStringSimulation.h:159-201)"""
        from scipy.linalg import expm
        nb = self.getNrBasisStates()
        H = np.zeros((nb, nb), dtype=np.complex128)
        for term in self.terms:
            tm = _PAULI[term.getOperatorForQubit(0)]
            for q in range(1, self.getNrQubits()):
                tm = np.kron(_PAULI[term.getOperatorForQubit(q)], tm)
            H += term.getCoefficient() * tm
        return expm(-1j * t * H)
