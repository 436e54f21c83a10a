"""QCSim's measurement-basis helpers and the two protocols built on them, over the engine: QC::MeasurementBasis
(Utils.h:53-212), the CHSH check BellInequalities::CheckCHSHInequality (CheckCHSHInequality.h:9-133) and
the BB84 key exchange QuantumCryptograpy::BB84Protocol (QuantumCryptograpy.h:12-226).

Both protocols are two-qubit and one-qubit circuits with a measurement after almost every gate, so every
step is one engine call.  Their classical random choices come from a seeded numpy generator (the reference
seeds a std::mt19937_64 from the clock); the quantum outcomes come from the register's own generator.
"""
from __future__ import annotations

import cmath
import math

import numpy as np

from . import gates as G
from .algorithms import QuantumAlgorithm
from .teleportation import BellState


class MeasurementBasis:
    """QC::MeasurementBasis (Utils.h:53-212): single-qubit (and Bell) basis changes before a computational
    measurement"""

    def __init__(self):
        self.hadamard = G.HadamardGate()
        self.hy = G.HyGate()
        self.cnot = G.CNOTGate()

    def switchToXBasis(self, reg, qubit: int = 0) -> bool:
        if qubit >= reg.getNrQubits():
            return False
        reg.ApplyGate(self.hadamard, qubit)
        return True

    def switchToYBasis(self, reg, qubit: int = 0) -> bool:
        if qubit >= reg.getNrQubits():
            return False
        reg.ApplyGate(self.hy, qubit)
        return True

    def switchToBellBasis(self, reg, qubit1: int = 0, qubit2: int = 1) -> bool:
        if qubit1 == qubit2 or qubit1 >= reg.getNrQubits() or qubit2 >= reg.getNrQubits():
            return False
        reg.ApplyGates([(self.cnot, qubit2, qubit1), (self.hadamard, qubit1)])
        return True

    switchToComputationalFromXBasis = switchToXBasis
    switchToComputationalFromYBasis = switchToYBasis

    def switchToComputationalFromBellBasis(self, reg, qubit1: int = 0, qubit2: int = 1) -> bool:
        if qubit1 == qubit2 or qubit1 >= reg.getNrQubits() or qubit2 >= reg.getNrQubits():
            return False
        reg.ApplyGates([(self.hadamard, qubit1), (self.cnot, qubit2, qubit1)])
        return True

    @staticmethod
    def operatorBasisMatrix(op, switchBack: bool = False) -> np.ndarray:
        """the unitary whose rows are the conjugated normalised eigenvectors of the 2 x 2 operator, the larger
        eigenvalue's first (Utils.h:143-199); with switchBack its adjoint.  The eigenvectors are taken in the
        same form as the reference's, (ev - d, c) or (b, ev - a), so the unitary carries the same phases."""
        op = np.asarray(op, dtype=np.complex128)
        a, b, c, d = op[0, 0], op[0, 1], op[1, 0], op[1, 1]
        halftrace = 0.5 * (a + d)
        sdelta = cmath.sqrt(halftrace * halftrace - (a * d - b * c))
        ev = (halftrace + sdelta, halftrace - sdelta)
        U = np.eye(2, dtype=np.complex128)
        if abs(c) > 1e-15:
            for k in range(2):
                row = np.array([np.conj(ev[k] - d), np.conj(c)])
                U[k] = row / math.sqrt(abs(row[0]) ** 2 + abs(row[1]) ** 2)
        elif abs(b) > 1e-15:
            for k in range(2):
                row = np.array([np.conj(b), np.conj(ev[k] - a)])
                U[k] = row / math.sqrt(abs(row[0]) ** 2 + abs(row[1]) ** 2)
        elif a.real < d.real:
            U = U[:, ::-1].copy()
        return U.conj().T if switchBack else U

    def switchToOperatorBasis(self, reg, op, qubit: int = 0, switchBack: bool = False) -> bool:
        m = op.getRawOperatorMatrix() if hasattr(op, "getRawOperatorMatrix") else np.asarray(op)
        if qubit >= reg.getNrQubits() or m.shape != (2, 2):
            return False
        reg.ApplyGate(G.SingleQubitGate(self.operatorBasisMatrix(m, switchBack)), qubit)
        return True


class CheckCHSHInequality(QuantumAlgorithm):
    """BellInequalities::CheckCHSHInequality (CheckCHSHInequality.h:9-133): the singlet-like Bell state |11>
    -> (|01> - |10>)/sqrt(2); Alice measures Q = Z or R = X, Bob S = (-Z - X)/sqrt(2) or T = (Z - X)/sqrt(2);
    <QS> + <RS> + <RT> - <QT> tends to 2 sqrt(2)"""

    def __init__(self, addseed: int = 0, choice_seed: int | None = None, **kw):
        super().__init__(2, addseed, **kw)
        self.Q = G.PauliZGate()
        self.R = G.PauliXGate()
        z, x = self.Q.getRawOperatorMatrix(), self.R.getRawOperatorMatrix()
        self.S = (-z - x) / math.sqrt(2.0)
        self.T = (z - x) / math.sqrt(2.0)
        self.bellState = BellState()
        self.measurementBasis = MeasurementBasis()
        self._rng = np.random.default_rng(choice_seed)
        self.ResetStatistics()

    def ResetStatistics(self) -> None:
        self.acc = {"QS": 0, "RS": 0, "RT": 0, "QT": 0}
        self.cnt = {"QS": 0, "RS": 0, "RT": 0, "QT": 0}

    def getValue(self) -> float:
        avg = {k: (self.acc[k] / self.cnt[k] if self.cnt[k] else 0.0) for k in self.acc}
        return avg["QS"] + avg["RS"] + avg["RT"] - avg["QT"]

    def Execute(self) -> int:
        return self.Check()

    def Check(self, separateMeasurements: bool = False) -> int:
        """CheckCHSHInequality.h:55-116"""
        self.bellState.setBellState11(self.reg)
        aM = bool(self._rng.integers(2))
        self.measurementBasis.switchToOperatorBasis(self.reg, self.R if aM else self.Q, 0)
        state, res1 = 0, -1
        if separateMeasurements:
            state = self.Measure(0)
            if state:
                res1 = 1
        bM = bool(self._rng.integers(2))
        self.measurementBasis.switchToOperatorBasis(self.reg, self.T if bM else self.S, 1)
        res2 = -1
        if separateMeasurements:
            state |= self.Measure(1) << 1
        else:
            state = self.Measure()
            if state & 1:
                res1 = 1
        if state & 2:
            res2 = 1
        key = ("R" if aM else "Q") + ("T" if bM else "S")
        self.acc[key] += res1 * res2
        self.cnt[key] += 1
        return state


class BB84Protocol(QuantumAlgorithm):
    """QuantumCryptograpy::BB84Protocol (QuantumCryptograpy.h:12-226) on one qubit: for each of nrBits bits the
    sender draws a basis and a bit by measuring the cat state, rotates into the X basis when chosen, an
    optional eavesdropper measures in a random basis (and rotates back), and the receiver measures in a random
    basis.  Half of the common-basis bits (a random choice) are compared; Execute returns 1 when they all
    match."""

    def __init__(self, addseed: int = 0, nrBits: int = 512, choice_seed: int | None = None, **kw):
        super().__init__(1, addseed, **kw)
        self.nrBits = nrBits
        self.X = G.PauliXGate()
        self.measurementBasis = MeasurementBasis()
        self.eavesdropping = False
        self.randomEavesdropping = False
        self._rng = np.random.default_rng(choice_seed)
        self.Init()

    def Init(self) -> None:
        z = lambda: np.zeros(self.nrBits, dtype=bool)  # noqa: E731
        self.send, self.sendBasis = z(), z()
        self.ereceive, self.ereceiveBasis = z(), z()
        self.receive, self.receiveBasis = z(), z()
        self.commonBasis, self.compare = z(), z()

    def Execute(self) -> int:
        self.Init()
        for b in range(self.nrBits):
            self.sendBasis[b] = self._cat_measure() == 1
            self.send[b] = self._cat_measure() == 1
            if self.sendBasis[b]:
                self.measurementBasis.switchToOperatorBasis(self.reg, self.X, 0, True)
            if self.eavesdropping and (not self.randomEavesdropping or self._random_bool()):
                self.Receive(b, self.ereceive, self.ereceiveBasis, True)
            self.Receive(b, self.receive, self.receiveBasis)
        self.commonBasis = self.sendBasis == self.receiveBasis
        return 1 if self.checkBitsMismatched() else 0

    def getEavesdropping(self) -> bool:
        return self.eavesdropping

    def setEavesdropping(self, val: bool = True) -> None:
        self.eavesdropping = bool(val)

    def getRandomEavesdropping(self) -> bool:
        return self.randomEavesdropping

    def setRandomEavesdropping(self, val: bool = True) -> None:
        self.randomEavesdropping = bool(val)

    def _key_bits(self) -> np.ndarray:
        return self.commonBasis & ~self.compare

    def compareKeys(self) -> bool:
        k = self._key_bits()
        return bool(np.all(self.receive[k] == self.send[k]))

    def getReceivedKey(self) -> list[bool]:
        return self.receive[self._key_bits()].tolist()

    def getSentKey(self) -> list[bool]:
        return self.send[self._key_bits()].tolist()

    def Receive(self, b: int, recv: np.ndarray, recvBasis: np.ndarray, switchBackToZ: bool = False) -> None:
        basis = self._random_bool()
        recvBasis[b] = basis
        if basis:
            self.measurementBasis.switchToOperatorBasis(self.reg, self.X)
        recv[b] = self.Measure() == 1
        if basis and switchBackToZ:
            self.measurementBasis.switchToOperatorBasis(self.reg, self.X, 0, True)

    def checkBitsMismatched(self) -> bool:
        """compare a random half of the common-basis bits; True when none differs (QuantumCryptograpy.h:160-177)"""
        match = True
        for b in range(self.nrBits):
            if self.commonBasis[b] and self._rng.integers(2) == 0:
                self.compare[b] = True
                if self.receive[b] != self.send[b]:
                    match = False
        return match

    def _cat_measure(self) -> int:
        self.setToCatState()
        return self.Measure()

    def _random_bool(self) -> bool:
        return bool(self._rng.integers(2))
