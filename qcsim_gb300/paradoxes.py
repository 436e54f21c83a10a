"""QCSim's paradox and game demonstrations over the engine: Paradoxes::QuantumEraser (QuantumEraser.h:9-62),
Paradoxes::HardyParadox (HardyParadox.h:11-100), Paradoxes::GeneralElitzurVaidmanBomb
(GeneralElitzurVaidmanBomb.h:11-125), Games::CoinFlipping (CoinFlipping.h:11-48) and Games::MagicSquare
(MagicSquare.h:9-225).  Each circuit goes to the engine as one gate list, and the statistics come from the
register's RepeatedMeasure.
"""
from __future__ import annotations

import math

import numpy as np

from . import gates as G
from .algorithms import QuantumAlgorithm


class QuantumEraser(QuantumAlgorithm):
    """Paradoxes::QuantumEraser (QuantumEraser.h:9-62): H on qubit 0, CNOT(1 <- 0) marks the path, H on qubit 0;
    with the eraser an H on qubit 1 removes the which-path mark, so only 00 and 11 remain"""

    def __init__(self, addseed: int = 0, **kw):
        super().__init__(2, addseed, **kw)
        self.eraser = False
        self.hadamard = G.HadamardGate()
        self.cnot = G.CNOTGate()

    def setEraser(self, e: bool = True) -> None:
        self.eraser = bool(e)

    def getEraser(self) -> bool:
        return self.eraser

    def Execute(self) -> int:
        self.ExecuteWithoutMeasurement()
        return self.Measure()

    def ExecuteWithMultipleMeasurements(self, nrMeasurements: int = 10000) -> dict:
        self.ExecuteWithoutMeasurement()
        return self.RepeatedMeasure(nrMeasurements)

    def ExecuteWithoutMeasurement(self) -> None:
        self.setToBasisState(0)
        ops = [(self.hadamard, 0), (self.cnot, 1, 0), (self.hadamard, 0)]
        if self.eraser:
            ops.append((self.hadamard, 1))
        self.ApplyGates(ops)


class HardyParadox(QuantumAlgorithm):
    """Paradoxes::HardyParadox (HardyParadox.h:11-100): RY(theta0) on qubit 0, RY(theta1) on qubit 1, Toffoli onto
    qubit 2, RY(pi - theta0), RY(pi - theta1); TheoreticalGamma is the probability of 00 among the outcomes
    with qubit 2 clear"""

    def __init__(self, addseed: int = 0, **kw):
        super().__init__(3, addseed, **kw)
        self.ccnot = G.ToffoliGate()
        self.setTheta0(0.575 * math.pi)
        self.setTheta1(0.575 * math.pi)

    def setTheta0(self, t: float) -> None:
        self.theta0 = t

    def getTheta0(self) -> float:
        return self.theta0

    def setTheta1(self, t: float) -> None:
        self.theta1 = t

    def getTheta1(self) -> float:
        return self.theta1

    def Execute(self) -> int:
        self.ExecuteWithoutMeasurement()
        return self.Measure()

    def ExecuteWithMultipleMeasurements(self, nrMeasurements: int = 10000) -> dict:
        self.ExecuteWithoutMeasurement()
        return self.RepeatedMeasure(nrMeasurements)

    def TheoreticalGamma(self) -> float:
        s0, s02, s1 = math.sin(self.theta0), math.sin(0.5 * self.theta0), math.sin(self.theta1)
        c0, c1 = math.cos(self.theta0), math.cos(self.theta1)
        return 0.25 * s0 * s0 * s1 * s1 / (2.0 * s02 * s02 * c1 + c0 + 3.0)

    def ExecuteWithoutMeasurement(self) -> None:
        self.setToBasisState(0)
        self.ApplyGates([(G.RyGate(self.theta0), 0), (G.RyGate(self.theta1), 1), (self.ccnot, 2, 0, 1),
                         (G.RyGate(math.pi - self.theta0), 0), (G.RyGate(math.pi - self.theta1), 1)])


class GeneralElitzurVaidmanBomb(QuantumAlgorithm):
    """Paradoxes::GeneralElitzurVaidmanBomb (GeneralElitzurVaidmanBomb.h:11-125): maxStages + 1 qubits; the
    photon (qubit 0) is rotated by RY(theta_i) = RY((pi - theta) / stages) before each stage, each stage's bomb
    (qubit k) is a CNOT from the photon, and a last RY(theta) closes the interferometer"""

    def __init__(self, maxStages: int, addseed: int = 0, **kw):
        super().__init__(maxStages + 1, addseed, **kw)
        assert self.getNrQubits() >= 2
        self.stages = maxStages
        self.theta = math.pi / (maxStages + 1.0)
        self.cnot = G.CNOTGate()

    def setStages(self, s: int) -> None:
        n = self.getNrQubits()
        self.stages = n - 1 if s >= n else (1 if s == 0 else s)

    def getStages(self) -> int:
        return self.stages

    def setTheta(self, t: float) -> None:
        self.theta = t

    def getTheta(self) -> float:
        return self.theta

    def getThetai(self) -> float:
        return (math.pi - self.theta) / self.stages

    def Execute(self) -> int:
        self.ExecuteWithoutMeasurement()
        return self.Measure()

    def ExecuteWithMultipleMeasurements(self, nrMeasurements: int = 10000) -> dict:
        self.ExecuteWithoutMeasurement()
        return self.RepeatedMeasure(nrMeasurements)

    def TheoreticalEfficiency(self) -> float:
        c = math.cos(0.5 * self.getThetai())
        s = math.sin(0.5 * self.theta)
        cl = math.cos(0.5 * self.theta)
        prod = math.pow(c * c, self.stages)
        return cl * cl * prod / (1.0 - s * s * prod)

    def ExecuteWithoutMeasurement(self) -> None:
        self.setToBasisState(0)
        ry = G.RyGate(self.getThetai())
        ops = [(ry, 0)]
        for stage in range(1, self.stages):
            ops += [(self.cnot, stage, 0), (ry, 0)]
        ops += [(self.cnot, self.stages, 0), (G.RyGate(self.theta), 0)]
        self.ApplyGates(ops)


class CoinFlipping(QuantumAlgorithm):
    """Games::CoinFlipping (CoinFlipping.h:11-48): the quantum player puts the coin in superposition, the
    classical player flips it or not (a seeded numpy choice here, a clock-seeded std::mt19937_64 in the
    reference), and the quantum player's second Hadamard always brings it back to heads (0)"""

    def __init__(self, addseed: int = 0, choice_seed: int | None = None, **kw):
        super().__init__(1, addseed, **kw)
        self.hadamardGate = G.HadamardGate()
        self.flipGate = G.PauliXGate()
        self._rng = np.random.default_rng(choice_seed)
        self.setToBasisState(0)

    def Execute(self) -> int:
        self.setToBasisState(0)
        ops = [(self.hadamardGate, 0)]
        if self._rng.integers(2):
            ops.append((self.flipGate, 0))
        ops.append((self.hadamardGate, 0))
        self.ApplyGates(ops)
        return self.Measure()


# The players' measurement operators of the quantum strategy for the Mermin-Peres magic-square game
# (Brassard, Broadbent and Tapp, "Recasting Mermin's multi-player game into the framework of
# pseudo-telepathy", 2005), as MagicSquare.h:25-90 states them: Alice's for rows 1-3, Bob's for columns 1-3.
_I = 1j
_R2 = 1.0 / math.sqrt(2.0)
_ALICE = (
    _R2 * np.array([[_I, 0, 0, 1], [0, -_I, 1, 0], [0, _I, 1, 0], [1, 0, 0, _I]]),
    0.5 * np.array([[_I, 1, 1, _I], [-_I, 1, -1, _I], [_I, 1, -1, -_I], [-_I, 1, 1, -_I]]),
    0.5 * np.array([[-1, -1, -1, 1], [1, 1, -1, 1], [1, -1, 1, 1], [1, -1, -1, -1]]),
)
_BOB = (
    0.5 * np.array([[_I, -_I, 1, 1], [-_I, -_I, 1, -1], [1, 1, -_I, _I], [-_I, _I, 1, 1]]),
    0.5 * np.array([[-1, _I, 1, _I], [1, _I, 1, -_I], [1, -_I, 1, _I], [-1, -_I, 1, -_I]]),
    _R2 * np.array([[1, 0, 0, 1], [-1, 0, 0, 1], [0, 1, 1, 0], [0, 1, -1, 0]]),
)


class MagicSquare(QuantumAlgorithm):
    """Games::MagicSquare (MagicSquare.h:9-225): Alice (qubits 0, 1) and Bob (qubits 2, 3) share two Bell pairs;
    given a row a and a column b they apply their strategy operator, measure two bits and complete the third by
    parity; they win when Alice's bit in column b equals Bob's bit in row a, which the quantum strategy does in
    every play.  The row, column and who-measures-first choices come from a seeded numpy generator (a
    clock-seeded std::mt19937_64 in the reference)."""

    def __init__(self, addseed: int = 0, choice_seed: int | None = None, **kw):
        super().__init__(4, addseed, **kw)
        self.nrPlays = 100
        self._rng = np.random.default_rng(choice_seed)
        self.A = [G.TwoQubitsGate(m) for m in _ALICE]
        self.B = [G.TwoQubitsGate(m) for m in _BOB]
        self.h, self.z, self.x, self.cnot = G.HadamardGate(), G.PauliZGate(), G.PauliXGate(), G.CNOTGate()
        self.setToBasisState(0)

    def getNrPlays(self) -> int:
        return self.nrPlays

    def setNrPlays(self, n: int) -> None:
        self.nrPlays = n

    def Execute(self) -> int:
        wins = 0
        for _ in range(self.nrPlays):
            a, b = (int(v) for v in self._rng.integers(1, 4, 2))
            wins += self.Play(a, b)[0]
        return wins

    def Play(self, a: int, b: int) -> tuple[bool, int, int]:
        """(won, Alice's three bits, Bob's three bits) for row a and column b in 1..3 (MagicSquare.h:110-145)"""
        self.Init()
        if self._rng.integers(2):
            ra = self.AliceOperations(a)
            rb = self.BobOperations(b)
        else:
            rb = self.BobOperations(b)
            ra = self.AliceOperations(a)
        return ((ra >> (3 - b)) & 1) == ((rb >> (3 - a)) & 1), ra, rb

    def Init(self) -> None:
        self.setToBasisState(0)
        self.ApplyGates([(self.h, 0), (self.h, 1), (self.z, 0), (self.z, 1), (self.cnot, 2, 0), (self.cnot, 3, 1),
                         (self.x, 2), (self.x, 3)])

    def AliceOperations(self, a: int) -> int:
        if 1 <= a <= 3:
            self.ApplyGate(self.A[a - 1], 0, 1)
        r = self.Measure(0, 1) << 1
        return r | 1 if r in (2, 4) else r

    def BobOperations(self, b: int) -> int:
        if 1 <= b <= 3:
            self.ApplyGate(self.B[b - 1], 2, 3)
        r = self.Measure(2, 3) << 1
        return r | 1 if r in (0, 6) else r
