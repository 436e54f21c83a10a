"""Algorithms of the hot path, mirroring QCSim's classes over the engine: the QC::QuantumAlgorithm base
(QuantumAlgorithm.h:9-205), the QC::SubAlgo classes
QuantumFourierTransform (QuantumFourierTransform.h:12-92), QubitsSwapper (QubitsSwapper.h:10-43),
OneQubitGateTransform / HadamardTransform / XTransform (HadamardTransform.h:9-41), the dense operator
gates NQubitsQuantumGate (NQubitsQuantumGate.h:9-78) / NQubitsControlledQuantumGate
(NQubitsControlledQuantumGate.h:9-97), phase estimation (PhaseEstimation.h:11-231), Grover's search
with the diagonal oracle matrix (GroverAlgorithm.h:14-124), Bernstein-Vazirani with its diagonal oracle
(BernsteinVazirani.h:14-106), Deutsch-Jozsa (DeutschJozsa.h:16-137) and Simon's algorithm (SimonAlgorithm.h:15-248)
with their permutation oracles, the QFT adders DraperAdder / DraperAdderWithCarry (DraperAdder.h:11-117), the ripple-carry qubit
adders (QuantumAdder.h), the three-qubit flip and sign codes (ErrorCorrectionBase.h, ErrorCorrection3Qubits.h) and
the nine-qubit Shor code (ShorCode.h), and Shor's factoring with
the tensor-product period finding (ShorAlgorithm.h:15-296, PhaseEstimation.h:100-149).

The QFT runs as one engine call (qcs_qft), which applies the reference's gate sequence; the one-qubit
transforms run as one gate list (qcs_one_qubit_transform); the dense operator gates run as one
qcs_apply_operator_on_qubits call on their 2^k x 2^k operator.
"""
from __future__ import annotations

import ctypes as C
import enum
import math

import numpy as np

from . import gates as G
from .register import QubitRegister

from .subalgo import (INT_MAX, HadamardTransform, NQubitsControlledQuantumGate,  # noqa: F401
                      NQubitsQuantumGate, OneQubitGateTransform, QuantumFourierTransform,
                      QuantumSubAlgorithmOnSubregister, QubitsSwapper, XTransform, _operator_qubits)


class QuantumAlgorithm:
    """QC::QuantumAlgorithm (QuantumAlgorithm.h:9-205): owns the register and forwards the state setters,
    gates, measurements and record / replay to it"""

    def __init__(self, N: int = 3, addseed: int = 0, *, precision: str = "fp64", seed: int | None = None):
        self.reg = QubitRegister(N, addseed, precision=precision, seed=seed)

    def getNrQubits(self) -> int:
        return self.reg.getNrQubits()

    def getNrBasisStates(self) -> int:
        return self.reg.getNrBasisStates()

    def getBasisStateAmplitude(self, State: int) -> complex:
        return self.reg.getBasisStateAmplitude(State)

    def getBasisStateProbability(self, State: int) -> float:
        return self.reg.getBasisStateProbability(State)

    def setToBasisState(self, State: int) -> None:
        self.reg.setToBasisState(State)

    def setToQubitState(self, q: int) -> None:
        self.reg.setToQubitState(q)

    def setToCatState(self) -> None:
        self.reg.setToCatState()

    def setToEqualSuperposition(self) -> None:
        self.reg.setToEqualSuperposition()

    def setRawAmplitude(self, State: int, val: complex) -> None:
        self.reg.setRawAmplitude(State, val)

    def Clear(self) -> None:
        self.reg.Clear()

    def Normalize(self) -> None:
        self.reg.Normalize()

    def AdjustPhaseAndNormalize(self) -> None:
        self.reg.AdjustPhaseAndNormalize()

    def getRegister(self) -> QubitRegister:
        return self.reg

    def getRegisterStorage(self) -> np.ndarray:
        return self.reg.getRegisterStorage()

    def setRegisterStorage(self, vals) -> None:
        self.reg.setRegisterStorage(vals)

    def ApplyGate(self, gate, qubit=None, controllingQubit: int = 0, controllingQubit2: int = 0) -> None:
        self.reg.ApplyGate(gate, qubit, controllingQubit, controllingQubit2)

    def ApplyGates(self, gates) -> None:
        self.reg.ApplyGates(gates)

    def ApplyOperatorMatrix(self, m) -> None:
        self.reg.ApplyOperatorMatrix(m)

    def RepeatedMeasure(self, *args) -> dict:
        return self.reg.RepeatedMeasure(*args)

    def Measure(self, *args) -> int:
        """Measure() = MeasureAll, Measure(q) = MeasureQubit, Measure(first, second) (QuantumAlgorithm.h:121-135)"""
        if not args:
            return self.reg.MeasureAll()
        if len(args) == 1:
            return self.reg.MeasureQubit(args[0])
        return self.reg.Measure(args[0], args[1])

    def stateFidelity(self, state) -> float:
        return self.reg.stateFidelity(state)

    def ComputeStart(self) -> None:
        self.reg.ComputeStart()

    def ComputeEnd(self) -> None:
        self.reg.ComputeEnd()

    def ComputeClear(self) -> None:
        self.reg.ComputeClear()

    def Compute(self) -> None:
        self.reg.Compute()

    def Uncompute(self) -> None:
        self.reg.Uncompute()

    def close(self) -> None:
        self.reg.close()


class PhaseEstimationBase:
    """SubAlgo::PhaseEstimationBase (PhaseEstimation.h:11-100): an L-qubit x register (qubits 0 .. L-1) and
    the function register above it"""

    def __init__(self, N: int = 7, L: int = 3):
        self.fRegisterStartQubit = L
        self.nrQubits = N
        self.fourier = QuantumFourierTransform(N, 0, L - 1)

    def getFunctionStartQubit(self) -> int:
        return self.fRegisterStartQubit

    def getNrQubits(self) -> int:
        return self.nrQubits

    def getPhase(self, mostMeasuredState: int, secondMostMeasuredState: int, estimatedProbability: float,
                 nrSteps: int = 10000) -> float:
        """the phase from the two most frequent outcomes (PhaseEstimation.h:32-66): the offset phi whose
        ideal peak probability is closest to the measured one"""
        nrStates = 1 << self.fRegisterStartQubit
        if secondMostMeasuredState == -1:
            return mostMeasuredState / nrStates
        p, phi = 1.0, 0.0
        pref = 1.0 / float(1 << (2 * self.fRegisterStartQubit))
        prefe = 2.0 * math.pi * 1j
        for i in range(1, nrSteps):
            curPhi = i / nrSteps
            e = prefe * curPhi
            a = (np.exp(e) - 1.0) / (np.exp(e / nrStates) - 1.0)
            curProb = pref * abs(a) ** 2
            if abs(estimatedProbability - curProb) < abs(estimatedProbability - p):
                p, phi = curProb, curPhi
        if mostMeasuredState != 0:
            if mostMeasuredState < secondMostMeasuredState and secondMostMeasuredState != nrStates - 1:
                return (mostMeasuredState + phi) / nrStates
            if mostMeasuredState > secondMostMeasuredState:
                return (mostMeasuredState - phi) / nrStates
        return 1.0 + (mostMeasuredState - phi) / nrStates

    def Init(self, reg) -> None:
        """the function register's lowest qubit set, Hadamards on the x register (PhaseEstimation.h:69-87)"""
        reg.setToQubitState(self.fRegisterStartQubit)
        self.ApplyHadamardOnXRegister(reg)

    def ApplyHadamardOnXRegister(self, reg) -> None:
        for i in range(self.fRegisterStartQubit):
            reg.ApplyGate(self.fourier.hadamard, i)

    def IQFT(self, reg, swap: bool = True) -> None:
        self.fourier.IQFT(reg, swap)


class PhaseEstimation(PhaseEstimationBase):
    """SubAlgo::PhaseEstimation (PhaseEstimation.h:153-231): the controlled powers U^(2^j) as
    NQubitsControlledQuantumGate (on the device, no extended matrix), then the IQFT without swaps"""

    def __init__(self, op, N: int = 7, L: int = 3):
        super().__init__(N, L)
        self.U = np.array(op, dtype=np.complex128)
        if self.U.shape[0] != self.U.shape[1]:
            raise ValueError("U must be square")

    def Execute(self, reg) -> int:
        self.ExecuteWithoutMeasurement(reg)
        return reg.Measure(0, self.getFunctionStartQubit() - 1)

    def ExecuteWithMultipleMeasurements(self, reg, nrMeasurements: int = 10000) -> dict:
        self.ExecuteWithoutMeasurement(reg)
        return reg.RepeatedMeasure(0, self.getFunctionStartQubit() - 1, nrMeasurements)

    def getU(self) -> np.ndarray:
        return self.U

    def ExecuteWithoutMeasurement(self, reg) -> None:
        self.Init(reg)
        controlled = self.U.copy()
        last = self.getFunctionStartQubit() - 1
        for ctrl in range(last, 0, -1):
            NQubitsControlledQuantumGate(self.getNrQubits(), controlled, self.getFunctionStartQubit(), ctrl).Execute(reg)
            controlled = controlled @ controlled
        NQubitsControlledQuantumGate(self.getNrQubits(), controlled, self.getFunctionStartQubit(), 0).Execute(reg)
        self.IQFT(reg, False)


class GroverOracle:
    """Grover::Oracle (GroverAlgorithm.h:16-40): the identity with -1 at the marked state"""

    def __init__(self):
        self.correctQuestionState = 0

    def setCorrectQuestionState(self, state: int) -> None:
        self.correctQuestionState = state

    def getOperatorMatrix(self, nrQubits: int) -> np.ndarray:
        m = np.eye(1 << nrQubits, dtype=np.complex128)
        if self.correctQuestionState < (1 << nrQubits):
            m[self.correctQuestionState, self.correctQuestionState] = -1
        return m


class GroverAlgorithm(QuantumAlgorithm):
    """Grover::GroverAlgorithm (GroverAlgorithm.h:42-124): round(pi / 4 sqrt(2^N)) rounds of the oracle and the
    diffusion operator, both applied as ApplyOperatorMatrix of their (diagonal) matrices, which the
    engine runs as one multiply per amplitude"""

    def __init__(self, N: int = 3, addseed: int = 0, **kw):
        super().__init__(N, addseed, **kw)
        o00 = GroverOracle()
        o00.setCorrectQuestionState(0)
        self.OracleOp00 = o00.getOperatorMatrix(N)
        self.hadamard = G.HadamardGate()
        self.setCorrectQuestionState(0)

    def setCorrectQuestionState(self, state: int) -> None:
        o = GroverOracle()
        o.setCorrectQuestionState(state)
        self.OracleOp = o.getOperatorMatrix(self.getNrQubits())

    def Execute(self) -> int:
        self.ExecuteWithoutMeasurement()
        return self.Measure()

    def ExecuteWithMultipleMeasurements(self, nrMeasurements: int = 10000) -> dict:
        self.ExecuteWithoutMeasurement()
        return self.RepeatedMeasure(nrMeasurements)

    def Init(self) -> None:
        self.setToEqualSuperposition()

    def ExecuteWithoutMeasurement(self) -> None:
        self.Init()
        repeat = int(math.floor(math.pi / 4.0 * math.sqrt(self.getNrBasisStates()) + 0.5))  # C round() for positives
        for _ in range(repeat):
            self.ApplyOperatorMatrix(self.OracleOp)
            self.ApplyDiffusionOperator()

    def ApplyHadamardOnAllQubits(self) -> None:
        for i in range(self.getNrQubits()):
            self.ApplyGate(self.hadamard, i)

    def ApplyDiffusionOperator(self) -> None:
        self.ApplyHadamardOnAllQubits()
        self.ApplyOperatorMatrix(self.OracleOp00)
        self.ApplyHadamardOnAllQubits()


class DraperAdder(QuantumAlgorithm):
    """Adders::DraperAdder (DraperAdder.h:11-57): registers a (qubits 0 .. N-1) and b (N .. 2N-1); b <- a + b
    mod 2^N by a QFT of b (no swaps), the controlled phases pi / 2^(q - N - c) from a's qubits c, and the
    inverse QFT.  The phases commute, so they go to the engine as one gate list."""

    def __init__(self, N: int = 3, addseed: int = 0, **kw):
        super().__init__(2 * N, addseed, **kw)
        self.n = N
        self.fourier = QuantumFourierTransform(2 * N, N)
        self.setToBasisState(0)

    def Execute(self) -> int:
        self.ExecuteWithoutMeasurement()
        return self.Measure()

    def ExecuteWithMultipleMeasurements(self, nrMeasurements: int = 10000) -> dict:
        self.ExecuteWithoutMeasurement()
        return self.RepeatedMeasure(nrMeasurements)

    def _sum_phases(self) -> list:
        ops = []
        for qbit in range(self.n, 2 * self.n):
            phase = math.pi
            for cbit in range(qbit - self.n, -1, -1):
                ops.append((G.ControlledPhaseShiftGate(phase), qbit, cbit))
                phase *= 0.5
        return ops

    def ExecuteWithoutMeasurement(self) -> None:
        self.fourier.QFT(self.reg, False)
        self.ApplyGates(self._sum_phases())
        self.fourier.IQFT(self.reg, False)


class DraperAdderWithCarry(DraperAdder):
    """Adders::DraperAdderWithCarry (DraperAdder.h:59-115): as DraperAdder with one more qubit (2N) above b
    that receives the carry: the QFT covers b and the carry qubit, which gets the phases pi / 2^(N - c)
    from a's qubits"""

    def __init__(self, N: int = 3, addseed: int = 0, **kw):
        QuantumAlgorithm.__init__(self, 2 * N + 1, addseed, **kw)
        self.n = N
        self.fourier = QuantumFourierTransform(2 * N + 1, N)
        self.setToBasisState(0)

    def ExecuteWithoutMeasurement(self) -> None:
        self.fourier.QFT(self.reg, False)
        ops = []
        phase = math.pi / 2
        for cbit in range(self.n - 1, -1, -1):
            ops.append((G.ControlledPhaseShiftGate(phase), 2 * self.n, cbit))
            phase *= 0.5
        self.ApplyGates(ops + self._sum_phases())
        self.fourier.IQFT(self.reg, False)


class TwoQubitsHalfAdder:
    """Adders::TwoQubitsHalfAdder (QuantumAdder.h:10-43): sum of qubit1 and qubit2 into qubit2, carry into aux
    (Toffoli, then CNOT); returns 1 for a qubit out of range and 2 for repeated qubits"""

    def __init__(self, qubit1: int, qubit2: int, qubitaux: int):
        self.q1, self.q2, self.aux = qubit1, qubit2, qubitaux
        self.toffoli, self.cnot = G.ToffoliGate(), G.CNOTGate()

    def Execute(self, reg) -> int:
        n = reg.getNrQubits()
        if self.aux >= n or self.q2 >= n or self.q1 >= n:
            return 1
        if len({self.q1, self.q2, self.aux}) < 3:
            return 2
        reg.ApplyGates([(self.toffoli, self.aux, self.q1, self.q2), (self.cnot, self.q2, self.q1)])
        return 0


class TwoQubitsFullAdder(TwoQubitsHalfAdder):
    """Adders::TwoQubitsFullAdder (QuantumAdder.h:45-85): two half adders and a CNOT that restores qubit2; the
    sum ends on cin and the carry on aux"""

    def __init__(self, qubit1: int, qubit2: int, cin: int, qubitaux: int):
        super().__init__(qubit1, qubit2, qubitaux)
        self.ci = cin
        self.halfAdder = TwoQubitsHalfAdder(qubit2, cin, qubitaux)

    def Execute(self, reg) -> int:
        n = reg.getNrQubits()
        if self.aux >= n or self.q2 >= n or self.q1 >= n or self.ci >= n:
            return 1
        if len({self.q1, self.q2, self.aux, self.ci}) < 4:
            return 2
        super().Execute(reg)
        self.halfAdder.Execute(reg)
        reg.ApplyGate(self.cnot, self.q2, self.q1)
        return 0


class NQubitsAdderAlgorithm(QuantumAlgorithm):
    """Adders::NQubitsAdderAlgorithm (QuantumAdder.h:87-125): 3N + 1 qubits, the addends on qubits 0..N-1 and
    N..2N-1 (kept), a ripple of full adders leaving the N + 1-bit sum on qubits 2N..3N; returns the measured
    register"""

    def __init__(self, N: int = 3, addseed: int = 0, **kw):
        super().__init__(3 * N + 1, addseed, **kw)
        self.setToBasisState(0)

    def Execute(self) -> int:
        nq = self.getNrQubits()
        assert nq >= 4
        n = (nq - 1) // 3
        for k in range(n):
            TwoQubitsFullAdder(k, n + k, 2 * n + k, 2 * n + k + 1).Execute(self.reg)
        return self.Measure()


class BernsteinVaziraniOracle:
    """BernsteinVazirani::Oracle (BernsteinVazirani.h:16-57): -1 on the basis states whose bitwise product
    with the hidden string has odd parity"""

    def __init__(self):
        self.stringFunction = 0

    def setString(self, s: int) -> None:
        self.stringFunction = s

    def f(self, x: int) -> int:
        return bin(x & self.stringFunction).count("1") % 2

    def getOperatorMatrix(self, nrQubits: int) -> np.ndarray:
        x = np.arange(1 << nrQubits)
        parity = np.zeros(x.size, dtype=np.int64)
        prod = x & self.stringFunction
        while prod.any():
            parity += prod & 1
            prod >>= 1
        return np.diag(np.where(parity % 2 == 1, -1.0, 1.0).astype(np.complex128))


class BernsteinVaziraniAlgorithm(QuantumAlgorithm):
    """BernsteinVazirani::BernsteinVaziraniAlgorithm (BernsteinVazirani.h:59-106): the equal superposition, the
    oracle matrix (diagonal: one multiply per amplitude on the engine), Hadamards on every qubit, and a
    measurement that returns the hidden string"""

    def __init__(self, N: int = 3, addseed: int = 0, **kw):
        super().__init__(N, addseed, **kw)
        self.hadamard = G.HadamardGate()
        self.setString(0)

    def setString(self, s: int) -> None:
        o = BernsteinVaziraniOracle()
        o.setString(s)
        self.OracleOp = o.getOperatorMatrix(self.getNrQubits())

    def Execute(self) -> int:
        self.setToEqualSuperposition()
        self.ApplyOperatorMatrix(self.OracleOp)
        for i in range(self.getNrQubits()):
            self.ApplyGate(self.hadamard, i)
        return self.Measure()


class DeutschJozsaAlgorithm(QuantumAlgorithm):
    """DeutschJozsa::DeutschJozsaAlgorithm (DeutschJozsa.h:16-137): is f on N - 1 bits constant or balanced?
    The register starts in |1>|0...0> (the answer qubit is the top one), gets Hadamards on every qubit, the
    oracle U|y>|x> = |y + f(x)>|x> as a 2^N x 2^N permutation matrix (ApplyOperatorMatrix), and Hadamards on
    every qubit but the top one; the x part of the measured state is zero exactly for a constant f.  The
    reference shuffles the balanced function with a clock-seeded generator; here it is a seeded numpy one
    (function_seed)."""

    class FunctionType(enum.IntEnum):
        constantZero = 0
        constantOne = 1
        balanced = 2

    def __init__(self, N: int = 2, addseed: int = 0, function_seed: int | None = None, **kw):
        assert N >= 2
        super().__init__(N, addseed, **kw)
        self.hadamard = G.HadamardGate()
        self.functionType = self.FunctionType.constantZero
        self.fvalues = np.zeros(0, dtype=np.int64)
        self._rng = np.random.default_rng(function_seed)

    def Execute(self) -> int:
        self.setToQubitState(self.getNrQubits() - 1)
        n = self.getNrQubits()
        self.ApplyGates([(self.hadamard, q) for q in range(n)])
        self.ApplyOperatorMatrix(self.getOracleMatrix())
        self.ApplyGates([(self.hadamard, q) for q in range(n - 1)])
        return self.Measure()

    def WasConstantResult(self, state: int) -> bool:
        return (state & ((self.getNrBasisStates() - 1) >> 1)) == 0

    def setFunction(self, ft) -> None:
        """balanced: half of the 2^(N-1) inputs map to 1, in a random order (DeutschJozsa.h:54-72)"""
        self.functionType = self.FunctionType(ft)
        if self.functionType == self.FunctionType.balanced:
            size = self.getNrBasisStates() >> 1
            v = np.zeros(size, dtype=np.int64)
            v[: size >> 1] = 1
            self.fvalues = self._rng.permutation(v)
        else:
            self.fvalues = np.zeros(0, dtype=np.int64)

    def getFunction(self):
        return self.functionType

    def f(self, x):
        if self.functionType == self.FunctionType.balanced:
            return self.fvalues[x]
        return np.full(np.shape(x), int(self.functionType), dtype=np.int64)

    def getOracleMatrix(self) -> np.ndarray:
        """U(ket, bra) = 1 where x_ket = x_bra and y_ket = y_bra + f(x_bra) mod 2 (DeutschJozsa.h:104-129)"""
        nb = self.getNrBasisStates()
        top = self.getNrQubits() - 1
        bra = np.arange(nb)
        x = bra & ((nb - 1) >> 1)
        ket = x | ((self.f(x) ^ (bra >> top)) << top)
        u = np.zeros((nb, nb), dtype=np.complex128)
        u[ket, bra] = 1
        return u


class SimonFunction:
    """Simon::SimonFunction (SimonAlgorithm.h:15-97): a random function on N bits that is one-to-one for the
    string 0 and two-to-one with f(x) = f(x ^ s) otherwise.  The reference shuffles with a clock-seeded
    generator; here it is a seeded numpy one."""

    def __init__(self, rng=None):
        self.stringFunction = 0
        self.functionTable = np.zeros(0, dtype=np.int64)
        self._rng = rng if rng is not None else np.random.default_rng()

    def __call__(self, x):
        if self.functionTable.size == 0:
            return np.zeros(np.shape(x), dtype=np.int64)
        return self.functionTable[np.asarray(x) & (self.functionTable.size - 1)]

    def setString(self, s: int, N: int) -> None:
        """a shuffled identity table, then for every x its partner x ^ s (taken once, in a shuffled order)
        gets the same value (SimonAlgorithm.h:27-64)"""
        self.stringFunction = s
        nb = 1 << N
        table = self._rng.permutation(nb)
        indices = list(self._rng.permutation(nb))
        for x in range(nb):
            for i in range(nb):
                y = indices[i]
                if y is None or x == y:
                    continue
                if (x ^ y) == s:
                    table[x] = table[y]
                    indices[i] = None
                    break
        self.functionTable = table.astype(np.int64)

    def checkFunction(self) -> bool:
        """one-to-one for s = 0; otherwise every value taken by exactly a pair {a, a ^ s} (SimonAlgorithm.h:66-93)"""
        t = self.functionTable
        if self.stringFunction == 0:
            return len(set(t.tolist())) == t.size
        groups: dict[int, list[int]] = {}
        for i, v in enumerate(t.tolist()):
            groups.setdefault(v, []).append(i)
        if len(groups) != t.size // 2:
            return False
        return all(len(g) == 2 and (g[0] ^ g[1]) in (0, self.stringFunction) for g in groups.values())


class SimonAlgorithm(QuantumAlgorithm):
    """Simon::SimonAlgorithm (SimonAlgorithm.h:148-248): 2N qubits, x in the low N and f(x) in the high N.  Each
    round prepares |0>, Hadamards on the x half, the oracle B|x>|y> = |x>|y ^ f(x)> as a permutation matrix
    (ApplyOperatorMatrix), Hadamards on the x half again and a measurement of the x half; every outcome b has
    b.s = 0 mod 2.  After up to 300 rounds (or all 2^N outcomes, meaning s = 0) the candidates of s with odd
    parity against a measured b are removed; Execute returns the one left, 0, or 2^N when ambiguous."""

    def __init__(self, N: int = 3, addseed: int = 0, function_seed: int | None = None, **kw):
        assert N >= 2
        super().__init__(2 * N, addseed, **kw)
        self.hadamard = G.HadamardGate()
        self.f = SimonFunction(np.random.default_rng(function_seed))
        self.setString(0)

    def setString(self, s: int) -> None:
        N = self.getNrQubits() >> 1
        self.f.setString(s, N)
        self.OracleOp = self.getOracleMatrix()

    def getOracleMatrix(self) -> np.ndarray:
        """B(ket, bra) = 1 where x_ket = x_bra and y_ket = y_bra ^ f(x_bra) (SimonAlgorithm.h:104-136)"""
        N = self.getNrQubits() >> 1
        nb = self.getNrBasisStates()
        bra = np.arange(nb)
        xmask = (1 << N) - 1
        x = bra & xmask
        ket = x | ((bra & (xmask << N)) ^ (self.f(x) << N))
        u = np.zeros((nb, nb), dtype=np.complex128)
        u[ket, bra] = 1
        return u

    def Execute(self) -> int:
        N = self.getNrQubits() >> 1
        mask = (1 << N) - 1
        measurements: dict[int, int] = {}
        for _ in range(300):
            self.setToBasisState(0)
            self.ApplyGates([(self.hadamard, q) for q in range(N)])
            self.ApplyOperatorMatrix(self.OracleOp)
            self.ApplyGates([(self.hadamard, q) for q in range(N)])
            m = self.Measure(0, N - 1)
            measurements[m] = measurements.get(m, 0) + 1
            if len(measurements) == 1 << N:
                return 0
        candidates = set(range(1, mask + 1))
        for b in measurements:
            if b:
                candidates = {c for c in candidates if bin(c & b).count("1") % 2 == 0}
        return next(iter(candidates)) if len(candidates) == 1 else mask + 1


class ErrorCorrectionBase(QuantumAlgorithm):
    """ErrorCorrection::ErrorCorrectionBase (ErrorCorrectionBase.h:8-50): a one-qubit state on qubit 0 and the
    qubit an error hits (N or more: no error)"""

    def __init__(self, N: int, addseed: int = 0, **kw):
        super().__init__(N, addseed, **kw)
        self.errorQubit = N
        self.cnot, self.ccnot, self.x = G.CNOTGate(), G.ToffoliGate(), G.PauliXGate()
        self.setToBasisState(0)

    def SetState(self, alpha: complex, beta: complex) -> None:
        self.Clear()
        self.setRawAmplitude(0, alpha)
        self.setRawAmplitude(1, beta)
        self.Normalize()

    def SetErrorQubit(self, q: int = 0) -> None:
        self.errorQubit = q

    def GetErrorQubit(self) -> int:
        return self.errorQubit


class ErrorCorrection3Qubits(ErrorCorrectionBase):
    """ErrorCorrection3Qubits (ErrorCorrection3Qubits.h:8-33): repetition code on qubits 0-2"""

    def __init__(self, addseed: int = 0, **kw):
        super().__init__(3, addseed, **kw)

    def Encode(self) -> None:
        self.ApplyGate(self.cnot, 1, 0)
        self.ApplyGate(self.cnot, 2, 0)

    def DetectAndCorrect(self) -> None:
        self.ApplyGate(self.cnot, 1, 0)
        self.ApplyGate(self.cnot, 2, 0)
        self.ApplyGate(self.ccnot, 0, 1, 2)


class ErrorCorrection3QubitsFlip(ErrorCorrection3Qubits):
    """bit-flip code (ErrorCorrection3Qubits.h:35-64): returns the syndrome on qubits 1-2 (3: qubit 0 was
    flipped, 1 / 2: qubit 1 / 2, 0: none)"""

    def Execute(self) -> int:
        self.Encode()
        self.ApplyError()
        self.DetectAndCorrect()
        return self.Measure(1, 2)

    def ApplyError(self) -> None:
        if self.errorQubit <= 2:
            self.ApplyGate(self.x, self.errorQubit)


class ErrorCorrection3QubitsSign(ErrorCorrection3Qubits):
    """sign-flip code (ErrorCorrection3Qubits.h:67-110): the flip code in the Hadamard basis"""

    def __init__(self, addseed: int = 0, **kw):
        super().__init__(addseed, **kw)
        self.hadamard = G.HadamardGate()

    def Execute(self) -> int:
        self.Encode()
        self.ApplyHadamardOnAllQubits()
        self.ApplyError()
        self.ApplyHadamardOnAllQubits()
        self.DetectAndCorrect()
        return self.Measure(1, 2)

    def ApplyError(self) -> None:
        if self.errorQubit <= 2:
            self.ApplyGate(self.hadamard, self.errorQubit)
            self.ApplyGate(self.x, self.errorQubit)
            self.ApplyGate(self.hadamard, self.errorQubit)

    def ApplyHadamardOnAllQubits(self) -> None:
        for i in range(self.getNrQubits()):
            self.ApplyGate(self.hadamard, i)


class ShorCode(ErrorCorrectionBase):
    """ErrorCorrection::ShorCode (ShorCode.h:8-107): the nine-qubit code; any single-qubit flip, sign or
    combined (iY) error on one of the nine qubits is corrected.  Execute returns the measurement of qubits
    1-8, which is 0 exactly when no error was applied."""

    class ErrorType(enum.IntEnum):
        Flip = 0
        Sign = 1
        Both = 2
        none = 3  # the reference's None: no error

    def __init__(self, addseed: int = 0, **kw):
        super().__init__(9, addseed, **kw)
        self.errorType = self.ErrorType.Flip
        self.hadamard = G.HadamardGate()
        self.z = G.PauliZGate()
        self.iy = G.SingleQubitGate(1j * G.PauliYGate().getRawOperatorMatrix())

    def setErrorType(self, t) -> None:
        self.errorType = self.ErrorType(t)

    def getErrorType(self):
        return self.errorType

    def Execute(self) -> int:
        self.Encode()
        self.ApplyError()
        self.DetectAndCorrect()
        return self.Measure(1, self.getNrQubits() - 1)

    def ApplyError(self) -> None:
        if self.errorQubit >= self.getNrQubits():
            return
        gate = {self.ErrorType.Flip: self.x, self.ErrorType.Sign: self.z, self.ErrorType.Both: self.iy}.get(self.errorType)
        if gate is not None:
            self.ApplyGate(gate, self.errorQubit)

    def Encode(self) -> None:
        """ShorCode.h:66-80: the sign code across qubits 0, 3, 6, each expanded into a flip code"""
        ops = [(self.cnot, 3, 0), (self.cnot, 6, 0)]
        for q in (0, 3, 6):
            ops += [(self.hadamard, q), (self.cnot, q + 1, q), (self.cnot, q + 2, q)]
        self.ApplyGates(ops)

    def DetectAndCorrect(self) -> None:
        """ShorCode.h:82-98"""
        ops = []
        for q in (0, 3, 6):
            ops += [(self.cnot, q + 1, q), (self.cnot, q + 2, q), (self.ccnot, q, q + 1, q + 2), (self.hadamard, q)]
        ops += [(self.cnot, 3, 0), (self.cnot, 6, 0), (self.ccnot, 0, 3, 6)]
        self.ApplyGates(ops)


class FxBase:
    """Shor::FxBase (ShorAlgorithm.h:15-52): x register = qubits 0 .. L-1, f register = L .. L+M-1, f(x) = A^x mod C"""

    def __init__(self, L: int, M: int, C: int):
        self.fRegisterStartQubit, self.fRegisterNrQubits, self.Number, self.A = L, M, C, 2

    def setParam(self, a: int) -> None:
        self.A = a

    def getParam(self) -> int:
        return self.A

    def mod(self, v: int) -> int:
        return v % self.Number

    def getFunctionStartQubit(self) -> int:
        return self.fRegisterStartQubit

    def getFunctionNrQubits(self) -> int:
        return self.fRegisterNrQubits


class Fx(FxBase):
    """Shor::Fx (ShorAlgorithm.h:54-104): for each x qubit l, the f register multiplied by A^(2^l) mod C where
    that qubit is one (values f >= C unchanged).  The reference applies each as a 2^N x 2^N matrix; here
    each is a 2^M x 2^M permutation controlled by qubit l on the device (ApplyOperatorOnQubits).  A^(2^l)
    is formed as the reference forms it, by repeated squaring in 64-bit unsigned arithmetic."""

    def Apply(self, reg) -> None:
        L, M = self.fRegisterStartQubit, self.fRegisterNrQubits
        d = 1 << M
        an = self.A
        for l in range(L):
            perm = np.zeros((d, d), dtype=np.complex128)
            mult = self.mod(an)
            for f in range(d):
                perm[self.mod(mult * f) if f < self.Number else f, f] = 1
            reg.ApplyOperatorOnQubits(perm, list(range(L, L + M)), [l])
            an = (an * an) & 0xFFFFFFFFFFFFFFFF


class ShorPhaseEstimation(PhaseEstimationBase):
    """SubAlgo::ShorPhaseEstimation (PhaseEstimation.h:100-149): Hadamards on x, f(x) into the f register, IQFT of
    x (with swaps), then a measurement of the whole register"""

    def __init__(self, f: FxBase, N: int = 7, L: int = 3):
        super().__init__(N, L)
        self.func = f

    def Execute(self, reg) -> int:
        self.ExecuteWithoutMeasurement(reg)
        return reg.MeasureAll()

    def ExecuteWithMultipleMeasurements(self, reg, nrMeasurements: int = 10000) -> dict:
        self.ExecuteWithoutMeasurement(reg)
        return reg.RepeatedMeasure(nrMeasurements)

    def ExecuteWithoutMeasurement(self, reg) -> None:
        self.Init(reg)
        self.func.Apply(reg)
        self.IQFT(reg)


class ShorAlgorithm(QuantumAlgorithm):
    """Shor::ShorAlgorithmBase + ShorAlgorithm (ShorAlgorithm.h:108-296): period finding on N qubits (x register
    of L qubits) and the classical steps of factorize.  The reference draws the base a from a device-seeded
    std::mt19937; here it comes from a seeded numpy generator (factor_seed)."""

    def __init__(self, C: int = 15, N: int = 7, L: int = 3, addseed: int = 0, factor_seed: int | None = None, **kw):
        super().__init__(N, addseed, **kw)
        self.Number = C
        self.fx = Fx(L, N - L, C)
        self.phaseEstimation = ShorPhaseEstimation(self.fx, N, L)
        self._rng = np.random.default_rng(factor_seed)

    def setA(self, a: int) -> None:
        self.fx.setParam(a)

    def Execute(self) -> int:
        return self.phaseEstimation.Execute(self.reg)

    def ExecuteWithMultipleMeasurements(self, nrMeasurements: int = 10000) -> dict:
        return self.phaseEstimation.ExecuteWithMultipleMeasurements(self.reg, nrMeasurements)

    @staticmethod
    def gcd(a: int, b: int) -> int:
        while b:
            a, b = b, a % b
        return a

    @staticmethod
    def continuedFraction(val: float, limitIter: int, limitPrecision: float = 1e-5) -> list[int]:
        res = []
        intPart = int(val)
        while limitIter:
            limitIter -= 1
            res.append(intPart)
            val -= intPart
            if abs(val) < limitPrecision:
                break
            val = 1.0 / val
            intPart = int(val)
        return res

    @staticmethod
    def getFractions(contFrac: list[int]) -> tuple[list[int], list[int]]:
        nums, denoms = [], []
        n2, n1, d2, d1 = 0, 1, 1, 0
        for c in contFrac:
            n, d = c * n1 + n2, c * d1 + d2
            nums.append(n)
            denoms.append(d)
            n2, d2, n1, d1 = n1, d1, n, d
        return nums, denoms

    def factorize(self, numAttempts: int = 10) -> tuple[bool, int, int]:
        """(quantum period finding used, p1, p2) as ShorAlgorithmBase::factorize (ShorAlgorithm.h:120-212)"""
        C = self.Number
        if C > 22:
            return False, 0, 0
        if C % 2 == 0:
            return False, 2, C // 2
        sq = int(round(math.sqrt(C)))
        if sq * sq == C:
            return False, sq, sq
        L = self.fx.getFunctionStartQubit()
        xmask = (1 << L) - 1
        for _ in range(numAttempts):
            a = int(self._rng.integers(2, C))  # uniform on [2, C - 1]
            g = self.gcd(C, a)
            if g > 1:
                return False, g, C // g
            self.setA(a)
            state = self.Execute() & xmask
            while not state:
                state = self.Execute() & xmask
            _, divs = self.getFractions(self.continuedFraction(state / (1 << L), L))
            for p in divs[1:]:
                if p % 2:
                    p *= 2
                while p < C:
                    if self.fx.mod(a ** p) == 1:
                        m = self.fx.mod(a ** (p // 2))
                        if m != 1 and m != C - 1:
                            p1, p2 = self.gcd(m - 1, C), self.gcd(m + 1, C)
                            t1, t2 = C // p1, C // p2
                            if p1 * t1 == C:
                                p2 = t1
                            else:
                                p1 = t2
                            return True, p1, p2
                    p *= 2
        return False, 1, C
