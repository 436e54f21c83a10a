"""QCSim's algorithm base and the sub-algorithms of the statevector hot path over the engine register:
QuantumAlgorithm (QuantumAlgorithm.h:9-205, the owner of a register that its algorithms derive from),
QubitsSwapper (QubitsSwapper.h:10-43), QuantumFourierTransform (QuantumFourierTransform.h:12-92),
OneQubitGateTransform / HadamardTransform / XTransform (HadamardTransform.h:9-41), and the dense operator
gates NQubitsQuantumGate (NQubitsQuantumGate.h:9-78) / NQubitsControlledQuantumGate
(NQubitsControlledQuantumGate.h:9-97), on the qubit range of QuantumSubAlgorithmOnSubregister
(QuantumAlgorithm.h:222-239).

The QFT runs as one engine call (qcs_qft), which applies the reference's gate sequence; the one-qubit
transforms run as one gate list (qcs_one_qubit_transform); the dense operator gates run as one
qcs_apply_operator_on_qubits call on their 2^k x 2^k operator.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import gates as G
from .register import QubitRegister

INT_MAX = 2**31 - 1


class QuantumSubAlgorithmOnSubregister:
    """QuantumSubAlgorithmOnSubregister (QuantumAlgorithm.h:222-239)"""

    def __init__(self, N: int, startQubit: int = 0, endQubit: int = INT_MAX):
        self.sQubit = startQubit
        self.eQubit = max(startQubit, min(N - 1, endQubit))

    def getStartQubit(self) -> int:
        return self.sQubit

    def getEndQubit(self) -> int:
        return self.eQubit


class QubitsSwapper(QuantumSubAlgorithmOnSubregister):
    """mirror swaps of [start, end] (QubitsSwapper.h:23-34)"""

    def __init__(self, N: int, startQubit: int = 0, endQubit: int = INT_MAX):
        super().__init__(N, startQubit, endQubit)
        self.swapOp = G.SwapGate()

    def Swap(self, reg) -> None:
        a, b = self.getStartQubit(), self.getEndQubit()
        ops = []
        while a < b:
            ops.append((self.swapOp, a, b, 0))
            a, b = a + 1, b - 1
        if ops:
            reg.ApplyGates(ops)

    def Execute(self, reg) -> int:
        self.Swap(reg)
        return reg.MeasureAll()


class QuantumFourierTransform(QubitsSwapper):
    """QFT / IQFT of QuantumFourierTransform.h:35-87; Execute measures after the transform"""

    def __init__(self, N: int, startQubit: int = 0, endQubit: int = INT_MAX):
        super().__init__(N, startQubit, endQubit)
        self.hadamard = G.HadamardGate()
        self.cPhaseShift = G.ControlledPhaseShiftGate()

    def Execute(self, reg) -> int:
        self.QFT(reg)
        return reg.MeasureAll()

    def _run(self, reg, inverse: bool, doSwap: bool) -> None:
        if reg.recordGates:
            # recording registers need the individual gates in their log
            from .circuits import qft_circuit
            for op in qft_circuit(self.getStartQubit(), self.getEndQubit(), inverse, doSwap):
                reg.ApplyGate(*op)
            return
        reg._ck(reg._lib.qcs_qft(reg.handle, self.getStartQubit(), self.getEndQubit(), int(inverse), int(doSwap)))

    def QFT(self, reg, doSwap: bool = True) -> None:
        self._run(reg, False, doSwap)

    def IQFT(self, reg, doSwap: bool = True) -> None:
        self._run(reg, True, doSwap)


class OneQubitGateTransform(QuantumSubAlgorithmOnSubregister):
    """the same one-qubit gate on every qubit of [start, end] (HadamardTransform.h:9-35)"""

    gate_class = G.HadamardGate

    def __init__(self, N: int, startQubit: int = 0, endQubit: int = INT_MAX, gate=None):
        super().__init__(N, startQubit, endQubit)
        self.gate = gate if gate is not None else self.gate_class()

    def Execute(self, reg) -> int:
        self.ApplyHadamardOnAllQubits(reg)
        return 0

    def ApplyHadamardOnAllQubits(self, reg) -> None:
        if reg.recordGates:
            for q in range(self.getStartQubit(), self.getEndQubit() + 1):
                reg.ApplyGate(self.gate, q)
            return
        m = np.ascontiguousarray(self.gate.getRawOperatorMatrix(), dtype=np.complex128)
        reg._ck(reg._lib.qcs_one_qubit_transform(reg.handle, m.view(np.float64).ctypes.data_as(C.POINTER(C.c_double)),
                                                 self.gate.traits(), self.getStartQubit(), self.getEndQubit()))


class HadamardTransform(OneQubitGateTransform):
    gate_class = G.HadamardGate


class XTransform(OneQubitGateTransform):
    gate_class = G.PauliXGate


def _operator_qubits(op) -> int:
    """getOperatorQubitsNumber (NQubitsQuantumGate.h:61-72): the bit length of rows - 1"""
    return int(op.shape[0] - 1).bit_length()


class NQubitsQuantumGate(QuantumSubAlgorithmOnSubregister):
    """SubAlgo::NQubitsQuantumGate: a dense 2^k x 2^k operator on qubits startQubit .. startQubit + k - 1.

    The reference's Execute (NQubitsQuantumGate.h:20-25) builds the 2^N x 2^N extended matrix and applies
    it with ApplyOperatorMatrix; here the operator itself goes to the device (ApplyOperatorOnQubits), and
    the extended matrix is built only for a register that records its gates (the log then holds what the
    reference's log holds).  The reference's end qubit is startQubit + k clamped to N - 1
    (QuantumAlgorithm.h:228-231), so its extended matrix stays within the operator's bounds only when the
    operator reaches the top qubit (startQubit + k = N, the placement PhaseEstimation uses); there the two
    agree exactly, and elsewhere this class applies the operator on its k qubits."""

    def __init__(self, N: int, op, startQubit: int = 0):
        self.U = np.array(op, dtype=np.complex128)
        k = _operator_qubits(self.U)
        if self.U.shape != (1 << k, 1 << k) or startQubit + k > N:
            raise ValueError("the operator must be 2^k x 2^k and fit on qubits startQubit .. N - 1")
        super().__init__(N, startQubit, startQubit + k)
        self.nrQubits = N

    def targets(self) -> list[int]:
        return list(range(self.getStartQubit(), self.getStartQubit() + self.getRawOperatorQubitsNumber()))

    def controls(self) -> list[int]:
        return []

    def Execute(self, reg) -> int:
        if reg.recordGates:
            reg.ApplyOperatorMatrix(self.getOperatorMatrix())
        else:
            reg.ApplyOperatorOnQubits(self.U, self.targets(), self.controls())
        return 0

    def getOperatorMatrix(self) -> np.ndarray:
        """the 2^N x 2^N extended matrix: identity on the other qubits (and, controlled, where the control
        is zero)"""
        s, k = self.getStartQubit(), self.getRawOperatorQubitsNumber()
        ext = np.kron(np.eye(1 << (self.nrQubits - s - k)), np.kron(self.U, np.eye(1 << s)))
        for c in self.controls():
            on = ((np.arange(1 << self.nrQubits) >> c) & 1).astype(bool)
            ext = np.where(np.outer(on, on), ext, np.eye(1 << self.nrQubits))
        return ext

    def getRawOperatorMatrix(self) -> np.ndarray:
        return self.U

    def getRawOperatorQubitsNumber(self) -> int:
        return _operator_qubits(self.U)


class NQubitsControlledQuantumGate(NQubitsQuantumGate):
    """SubAlgo::NQubitsControlledQuantumGate (NQubitsControlledQuantumGate.h:9-97): the operator where the
    controlling qubit is one, the identity where it is zero"""

    def __init__(self, N: int, op, startQubit: int = 1, controllingQubit: int = 0):
        super().__init__(N, op, startQubit)
        if startQubit <= controllingQubit < startQubit + self.getRawOperatorQubitsNumber() or controllingQubit >= N:
            raise ValueError("the controlling qubit must be outside the operator's qubits")
        self.ctrlQubit = controllingQubit

    def controls(self) -> list[int]:
        return [self.ctrlQubit]

    def getNrQubits(self) -> int:
        return self.nrQubits


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
