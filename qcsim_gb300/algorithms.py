"""Sub-algorithms of the hot path, mirroring QCSim's QC::SubAlgo classes over the engine:
QuantumFourierTransform (QuantumFourierTransform.h:12-92), QubitsSwapper (QubitsSwapper.h:10-43) and
OneQubitGateTransform / HadamardTransform / XTransform (HadamardTransform.h:9-41).

The QFT runs as one engine call (qcs_qft), which applies the reference's gate sequence; the one-qubit
transforms run as one gate list (qcs_one_qubit_transform).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import gates as G

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
