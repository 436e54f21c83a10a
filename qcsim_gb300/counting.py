"""QCSim's quantum counting over the engine: QuantumCounting::QuantumCountingAlgorithm
(QuantumCountingAlgorithm.h:26-200) with the n-controlled NOT it is built from,
QC::SubAlgo::NControlledNotWithAncilla (NControlledNotWithAncilla.h:13-150).

Counting runs 2^P - 1 controlled Grover iterations, each a few hundred gates, on P + 2G qubits.  The
reference applies them one ApplyGate at a time.  Here the whole controlled-Grover part is built on the host
as one gate list, in the reference's order and with the reference's record / replay of the ancilla
computation (ComputeStart / ComputeEnd / Uncompute, QubitRegister.h:536-590).  It goes to the engine as a
single ApplyGates call, which packs the gates into shared-memory passes.  The inverse QFT on the precision
qubits follows as one qcs_qft call.
"""
from __future__ import annotations

import math

import numpy as np

from . import gates as G
from .algorithms import INT_MAX, QuantumAlgorithm, QuantumFourierTransform, QuantumSubAlgorithmOnSubregister


class GateSequence:
    """A host-side gate list with the register's record / replay interface (ApplyGate, ComputeStart,
    ComputeEnd, Uncompute), so that sub-algorithms written against a register can append to it.  Uncompute
    appends the recorded gates in reverse order, each replaced by its adjoint; a self-adjoint gate (CNOT,
    Toffoli) is appended as itself."""

    def __init__(self):
        self.ops: list[tuple] = []
        self._recorded: list[tuple] = []
        self._recording = False

    def ApplyGate(self, gate, qubit: int, controllingQubit1: int = 0, controllingQubit2: int = 0) -> None:
        op = (gate, qubit, controllingQubit1, controllingQubit2)
        self.ops.append(op)
        if self._recording:
            self._recorded.append(op)

    def ComputeStart(self) -> None:
        self._recording = True
        self._recorded = []

    def ComputeEnd(self) -> None:
        self._recording = False

    def Uncompute(self) -> None:
        for gate, q0, q1, q2 in reversed(self._recorded):
            m = gate.getRawOperatorMatrix()
            adj = m.conj().T
            self.ops.append((gate if np.array_equal(adj, m) else G.AppliedGate(adj, q0, q1, q2), q0, q1, q2))


class NControlledNotWithAncilla(QuantumSubAlgorithmOnSubregister):
    """QC::SubAlgo::NControlledNotWithAncilla (NControlledNotWithAncilla.h:13-150): a NOT on the target
    controlled by any number of qubits.  One or two controls map to CNOT / Toffoli.  For more controls,
    Toffolis AND pairs of controls into fresh ancillas, then pairs of ancillas into further ancillas, until
    one Toffoli (or CNOT) reaches the target.  With clearAncillaAtTheEnd the ancilla computation is recorded
    and undone afterwards."""

    def __init__(self, N: int = INT_MAX, startQubit: int = 0, endQubit: int = INT_MAX):
        super().__init__(N, startQubit, endQubit)
        self.targetQubit = 0
        self.startAncillaQubits = 1
        self.clearAncillaAtTheEnd = True
        self.controlQubits: list[int] = []
        self.cnot = G.CNOTGate()
        self.ccnot = G.ToffoliGate()

    def Execute(self, reg) -> int:
        cq = self.controlQubits
        if not cq:
            return 1
        if len(cq) == 2:
            reg.ApplyGate(self.ccnot, self.targetQubit, cq[0], cq[1])
            return 0
        if len(cq) == 1:
            reg.ApplyGate(self.cnot, self.targetQubit, cq[0])
            return 0
        clear = self.clearAncillaAtTheEnd
        if clear:
            reg.ComputeStart()
        free = self.startAncillaQubits
        for i in range(0, len(cq) - 1, 2):
            reg.ApplyGate(self.ccnot, free, cq[i], cq[i + 1])
            free += 1
        anc = self.startAncillaQubits
        if len(cq) % 2:
            if free == self.startAncillaQubits + 1:
                if clear:
                    reg.ComputeEnd()
                reg.ApplyGate(self.ccnot, self.targetQubit, cq[-1], anc)
                if clear:
                    reg.Uncompute()
                return 0
            reg.ApplyGate(self.ccnot, free, cq[-1], anc)
            free += 1
            anc += 1
        while free - anc > 2:
            reg.ApplyGate(self.ccnot, free, anc, anc + 1)
            free += 1
            anc += 2
        if clear:
            reg.ComputeEnd()
        if free - anc == 2:
            reg.ApplyGate(self.ccnot, self.targetQubit, anc, anc + 1)
        else:
            reg.ApplyGate(self.cnot, self.targetQubit, anc)
        if clear:
            reg.Uncompute()
        return 0

    def GetControlQubits(self) -> list[int]:
        return self.controlQubits

    def SetControlQubits(self, cq) -> None:
        self.controlQubits = list(cq)

    def GetTargetQubit(self) -> int:
        return self.targetQubit

    def SetTargetQubit(self, tq: int) -> None:
        self.targetQubit = tq

    def GetStartAncillaQubits(self) -> int:
        return self.startAncillaQubits

    def SetStartAncillaQubits(self, saq: int) -> None:
        self.startAncillaQubits = saq

    def ClearAncillaAtTheEnd(self) -> bool:
        return self.clearAncillaAtTheEnd

    def SetClearAncillaAtTheEnd(self, v: bool) -> None:
        self.clearAncillaAtTheEnd = bool(v)


class QuantumCountingAlgorithm(QuantumAlgorithm):
    """QuantumCounting::QuantumCountingAlgorithm (QuantumCountingAlgorithm.h:26-200): phase estimation of the
    Grover operator over G qubits with P precision qubits; the register is P + 2G qubits (precision, Grover,
    then G ancillas, the first of them the oracle's phase-kickback qubit).  The measured precision value x
    gives theta = x / 2^P (folded below 1/2) and the count round(2^G sin^2(pi theta))."""

    def __init__(self, PrecisionQubits: int = 6, GroverQubits: int = 4, addseed: int = 0, **kw):
        assert PrecisionQubits >= 3 and GroverQubits >= 1
        super().__init__(PrecisionQubits + 2 * GroverQubits, addseed, **kw)
        self.precisionQubits = PrecisionQubits
        self.groverQubits = GroverQubits
        self.fourier = QuantumFourierTransform(PrecisionQubits, 0, PrecisionQubits - 1)
        self.markedStates: set[int] = set()
        first = PrecisionQubits + GroverQubits
        self.nControlledNOT = NControlledNotWithAncilla()
        self.nControlledNOT.SetTargetQubit(first)
        self.nControlledNOT.SetStartAncillaQubits(first + 1)
        self.hadamard = G.HadamardGate()
        self.chadamard = G.ControlledHadamardGate()
        self.x = G.PauliXGate()
        self.cx = G.CNOTGate()

    def Execute(self) -> int:
        self.ExecuteWithoutMeasurement()
        return self.Measure(0, self.precisionQubits - 1)

    def ExecuteWithMultipleMeasurements(self, nrMeasurements: int = 10000) -> dict:
        self.ExecuteWithoutMeasurement()
        return self.RepeatedMeasure(0, self.precisionQubits - 1, nrMeasurements)

    def ClearMarkedStates(self) -> None:
        self.markedStates.clear()

    def AddMarkedState(self, state: int) -> None:
        if state < (1 << self.groverQubits):
            self.markedStates.add(int(state))

    def SetMarkedStates(self, states) -> None:
        self.ClearMarkedStates()
        for s in states:
            self.AddMarkedState(s)

    def GetNumberOfMarkedStates(self) -> int:
        return len(self.markedStates)

    def GetCorrectThetaForMarkedStates(self) -> float:
        return math.asin(math.sqrt(self.GetNumberOfMarkedStates() / (1 << self.groverQubits))) / math.pi

    def GetThetaForState(self, state: int) -> float:
        theta = state / (1 << self.precisionQubits)
        return 1.0 - theta if theta >= 0.5 else theta

    def GetCountForState(self, state: int) -> int:
        s = math.sin(math.pi * self.GetThetaForState(state))
        return int(math.floor((1 << self.groverQubits) * s * s + 0.5))  # C's round, half away from zero

    def circuit(self) -> list[tuple]:
        """the gates of ExecuteWithoutMeasurement before the inverse QFT (QuantumCountingAlgorithm.h:104-128),
        as (gate, q0, q1, q2) tuples"""
        seq = GateSequence()
        first = self.precisionQubits + self.groverQubits
        for q in range(first):
            seq.ApplyGate(self.hadamard, q)
        seq.ApplyGate(self.x, first)
        seq.ApplyGate(self.hadamard, first)
        for q in range(self.precisionQubits):
            ctrl = self.precisionQubits - q - 1
            for _ in range(1 << q):
                self._controlled_grover(seq, ctrl)
        seq.ApplyGate(self.hadamard, first)
        seq.ApplyGate(self.x, first)
        return seq.ops

    def ExecuteWithoutMeasurement(self) -> None:
        self.setToBasisState(0)
        self.ApplyGates(self.circuit())
        self.fourier.IQFT(self.reg, False)

    def _controlled_grover(self, seq: GateSequence, ctrl: int) -> None:
        for state in sorted(self.markedStates):
            self._controlled_oracle(seq, ctrl, state)
        self._controlled_diffusion(seq, ctrl)

    def _controlled_oracle(self, seq: GateSequence, ctrl: int, state: int) -> None:
        """flip the kickback qubit where the Grover register holds state and ctrl is set
        (QuantumCountingAlgorithm.h:137-164)"""
        p = self.precisionQubits
        flips = [p + q for q in range(self.groverQubits) if not (state >> q) & 1]
        for t in flips:
            seq.ApplyGate(self.cx, t, ctrl)
        self.nControlledNOT.SetControlQubits(list(range(p, p + self.groverQubits)) + [ctrl])
        self.nControlledNOT.Execute(seq)
        for t in flips:
            seq.ApplyGate(self.cx, t, ctrl)

    def _controlled_diffusion(self, seq: GateSequence, ctrl: int) -> None:
        """QuantumCountingAlgorithm.h:167-179"""
        p = self.precisionQubits
        for q in range(self.groverQubits):
            seq.ApplyGate(self.chadamard, p + q, ctrl)
        for state in range(1, 1 << self.groverQubits):
            self._controlled_oracle(seq, ctrl, state)
        for q in range(self.groverQubits):
            seq.ApplyGate(self.chadamard, p + q, ctrl)
