"""QCSim's teleportation family over the engine: the cat entangler / disentangler sub-algorithms
(CatEntangler.h, CatDisentangler.h), Bell-state preparation (QC::BellState, Utils.h:9-52), the teleportation
sub-algorithm QC::SubAlgo::Teleport and the algorithms Teleportation::QuantumTeleportation /
QuantumTeleportationRealization (Teleportation.h:10-198), entanglement swapping
(Teleportation::EntanglementSwapping, EntanglementSwapping.h:17-57) and superdense coding (Coding::SuperdenseCoding,
SuperdenseCoding.h:15-104).

They are small circuits with mid-circuit measurements: every gate and measurement is one engine call on
the register's stream, in the reference's order, and the classical bits that steer later gates come back
from the device measurement.
"""
from __future__ import annotations

from . import gates as G
from .algorithms import INT_MAX, QuantumAlgorithm, QuantumSubAlgorithmOnSubregister


def _parity(v: int) -> int:
    return bin(v).count("1") & 1


class CatEntangler(QuantumSubAlgorithmOnSubregister):
    """QC::SubAlgo::CatEntangler (CatEntangler.h:11-41): a Hadamard on the first qubit of the range, then a
    CNOT chain down the range, giving (|0..0> + |1..1>)/sqrt(2) from |0..0>"""

    def __init__(self, N: int, startQubit: int = 0, endQubit: int = INT_MAX):
        super().__init__(N, startQubit, endQubit)
        self.hadamard = G.HadamardGate()
        self.cnot = G.CNOTGate()

    def Execute(self, reg) -> int:
        s, e = self.getStartQubit(), self.getEndQubit()
        reg.ApplyGates([(self.hadamard, s)] + [(self.cnot, q + 1, q) for q in range(s, e)])
        return 0


class CatDisentangler(QuantumSubAlgorithmOnSubregister):
    """QC::SubAlgo::CatDisentangler (CatDisentangler.h:11-52): Hadamards on the range, a measurement of it, and
    a Z on the restored qubit when the measured bits have odd parity; returns the measurement"""

    def __init__(self, N: int, restoredQubit: int = 0, startQubit: int = 1, endQubit: int = INT_MAX):
        super().__init__(N, startQubit, endQubit)
        self.rQubit = restoredQubit
        self.hadamard = G.HadamardGate()
        self.z = G.PauliZGate()

    def Execute(self, reg) -> int:
        s, e = self.getStartQubit(), self.getEndQubit()
        reg.ApplyGates([(self.hadamard, q) for q in range(s, e + 1)])
        measurement = reg.Measure(s, e)
        if _parity(measurement):
            reg.ApplyGate(self.z, self.rQubit)
        return measurement


class BellState:
    """QC::BellState (Utils.h:9-52): |s2 s1> on (qubit2, qubit1), then H on qubit1 and CNOT(qubit2 <- qubit1)"""

    def __init__(self):
        self.hadamard = G.HadamardGate()
        self.cnot = G.CNOTGate()

    def setBellState(self, reg, qubit1: int = 0, qubit2: int = 1, s1: bool = False, s2: bool = False) -> bool:
        if qubit1 == qubit2 or qubit1 >= reg.getNrQubits() or qubit2 >= reg.getNrQubits():
            return False
        reg.setToBasisState(((1 << qubit1) if s1 else 0) | ((1 << qubit2) if s2 else 0))
        reg.ApplyGates([(self.hadamard, qubit1), (self.cnot, qubit2, qubit1)])
        return True

    def setBellState00(self, reg, qubit1: int = 0, qubit2: int = 1) -> bool:
        return self.setBellState(reg, qubit1, qubit2, False, False)

    def setBellState01(self, reg, qubit1: int = 0, qubit2: int = 1) -> bool:
        return self.setBellState(reg, qubit1, qubit2, False, True)

    def setBellState10(self, reg, qubit1: int = 0, qubit2: int = 1) -> bool:
        return self.setBellState(reg, qubit1, qubit2, True, False)

    def setBellState11(self, reg, qubit1: int = 0, qubit2: int = 1) -> bool:
        return self.setBellState(reg, qubit1, qubit2, True, True)


class Teleport(QuantumSubAlgorithmOnSubregister):
    """QC::SubAlgo::Teleport (Teleportation.h:163-194): a cat state on (entangled, target), CNOT from the
    source onto the entangled qubit, a measurement of the entangled qubit with an X on the target when it is
    1, and the cat disentangler on the source restoring the target; returns measurement2 | measurement << 1"""

    def __init__(self, N: int = 3, sourceQubit: int = 0, entangledQubit: int = 1, targetQubit: int = 2):
        super().__init__(N, entangledQubit, targetQubit)
        self.sQubit_ = sourceQubit
        self.cnot = G.CNOTGate()
        self.x = G.PauliXGate()
        self.entangler = CatEntangler(N, entangledQubit, targetQubit)
        self.disentangler = CatDisentangler(N, targetQubit, sourceQubit, sourceQubit)

    def Execute(self, reg) -> int:
        ent, target = self.getStartQubit(), self.getEndQubit()
        self.entangler.Execute(reg)
        reg.ApplyGate(self.cnot, ent, self.sQubit_)
        measurement = reg.MeasureQubit(ent)
        if measurement:
            reg.ApplyGate(self.x, target)
        measurement2 = self.disentangler.Execute(reg)
        return measurement2 | (measurement << 1)


class QuantumTeleportation(QuantumAlgorithm):
    """Teleportation::QuantumTeleportation (Teleportation.h:10-103)"""

    def __init__(self, N: int = 3, addseed: int = 0, **kw):
        super().__init__(N, addseed, **kw)
        self.hadamard = G.HadamardGate()
        self.cnot = G.CNOTGate()
        self.x = G.PauliXGate()
        self.z = G.PauliZGate()
        self.cz = G.ControlledZGate()
        self.setToBasisState(0)

    def Entangle(self, q1: int = 1, q2: int = 2) -> None:
        """an EPR pair on (q1, q2): H on q1, CNOT(q2 <- q1)"""
        self.ApplyGates([(self.hadamard, q1), (self.cnot, q2, q1)])

    def ApplyTeleportationCircuit(self, sentQubit: int = 0, q2: int = 1) -> None:
        """CNOT(q2 <- sent), H on sent: the Bell-basis change before the measurements"""
        self.ApplyGates([(self.cnot, q2, sentQubit), (self.hadamard, sentQubit)])

    def RestoreState(self, sentQubitMeasurement: bool, firstEntangledQubitMeasurement: bool, targetQubit: int = 2) -> None:
        if firstEntangledQubitMeasurement:
            self.ApplyGate(self.x, targetQubit)
        if sentQubitMeasurement:
            self.ApplyGate(self.z, targetQubit)

    def Teleport(self, sentQubit: int = 0, firstEntangledQubit: int = 1, targetQubit: int = 2,
                 explicitClassicalTransmission: bool = False) -> int:
        """Teleportation.h:53-88: returns the two measured bits (sent qubit in bit 0); Bob's correction is
        either the classically controlled X / Z or the coherent CNOT + CZ"""
        self.Entangle(firstEntangledQubit, targetQubit)
        self.ApplyTeleportationCircuit(sentQubit, firstEntangledQubit)
        measuredValues = self.Measure(sentQubit)
        measuredValues |= self.Measure(firstEntangledQubit) << 1
        if explicitClassicalTransmission:
            self.RestoreState(bool(measuredValues & 1), bool(measuredValues & 2), targetQubit)
        else:
            self.ApplyGates([(self.cnot, targetQubit, firstEntangledQubit), (self.cz, targetQubit, sentQubit)])
        return measuredValues


class QuantumTeleportationRealization(QuantumTeleportation):
    """Teleportation::QuantumTeleportationRealization (Teleportation.h:107-149): three qubits, the state to
    send on qubit 0, Bob's qubit 2"""

    def __init__(self, addseed: int = 0, **kw):
        super().__init__(3, addseed, **kw)

    def SetState(self, alpha: complex, beta: complex) -> None:
        self.Clear()
        self.setRawAmplitude(0, alpha)
        self.setRawAmplitude(1, beta)
        self.Normalize()

    def Teleport(self, explicitClassicalTransmission: bool = False) -> int:  # type: ignore[override]
        return super().Teleport(0, 1, 2, explicitClassicalTransmission)

    def Execute(self) -> int:
        self.Teleport()
        return self.Measure(2)


class EntanglementSwapping(QuantumTeleportation):
    """Teleportation::EntanglementSwapping (EntanglementSwapping.h:17-57): six qubits; a Bell pair on (0, 2)
    is swapped onto (4, 5) by teleporting qubit 0 through the pair (1, 4) and qubit 2 through (3, 5)"""

    def __init__(self, addseed: int = 0, **kw):
        super().__init__(6, addseed, **kw)

    def SetBellStateToBeSent(self, s1: bool = False, s2: bool = False) -> None:
        BellState().setBellState(self.reg, 0, 2, s1, s2)

    def Teleport(self, explicitClassicalTransmission: bool = False) -> int:  # type: ignore[override]
        """the measured bits of qubits 0..3"""
        res = super().Teleport(0, 1, 4, explicitClassicalTransmission)
        return res | (super().Teleport(2, 3, 5, explicitClassicalTransmission) << 2)

    def Execute(self) -> int:
        self.Teleport()
        return self.Measure(4, 5)


class SuperdenseCoding(QuantumAlgorithm):
    """Coding::SuperdenseCoding (SuperdenseCoding.h:15-104): two classical bits sent on one qubit of a Bell
    pair; Alice applies X (bit2) and Z (bit1) to qubit 0, Bob decodes with CNOT(1 <- 0) and H on 0, and the
    measurement returns bit1 in bit 0 and bit2 in bit 1"""

    def __init__(self, addseed: int = 0, **kw):
        super().__init__(2, addseed, **kw)
        self.b1 = self.b2 = False
        self.bellState = BellState()
        self.hadamard = G.HadamardGate()
        self.cnot = G.CNOTGate()
        self.x = G.PauliXGate()
        self.z = G.PauliZGate()

    def Send(self, bit1: bool, bit2: bool) -> None:
        self.bellState.setBellState00(self.reg)
        gates = ([(self.x, 0)] if bit2 else []) + ([(self.z, 0)] if bit1 else [])
        if gates:
            self.ApplyGates(gates)

    def Receive(self) -> int:
        self.ApplyGates([(self.cnot, 1, 0), (self.hadamard, 0)])
        return self.Measure()

    def SetBits(self, bit1: bool, bit2: bool) -> None:
        self.b1, self.b2 = bool(bit1), bool(bit2)

    def Execute(self) -> int:
        self.Send(self.b1, self.b2)
        return self.Receive()
