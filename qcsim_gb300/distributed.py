"""QCSim's distributed-gate protocols over the engine: Distributed::DistributedCU / DistributedCNOT
(DistributedCNOT.h:9-79), a controlled gate between two parties built from one shared Bell pair, two
measurements and classically controlled corrections, and Distributed::TeleportedCNOT (TeleportedCNOT.h:11-80),
a CNOT applied between two teleported qubits.  Each gate and each mid-circuit measurement is one engine call.
"""
from __future__ import annotations

from . import gates as G
from .algorithms import QuantumAlgorithm


class DistributedCU(QuantumAlgorithm):
    """Distributed::DistributedCU (DistributedCNOT.h:9-66): the control on ctrlq and the target on targetq are
    held by different parties, which share the Bell pair (entq1, entq2).  Returns the two measured bits
    (entq2's in bit 1, entq1's in bit 0)."""

    def __init__(self, nrQubits: int = 4, ctrlq: int = 0, targetq: int = 3, entq1: int = 1, entq2: int = 2,
                 addseed: int = 0, cU=None, **kw):
        super().__init__(nrQubits, addseed, **kw)
        self.ctrlQubit, self.targetQubit = ctrlq, targetq
        self.entQubit1, self.entQubit2 = entq1, entq2
        self.cnot = G.CNOTGate()
        self.cU = cU if cU is not None else G.CNOTGate()
        self.hadamard = G.HadamardGate()
        self.x = G.PauliXGate()
        self.z = G.PauliZGate()
        self.setToBasisState(0)

    def Execute(self) -> int:
        e1, e2 = self.entQubit1, self.entQubit2
        self.ApplyGates([(self.hadamard, e1), (self.cnot, e2, e1), (self.cnot, e1, self.ctrlQubit)])
        m1 = self.Measure(e1)
        if m1:
            self.ApplyGate(self.x, e2)
        self.ApplyGates([(self.cU, self.targetQubit, e2), (self.hadamard, e2)])
        m2 = self.Measure(e2)
        if m2:
            self.ApplyGate(self.z, self.ctrlQubit)
        return (m2 << 1) | m1


class DistributedCNOT(DistributedCU):
    """Distributed::DistributedCNOT (DistributedCNOT.h:68-79): control on qubit 0, target on qubit 3, the Bell
    pair on qubits 1 and 2"""

    def __init__(self, addseed: int = 0, **kw):
        super().__init__(4, 0, 3, 1, 2, addseed, **kw)


class TeleportedCNOT(QuantumAlgorithm):
    """Distributed::TeleportedCNOT (TeleportedCNOT.h:11-80): six qubits; the target on qubit 0 and the control on
    qubit 5 are teleported through the Bell pairs (1, 2) and (3, 4) while a CNOT acts between qubits 2 and 3;
    the corrections from the four measured bits leave CNOT(target, control) on qubits 2 (target) and 3
    (control).  Returns measurements1 | measurements2 << 4."""

    def __init__(self, addseed: int = 0, **kw):
        super().__init__(6, addseed, **kw)
        self.cnot = G.CNOTGate()
        self.hadamard = G.HadamardGate()
        self.x = G.PauliXGate()
        self.z = G.PauliZGate()
        self.setToBasisState(0)

    def Execute(self) -> int:
        h, cx = self.hadamard, self.cnot
        self.ApplyGates([(h, 1), (cx, 2, 1), (h, 3), (cx, 4, 3), (cx, 2, 3), (cx, 1, 0), (h, 0), (cx, 4, 5), (h, 5)])
        m1 = self.Measure(0, 1)
        m2 = self.Measure(4, 5)
        fix = []
        if m2 & 1:
            fix += [(self.x, 2), (self.x, 3)]
        if m2 & 2:
            fix.append((self.z, 3))
        if m1 & 2:
            fix.append((self.x, 2))
        if m1 & 1:
            fix += [(self.z, 2), (self.z, 3)]
        if fix:
            self.ApplyGates(fix)
        return m1 | (m2 << 4)
