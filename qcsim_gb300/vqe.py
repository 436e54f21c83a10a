"""QCSim's variational quantum eigensolver (VQE.h) over the engine: Pauli-string terms whose energies are
estimated from sampled measurements (RepeatedMeasure), a RY/RZ + CNOT-ring ansatz, and the Nelder-Mead
search of VariationalQuantumEigensolver.  The arithmetic follows the reference line by line, including
its energy estimate, which takes the parity of every measured bit (VQE.h:116-142)."""
from __future__ import annotations

import math

from . import gates as G
from .algorithms import QuantumAlgorithm


class PauliStringVQE:
    """VQE::PauliStringVQE (VQE.h:21-150): one Pauli string (an operator 'X', 'Y' or 'Z' per qubit, Z by default as
    in the reference's PauliString, PauliString.h:15) with a coefficient.  The reference's energy estimate takes the
    parity of every qubit, so a qubit left at Z (or given 'I', accepted as a synonym here) enters it as Z."""

    _CODES = {0: "Z", 1: "X", 2: "Y"}  # PauliString::PauliOp (PauliString.h:8-13)

    def __init__(self, nrQubits: int):
        self.ops = ["Z"] * nrQubits
        self.coefficient = 1.0
        self.rx, self.ry = G.RxGate(0.5 * math.pi), G.RyGate(-0.5 * math.pi)
        self.cnot = G.CNOTGate()

    def setOperatorForQubit(self, qubit: int, op) -> None:
        """op: 'X', 'Y', 'Z' (or 'I', the same as Z here), or the reference's PauliOp code 0 = Z, 1 = X, 2 = Y"""
        op = self._CODES.get(op, op) if isinstance(op, int) else op
        if op not in ("I", "X", "Y", "Z"):
            raise ValueError("Pauli operator must be X, Y or Z (or I)")
        if qubit < len(self.ops):
            self.ops[qubit] = op

    def getOperatorForQubit(self, qubit: int) -> str:
        return self.ops[qubit]

    def getCoefficient(self) -> float:
        return self.coefficient

    def setCoefficient(self, c: float) -> None:
        self.coefficient = c

    def Execute(self, reg) -> int:
        """rotate each qubit into the measured operator's eigenbasis (VQE.h:33-44)"""
        for q in range(reg.getNrQubits()):
            op = self.getOperatorForQubit(q) if q < len(self.ops) else "Z"
            if op == "X":
                reg.ApplyGate(self.ry, q)
            elif op == "Y":
                reg.ApplyGate(self.rx, q)
        return 0

    def SingleQubitAnsatz(self, reg, qubit: int, theta: float, phi: float) -> None:
        reg.ApplyGate(G.RyGate(theta), qubit)
        reg.ApplyGate(G.RzGate(phi), qubit)


    def Ansatz(self, reg, params) -> None:
        """RY(theta) RZ(phi) on every qubit, then layers of a CNOT ring (alternating direction) followed by
        more single-qubit rotations while parameters remain (VQE.h:74-114)"""
        n = reg.getNrQubits()
        if len(params) < n:
            return
        pos = 0
        q = 0
        while q < n and pos < len(params) - 1:
            self.SingleQubitAnsatz(reg, q, params[pos], params[pos + 1])
            pos += 2
            q += 1
        flip = False
        while pos < len(params) - 1:
            if flip:
                for q in range(n - 1, 0, -1):
                    reg.ApplyGate(self.cnot, q - 1, q)
                if n > 2:
                    reg.ApplyGate(self.cnot, n - 1, 0)
            else:
                for q in range(n - 1):
                    reg.ApplyGate(self.cnot, q + 1, q)
                if n > 2:
                    reg.ApplyGate(self.cnot, 0, n - 1)
            flip = not flip
            q = 0
            while q < n and pos < len(params) - 1:
                self.SingleQubitAnsatz(reg, q, params[pos], params[pos + 1])
                pos += 2
                q += 1

    def EstimateEnergy(self, reg, params, nrMeasurements: int = 10000) -> float:
        reg.setToBasisState(0)
        self.Ansatz(reg, params)
        self.Execute(reg)
        energy = 0.0
        n = reg.getNrQubits()
        for state, count in reg.RepeatedMeasure(nrMeasurements).items():
            e = 1.0
            val, q = state, 0
            while val and q < n:
                if val & 1:
                    e = -e
                val >>= 1
                q += 1
            energy += e * count
        return self.getCoefficient() * energy / nrMeasurements


class VariationalQuantumEigensolver(QuantumAlgorithm):
    """VQE::VariationalQuantumEigensolver (VQE.h:157-487): Nelder-Mead over the ansatz parameters, the energy of a
    point being the sum of its terms' sampled energies"""

    def __init__(self, N: int = 2, addSeed: bool = False, **kw):
        super().__init__(N, int(addSeed), **kw)
        self.terms: list[PauliStringVQE] = []
        self.nrMeasurements = 10000
        self.vertices: list[list[float]] = []
        self.terminateLimit = 10
        self.delta = 0.0001
        self.vertexEnergies: list[float] = []

    def AddTerm(self, term: PauliStringVQE) -> None:
        self.terms.append(term)

    def Clear(self) -> None:
        self.terms.clear()

    def Execute(self) -> int:
        if not self.vertices:
            return 0
        self.EstimateEnergiesForVertices()
        old = self.GetMinEnergy()
        terminate = 0
        for _ in range(1000):
            self.NelderMeadStep()
            new = self.GetMinEnergy()
            terminate = terminate + 1 if abs(new - old) < self.delta else 0
            old = new
            if terminate >= self.terminateLimit:
                break
        return 0

    def EstimateEnergy(self, params, nrMeas: int = 10000) -> float:
        return sum(t.EstimateEnergy(self.reg, params, nrMeas) for t in self.terms)

    def SetNrMeasurements(self, n: int) -> None:
        self.nrMeasurements = n

    def GetNrMeasurements(self) -> int:
        return self.nrMeasurements

    def SetVertices(self, v) -> None:
        self.vertices = [list(p) for p in v]

    def GetVertices(self):
        return self.vertices

    def SetTerminateLimit(self, limit: int) -> None:
        self.terminateLimit = limit

    def GetTerminateLimit(self) -> int:
        return self.terminateLimit

    def SetDelta(self, d: float) -> None:
        self.delta = d

    def GetDelta(self) -> float:
        return self.delta

    def GetMinEnergy(self) -> float:
        return min(self.vertexEnergies) if self.vertexEnergies else 0.0

    def GetMinVertex(self):
        if not self.vertexEnergies:
            return []
        return self.vertices[min(range(len(self.vertexEnergies)), key=lambda i: (self.vertexEnergies[i], i))]

    def NelderMeadStep(self) -> None:
        """one step (VQE.h:287-381): reflect the worst vertex through the centroid of the others, then expand,
        contract or shrink"""
        if not self.vertices:
            return
        minE, maxE, maxE2, minI, maxI, _ = self.GetMinMaxEnergy()
        centroid = self.Centroid(self.vertices, maxI)
        refl = self.ReflectionPoint(self.vertices[maxI], centroid, 2.0)
        reflE = self.EstimateEnergy(refl, self.nrMeasurements)
        if reflE > maxE2:
            shrink = False
            if reflE < maxE:
                cp = self.ReflectionPoint(centroid, refl, 0.5)
                cE = self.EstimateEnergy(cp, self.nrMeasurements)
                if cE < reflE:
                    self.vertices[maxI], self.vertexEnergies[maxI] = cp, cE
                else:
                    self.vertices[maxI], self.vertexEnergies[maxI] = refl, reflE
                    shrink = True
            else:
                cp = self.ReflectionPoint(centroid, self.vertices[maxI], 0.5)
                cE = self.EstimateEnergy(cp, self.nrMeasurements)
                if cE < maxE:
                    self.vertices[maxI], self.vertexEnergies[maxI] = cp, cE
                else:
                    cp = self.ReflectionPoint(centroid, self.vertices[maxI], 1.5)
                    cE = self.EstimateEnergy(cp, self.nrMeasurements)
                    if cE < maxE:
                        self.vertices[maxI], self.vertexEnergies[maxI] = cp, cE
                    shrink = True
            if shrink:
                self.ShrinkVertices(minI)
        else:
            ep = self.ReflectionPoint(centroid, refl, 2.0)
            eE = self.EstimateEnergy(ep, self.nrMeasurements)
            if eE < reflE:
                self.vertices[maxI], self.vertexEnergies[maxI] = ep, eE
            else:
                self.vertices[maxI], self.vertexEnergies[maxI] = refl, reflE

    def ShrinkVertices(self, minIndex: int) -> None:
        for i in range(len(self.vertices)):
            if i == minIndex:
                continue
            self.vertices[i] = self.ReflectionPoint(self.vertices[minIndex], self.vertices[i], 0.5)
            self.vertexEnergies[i] = self.EstimateEnergy(self.vertices[i], self.nrMeasurements)

    @staticmethod
    def Centroid(points, excludeIndex: int = -1) -> list[float]:
        if not points:
            return []
        c = [0.0] * len(points[0])
        for pi, p in enumerate(points):
            if pi == excludeIndex:
                continue
            for i, x in enumerate(p):
                c[i] += x
        count = len(points) if excludeIndex == -1 else len(points) - 1
        return [x / count for x in c]

    @staticmethod
    def ReflectionPoint(p1, p2, alpha: float) -> list[float]:
        return [a + alpha * (b - a) for a, b in zip(p1, p2)]

    def EstimateEnergiesForVertices(self) -> None:
        self.vertexEnergies = [self.EstimateEnergy(v, self.nrMeasurements) for v in self.vertices]

    def GetMinMaxEnergy(self):
        """(minEnergy, maxEnergy, maxEnergy2, minIndex, maxIndex, maxIndex2) as VQE.h:418-452 finds them"""
        e = self.vertexEnergies
        maxE, maxI = e[0], 0
        maxE2, maxI2 = maxE, 0
        minE, minI = maxE, 0
        for i in range(1, len(e)):
            if e[i] > maxE:
                maxE2, maxI2 = maxE, maxI
                maxE, maxI = e[i], i
            elif e[i] < minE:
                minE, minI = e[i], i
        return minE, maxE, maxE2, minI, maxI, maxI2
