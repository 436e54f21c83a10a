"""QCSim's gate-built oracles over the engine: QC::SubAlgo::NControlledGatesWithAncilla
(NControlledGateWithAncilla.h:11-170), QC::Oracles::OracleWithGatesSimpleFunction and OracleWithGates
(Oracle.h:10-243), and the algorithms that use them in place of a 2^n x 2^n oracle matrix:
DeutschJozsaAlgorithmWithGatesOracle (DeutschJozsa.h:141-290), BernsteinVaziraniAlgorithmWithGatesOracle
(BernsteinVazirani.h:108-210) and SimonAlgorithmWithGatesOracle (SimonAlgorithm.h:250-367).

An oracle expands into X gates, Toffolis onto ancillas and controlled gates, one n-controlled operation per
basis state where the function is non-zero.  The whole expansion, with the ancilla computation recorded and
undone, is built on the host as one gate list (counting.GateSequence) and sent to the engine as one
ApplyGates call.
"""
from __future__ import annotations

import numpy as np

from . import gates as G
from .algorithms import (INT_MAX, DeutschJozsaAlgorithm, QuantumAlgorithm, QuantumSubAlgorithmOnSubregister,
                         SimonFunction)
from .counting import GateSequence, NControlledNotWithAncilla


class NControlledGatesWithAncilla(QuantumSubAlgorithmOnSubregister):
    """QC::SubAlgo::NControlledGatesWithAncilla (NControlledGateWithAncilla.h:11-170): one- or two-qubit gates
    controlled by any number of qubits.  With one control the gates take it directly; otherwise Toffolis AND the
    controls into ancillas (pairs, then the odd one with the first ancilla, then pairs of ancillas) and the last
    ancilla controls the gates; the ancilla computation is recorded and undone."""

    def __init__(self, N: int = INT_MAX, startQubit: int = 0, endQubit: int = INT_MAX):
        super().__init__(N, startQubit, endQubit)
        self.startAncillaQubits = 1
        self.clearAncillaAtTheEnd = True
        self.controlQubits: list[int] = []
        self.gates: list[list] = []  # [controlled matrix, q1, q2, q3]; the control goes into the last slot
        self.ccnot = G.ToffoliGate()

    def Execute(self, reg) -> int:
        cq = self.controlQubits
        if not cq:
            return 1
        if len(cq) == 1:
            self._apply_gates(reg, cq[0])
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
            reg.ApplyGate(self.ccnot, free, cq[-1], anc)
            free += 1
            anc += 1
        while free - anc > 1:
            reg.ApplyGate(self.ccnot, free, anc, anc + 1)
            free += 1
            anc += 2
        if clear:
            reg.ComputeEnd()
        self._apply_gates(reg, free - 1)
        if clear:
            reg.Uncompute()
        return 0

    def _apply_gates(self, reg, ctrl: int) -> None:
        for g in self.gates:
            m, q1, q2, q3 = g
            if m.shape[0] == 4:
                q2 = g[2] = ctrl
            else:
                q3 = g[3] = ctrl
            reg.ApplyGate(G.AppliedGate(m, q1, q2, q3), q1, q2, q3)

    def GetControlQubits(self) -> list[int]:
        return self.controlQubits

    def SetControlQubits(self, cq) -> None:
        self.controlQubits = list(cq)

    def GetStartAncillaQubits(self) -> int:
        return self.startAncillaQubits

    def SetStartAncillaQubits(self, saq: int) -> None:
        self.startAncillaQubits = saq

    def GetGates(self) -> list:
        return self.gates

    def AddGate(self, gate) -> bool:
        """the gate (an AppliedGate of one or two qubits) extended by one control as the top qubit: identity with
        the gate's matrix in the lower-right block (NControlledGateWithAncilla.h:116-147)"""
        k = gate.getQubitsNumber()
        m = np.asarray(gate.getRawOperatorMatrix(), dtype=np.complex128)
        if k not in (1, 2) or m.shape not in ((2, 2), (4, 4)):
            return False
        d = m.shape[0]
        op = np.eye(2 * d, dtype=np.complex128)
        op[d:, d:] = m
        self.gates.append([op, gate.getQubit1(), gate.getQubit2() if d == 4 else 0, 0])
        return True

    def ClearGates(self) -> None:
        self.gates = []

    def ClearAncillaAtTheEnd(self) -> bool:
        return self.clearAncillaAtTheEnd

    def SetClearAncillaAtTheEnd(self, v: bool) -> None:
        self.clearAncillaAtTheEnd = bool(v)


def _basis_state_walk(reg, x, start: int, nq: int, states, before_each) -> None:
    """the X-gate walk of Oracle.h:61-82 / :133-167: before each selected basis state, X gates turn the
    qubits where it has a 0 into 1s (toggling only those that differ from the previous state), then the
    n-controlled operation runs; the X gates left at the end are undone"""
    flipped = [False] * nq
    for state in states:
        v = state << start
        for q in range(nq):
            if flipped[q] != ((v & 1) == 0):
                reg.ApplyGate(x, start + q)
                flipped[q] = not flipped[q]
            v >>= 1
        before_each(state)
    for q in range(nq):
        if flipped[q]:
            reg.ApplyGate(x, start + q)


class OracleWithGatesSimpleFunction(QuantumSubAlgorithmOnSubregister):
    """QC::Oracles::OracleWithGatesSimpleFunction (Oracle.h:10-95): |x>|y> -> |x>|y ^ f(x)> for a boolean f on
    the qubits [startQubit, endQubit], one n-controlled NOT onto the target per x with f(x) = 1"""

    def __init__(self, N: int, startQubit: int = 0, endQubit: int = INT_MAX, targetQubit: int = 0,
                 startAncilla: int = INT_MAX):
        super().__init__(N, startQubit, endQubit)
        self.target = targetQubit
        self.nControlledNOT = NControlledNotWithAncilla(INT_MAX)
        self.nControlledNOT.SetControlQubits(range(startQubit, endQubit + 1))
        self.nControlledNOT.SetTargetQubit(targetQubit)
        self.nControlledNOT.SetStartAncillaQubits(startAncilla)
        self.x = G.PauliXGate()
        self.func = lambda state: False

    def setFunction(self, f) -> None:
        self.func = f

    def Execute(self, reg) -> int:
        s, e = self.getStartQubit(), self.getEndQubit()
        nq = e - s + 1
        states = [st for st in range(1 << nq) if self.func(st)]
        _basis_state_walk(reg, self.x, s, nq, states, lambda st: self.nControlledNOT.Execute(reg))
        return 0


class OracleWithGates(QuantumSubAlgorithmOnSubregister):
    """QC::Oracles::OracleWithGates (Oracle.h:97-243): |x>|y> -> |x>|y ^ f(x)> for an integer-valued f, with y on
    the qubits from startTargetQubits up; per x with f(x) != 0 one n-controlled NOT onto every set bit of f(x)"""

    def __init__(self, N: int, startQubit: int = 0, endQubit: int = INT_MAX, startTargetQubits: int = 0,
                 startAncilla: int = INT_MAX):
        super().__init__(N, startQubit, endQubit)
        self.target = startTargetQubits
        self.nControlledNOTs = NControlledGatesWithAncilla(INT_MAX)
        self.nControlledNOTs.SetControlQubits(range(startQubit, endQubit + 1))
        self.nControlledNOTs.SetStartAncillaQubits(startAncilla)
        self.x = G.PauliXGate()
        self.func = lambda state: 0

    def setFunction(self, f) -> None:
        self.func = f

    def Execute(self, reg) -> int:
        s, e = self.getStartQubit(), self.getEndQubit()
        nq = e - s + 1
        values = {st: int(self.func(st)) for st in range(1 << nq)}
        xm = self.x.getRawOperatorMatrix()

        def controlled_nots(state: int) -> None:
            self.nControlledNOTs.ClearGates()
            fval, q = values[state], self.target
            while fval:
                if fval & 1:
                    self.nControlledNOTs.AddGate(G.AppliedGate(xm, q))
                fval >>= 1
                q += 1
            self.nControlledNOTs.Execute(reg)

        _basis_state_walk(reg, self.x, s, nq, [st for st in range(1 << nq) if values[st]], controlled_nots)
        return 0


class DeutschJozsaAlgorithmWithGatesOracle(QuantumAlgorithm):
    """DeutschJozsa::DeutschJozsaAlgorithmWithGatesOracle (DeutschJozsa.h:141-290): N algorithm qubits plus N - 3
    ancillas (2 qubits for N = 2); the balanced oracle is built from n-controlled NOTs, the constant ones are
    nothing or an X on the answer qubit.  The balanced function is shuffled by a seeded numpy generator here
    (a clock-seeded engine in the reference)."""

    FunctionType = DeutschJozsaAlgorithm.FunctionType

    def __init__(self, N: int = 2, addseed: int = 0, function_seed: int | None = None, **kw):
        assert N >= 2
        nq = 2 if N == 2 else 2 * N - 3
        super().__init__(nq, addseed, **kw)
        self.oracle = OracleWithGatesSimpleFunction(nq, 0, N - 2, N - 1, N)
        self.hadamard = G.HadamardGate()
        self.x = G.PauliXGate()
        self.functionType = self.FunctionType.constantZero
        self.fvalues = np.zeros(0, dtype=bool)
        self._rng = np.random.default_rng(function_seed)

    def getAlgoQubits(self) -> int:
        n = self.getNrQubits()
        return 2 if n == 2 else (n + 3) // 2

    def getAlgoNrBasisStates(self) -> int:
        return 1 << self.getAlgoQubits()

    def setFunction(self, ft) -> None:
        self.functionType = self.FunctionType(ft)
        if self.functionType == self.FunctionType.balanced:
            size = self.getAlgoNrBasisStates() >> 1
            v = np.zeros(size, dtype=bool)
            v[: size >> 1] = True
            self.fvalues = self._rng.permutation(v)
        else:
            self.fvalues = np.zeros(0, dtype=bool)
        fv, balanced = self.fvalues, self.functionType == self.FunctionType.balanced
        self.oracle.setFunction(lambda state: bool(fv[state]) if balanced else False)

    def getFunction(self):
        return self.functionType

    def WasConstantResult(self, state: int) -> bool:
        return (state & ((self.getAlgoNrBasisStates() - 1) >> 1)) == 0

    def Execute(self) -> int:
        a = self.getAlgoQubits()
        self.setToQubitState(a - 1)
        seq = GateSequence()
        for q in range(a):
            seq.ApplyGate(self.hadamard, q)
        if self.functionType == self.FunctionType.constantOne:
            seq.ApplyGate(self.x, a - 1)
        elif self.functionType == self.FunctionType.balanced:
            self.oracle.Execute(seq)
        for q in range(a - 1):
            seq.ApplyGate(self.hadamard, q)
        self.ApplyGates(seq.ops)
        return self.Measure(0, a - 2)


class BernsteinVaziraniFunction:
    """BernsteinVazirani::BernsteinVaziraniFunction (BernsteinVazirani.h:108-132): the parity of state & s"""

    def __init__(self, s: int = 0):
        self.stringFunction = s

    def __call__(self, state: int) -> bool:
        return bin(state & self.stringFunction).count("1") % 2 == 1


class BernsteinVaziraniAlgorithmWithGatesOracle(QuantumAlgorithm):
    """BernsteinVazirani::BernsteinVaziraniAlgorithmWithGatesOracle (BernsteinVazirani.h:134-210): N algorithm
    qubits, the answer qubit N and N - 2 ancillas; the oracle flips the answer qubit for every x of odd parity
    with the hidden string"""

    def __init__(self, N: int = 3, addseed: int = 0, **kw):
        assert N >= 1
        super().__init__(2 * N - 1, addseed, **kw)
        self.oracle = OracleWithGatesSimpleFunction(2 * N - 1, 0, N - 1, N, N + 1)
        self.hadamard = G.HadamardGate()

    def setString(self, s: int) -> None:
        self.oracle.setFunction(BernsteinVaziraniFunction(s))

    def getAlgoQubits(self) -> int:
        return (self.getNrQubits() + 1) // 2

    def Execute(self) -> int:
        a = self.getAlgoQubits()
        self.setToQubitState(a)
        seq = GateSequence()
        for q in range(a + 1):
            seq.ApplyGate(self.hadamard, q)
        self.oracle.Execute(seq)
        for q in range(a + 1):
            seq.ApplyGate(self.hadamard, q)
        self.ApplyGates(seq.ops)
        return self.Measure(0, a - 1)


class SimonAlgorithmWithGatesOracle(QuantumAlgorithm):
    """Simon::SimonAlgorithmWithGatesOracle (SimonAlgorithm.h:250-367): 2N algorithm qubits plus N - 1 ancillas;
    the oracle writes f(x) into the high half with n-controlled NOTs.  Rounds, stopping rule and the elimination
    of candidate strings as SimonAlgorithm."""

    def __init__(self, N: int = 3, addseed: int = 0, function_seed: int | None = None, **kw):
        assert N >= 2
        super().__init__(3 * N - 1, addseed, **kw)
        self.oracle = OracleWithGates(3 * N - 1, 0, N - 1, N, 2 * N)
        self.hadamard = G.HadamardGate()
        self.f = SimonFunction(np.random.default_rng(function_seed))
        self.setString(0)

    def getAlgoQubits(self) -> int:
        return (self.getNrQubits() + 1) // 3 * 2

    def setString(self, s: int) -> None:
        N = self.getAlgoQubits() >> 1
        self.f.setString(s, N)
        f = self.f
        self.oracle.setFunction(lambda state: int(f(state)))
        seq = GateSequence()
        for q in range(N):
            seq.ApplyGate(self.hadamard, q)
        self.oracle.Execute(seq)
        for q in range(N):
            seq.ApplyGate(self.hadamard, q)
        self._round = G.PreparedGates(seq.ops)  # one round's circuit after the reset, converted once per string

    def Execute(self) -> int:
        N = self.getAlgoQubits() >> 1
        mask = (1 << N) - 1
        measurements: dict[int, int] = {}
        for _ in range(300):
            self.setToBasisState(0)
            self.ApplyGates(self._round)
            m = self.Measure(0, N - 1)
            measurements[m] = measurements.get(m, 0) + 1
            if len(measurements) == 1 << N:
                return 0
        candidates = set(range(1, mask + 1))
        for b in measurements:
            if b:
                candidates = {c for c in candidates if bin(c & b).count("1") % 2 == 0}
        return next(iter(candidates)) if len(candidates) == 1 else mask + 1
