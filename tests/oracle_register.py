"""A register with the members QCSim's small protocols call (state setters, gates, measurements with
collapse, amplitudes), over the CPU oracle's gate application and with seeded numpy sampling.  Test
infrastructure: it lets the algorithm mirrors' host logic run end to end without a GPU."""
import numpy as np

from oracle import bind as B
from qcsim_gb300 import gates as G


class OracleBackedRegister:
    # the QFT mirror sends a recording register its individual gates (through ApplyGate) instead of one
    # engine call, which is what this stand-in needs
    recordGates = True

    def __init__(self, N, addseed=0, *, precision="fp64", seed=None):
        self.n = N
        self.r = B.OracleRegister(N)
        self.rng = np.random.default_rng(seed)
        self.setToBasisState(0)

    # ---- sizes and state ----
    def getNrQubits(self):
        return self.n

    def getNrBasisStates(self):
        return 1 << self.n

    def _set(self, v):
        self.r.set_state(np.ascontiguousarray(v, dtype=np.complex128))

    def getRegisterStorage(self):
        return self.r.state()

    def setRegisterStorage(self, v):
        v = np.asarray(v, dtype=np.complex128)
        self._set(v / np.linalg.norm(v))

    def getBasisStateAmplitude(self, s):
        return complex(self.r.state()[s])

    def getBasisStateProbability(self, s):
        return abs(self.r.state()[s]) ** 2

    def setToBasisState(self, s):
        v = np.zeros(1 << self.n, dtype=np.complex128)
        v[s] = 1
        self._set(v)

    def setToQubitState(self, q):
        self.setToBasisState(1 << q)

    def setToCatState(self):
        v = np.zeros(1 << self.n, dtype=np.complex128)
        v[0] = v[-1] = 1 / np.sqrt(2)
        self._set(v)

    def setToEqualSuperposition(self):
        self._set(np.full(1 << self.n, 1 / np.sqrt(1 << self.n), dtype=np.complex128))

    def Clear(self):
        self._set(np.zeros(1 << self.n, dtype=np.complex128))

    def setRawAmplitude(self, s, val):
        v = self.r.state()
        v[s] = val
        self._set(v)

    def Normalize(self):
        v = self.r.state()
        self._set(v / np.linalg.norm(v))

    # ---- gates ----
    @staticmethod
    def _oracle_op(gate, q0, q1=0, q2=0):
        # a gate class the oracle has no code for (a plain SingleQubitGate of a given matrix) goes as a
        # matrix-only gate, which both apply through the generic path
        if getattr(gate, "code", -1) < 0:
            gate = G.AppliedGate(gate.getRawOperatorMatrix(), q0, q1, q2)
        return (gate, q0, q1, q2)

    def ApplyGate(self, gate, qubit=None, c1=0, c2=0):
        if qubit is None:
            qubit, c1, c2 = gate.getQubit1(), gate.getQubit2(), gate.getQubit3()
        self.r.apply([self._oracle_op(gate, qubit, c1, c2)])
        if self._recording:
            self._recorded.append((gate.getRawOperatorMatrix().copy(), qubit, c1, c2))

    # record / replay as the register's ComputeStart / ComputeEnd / Uncompute (QubitRegister.h:536-590)
    _recording = False

    def ComputeStart(self):
        self._recording, self._recorded = True, []

    def ComputeEnd(self):
        self._recording = False

    def Uncompute(self):
        self.r.apply([(G.AppliedGate(m.conj().T, q0, q1, q2), q0, q1, q2) for m, q0, q1, q2 in reversed(self._recorded)])

    def ApplyGates(self, ops):
        ops = getattr(ops, "ops", ops)  # a gates.PreparedGates carries its tuples
        ops = [self._oracle_op(*op) if isinstance(op, tuple) else
               self._oracle_op(op, op.getQubit1(), op.getQubit2(), op.getQubit3()) for op in ops]
        if ops:
            self.r.apply(ops)

    def ApplyOperatorOnQubits(self, m, qubits, controls=()):
        from oracle import nqubits
        self._set(nqubits.apply_on_qubits(self.r.state(), np.asarray(m, dtype=np.complex128), list(qubits), list(controls)))

    def ApplyOperatorMatrix(self, m):
        self._set(np.asarray(m, dtype=np.complex128) @ self.r.state())

    # ---- measurements (sampled with the numpy generator, collapse and renormalise) ----
    def Measure(self, first, second):
        v = self.r.state()
        idx = np.arange(v.size)
        sub = (idx >> first) & ((1 << (second - first + 1)) - 1)
        p = np.bincount(sub, weights=np.abs(v) ** 2, minlength=1 << (second - first + 1))
        m = int(self.rng.choice(p.size, p=p / p.sum()))
        v = np.where(sub == m, v, 0)
        self._set(v / np.linalg.norm(v))
        return m

    def MeasureQubit(self, q):
        return self.Measure(q, q)

    def MeasureAll(self):
        return self.Measure(0, self.n - 1)

    def RepeatedMeasure(self, *args):
        if len(args) >= 2:
            first, second, shots = args[0], args[1], (args[2] if len(args) > 2 else 1000)
        else:
            first, second, shots = 0, self.n - 1, (args[0] if args else 1000)
        v = self.r.state()
        sub = (np.arange(v.size) >> first) & ((1 << (second - first + 1)) - 1)
        p = np.bincount(sub, weights=np.abs(v) ** 2, minlength=1 << (second - first + 1))
        counts = self.rng.multinomial(shots, p / p.sum())
        return {int(i): int(c) for i, c in enumerate(counts) if c}

    def close(self):
        pass
