"""QubitRegister: the Python-side mirror of QC::QubitRegister (QCSim/QubitRegister.h) over the C ABI.

Method names, argument meanings, defaults and error behaviour follow the reference class, so code
written against QubitRegister reads the same here.  The amplitudes live on the GPU (libqcs_gpu.so);
every gate and measurement runs there.  Randomness follows the reference: a std::mt19937_64 with a
std::uniform_real_distribution<double>(0, 1), drawn on the host, and each measurement uses
prob = 1 - uniform (QubitRegister.h:171, 210, 267, 621, 707).
"""
from __future__ import annotations

import ctypes as C
import os
import time

import numpy as np

from . import _lib as L
from .gates import AppliedGate, QuantumGate

OneQubitOmpLimit = 8192  # QubitRegisterCalculator.h:1276 (kept for API compatibility)


class Rng:
    """std::mt19937_64 + std::uniform_real_distribution<double>(0, 1) from the engine's C runtime."""

    def __init__(self, seed: int):
        lib = L.load()
        self._lib = lib
        self._h = C.c_void_p()
        L.check(lib.qcs_rng_create(C.c_uint64(seed & 0xFFFFFFFFFFFFFFFF), C.byref(self._h)))

    def uniform(self, n: int = 1) -> np.ndarray:
        out = np.empty(n, dtype=np.float64)
        L.check(self._lib.qcs_rng_uniform(self._h, L.dptr(out), n))
        return out

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._lib.qcs_rng_destroy(h)
            self._h = None


class QubitRegister:
    """QC::QubitRegister<> (QubitRegister.h:11-728)."""

    def __init__(self, N: int = 3, addseed: int = 0, *, precision: str = "fp64", seed: int | None = None):
        assert N > 0  # QubitRegister.h:22
        self._lib = L.load()
        prec = L.QCS_FP64 if precision == "fp64" else L.QCS_FP32
        self._h = C.c_void_p()
        L.check(self._lib.qcs_create(N, prec, C.byref(self._h)))
        self.NrQubits = N
        self.NrBasisStates = 1 << N
        self.precision = precision
        if seed is None:
            # QubitRegister.h:26-34 seeds from the clock plus a random addend
            seed = (time.perf_counter_ns() + (addseed or int.from_bytes(os.urandom(4), "little"))) & (2**64 - 1)
        self.rng = Rng(seed)
        self.computeGates: list[AppliedGate] = []
        self.recordGates = False
        self._multithreading = True

    # ---- lifetime ----
    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.qcs_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, status: int) -> None:
        if status != L.QCS_OK:
            L.check(status, self._h)

    @property
    def handle(self):
        return self._h

    def set_passes(self, enabled: bool) -> None:
        """gate lists as shared-memory passes (default) or one kernel per gate"""
        self._ck(self._lib.qcs_set_option(self._h, L.QCS_OPT_PASSES, int(bool(enabled))))

    def set_fusion(self, mode: int, max_qubits: int | None = None) -> None:
        """fuse gate lists into dense blocks: 0 off, 1 greedy, 2 learned partition (FP32 default: 1, blocks of at
        most 4 qubits from 26 qubits up with the tensor cores on, else at most 3)"""
        self._ck(self._lib.qcs_set_option(self._h, L.QCS_OPT_FUSION, int(mode)))
        if max_qubits is not None:
            self._ck(self._lib.qcs_set_option(self._h, L.QCS_OPT_FUSION_MAX_QUBITS, int(max_qubits)))

    def set_tensor_cores(self, enabled: bool) -> None:
        """FP32 registers: fused 4- and 5-qubit blocks as 3xTF32 tensor-core products (default) or FP32
        FMAs on the CUDA cores"""
        self._ck(self._lib.qcs_set_option(self._h, L.QCS_OPT_TENSOR_CORES, int(bool(enabled))))

    def profile(self, enable: bool = True) -> None:
        """bracket every kernel launch of this register with CUDA events (see read_profile)"""
        self._ck(self._lib.qcs_profile_enable(self._h, int(bool(enable))))

    def read_profile(self, fp_ops: bool = False) -> dict:
        """{kernel family: (launches, device ms, algorithmic bytes[, floating-point instructions])} since
        the last read"""
        cap = 64
        arr = (L.qcs_profile_entry * cap)()
        n = C.c_int()
        self._ck(self._lib.qcs_profile_read(self._h, C.cast(arr, C.c_void_p), cap, C.byref(n)))
        out = {}
        for i in range(n.value):
            e = arr[i]
            row = (int(e.launches), float(e.milliseconds), float(e.bytes))
            out[e.name.decode()] = row + (float(e.fp_ops),) if fp_ops else row
        return out

    def seed(self, s: int) -> None:
        """reseed the register's generator (the reference's protected rng, QubitRegister.h:723)"""
        self.rng = Rng(s)

    def _prob(self) -> float:
        return 1.0 - float(self.rng.uniform(1)[0])

    # ---- sizes and element access (QubitRegister.h:59-72) ----
    def getNrQubits(self) -> int:
        return self.NrQubits

    def getNrBasisStates(self) -> int:
        return self.NrBasisStates

    def getBasisStateAmplitude(self, State: int) -> complex:
        out = np.zeros(2)
        self._ck(self._lib.qcs_get_amplitude(self._h, State, L.dptr(out)))
        return complex(out[0], out[1])

    def getBasisStateProbability(self, State: int) -> float:
        if State >= self.NrBasisStates:
            return 0.0
        a = self.getBasisStateAmplitude(State)
        return a.real * a.real + a.imag * a.imag

    # ---- setters (QubitRegister.h:74-122) ----
    def setToBasisState(self, State: int) -> None:
        self._ck(self._lib.qcs_set_basis(self._h, State))

    def setToQubitState(self, q: int) -> None:
        self._ck(self._lib.qcs_set_qubit_state(self._h, q))

    def setToCatState(self) -> None:
        self._ck(self._lib.qcs_set_cat(self._h))

    def Reset(self) -> None:
        self.setToBasisState(0)

    def setToEqualSuperposition(self) -> None:
        self._ck(self._lib.qcs_set_equal(self._h))

    def setRawAmplitude(self, State: int, val: complex) -> None:
        val = complex(val)
        self._ck(self._lib.qcs_set_amplitude(self._h, State, val.real, val.imag))

    def Clear(self) -> None:
        self._ck(self._lib.qcs_clear(self._h))

    def Normalize(self) -> None:
        self._ck(self._lib.qcs_normalize(self._h))

    def AdjustPhaseAndNormalize(self) -> None:
        self._ck(self._lib.qcs_adjust_phase_normalize(self._h))

    # ---- measurement (QubitRegister.h:169-429) ----
    def MeasureAll(self) -> int:
        out = C.c_uint64()
        self._ck(self._lib.qcs_measure_all(self._h, self._prob(), C.byref(out)))
        return out.value

    def MeasureQubit(self, qubit: int) -> int:
        return self.Measure(qubit, qubit)

    def Measure(self, firstQubit: int, secondQubit: int) -> int:
        out = C.c_uint64()
        self._ck(self._lib.qcs_measure(self._h, firstQubit, secondQubit, self._prob(), C.byref(out)))
        return out.value

    def MeasureNoCollapse(self, firstQubit: int | None = None, secondQubit: int | None = None) -> int:
        out = C.c_uint64()
        self._ck(self._lib.qcs_measure_no_collapse(self._h, self._prob(), C.byref(out)))
        if firstQubit is None:
            return out.value
        second = firstQubit if secondQubit is None else secondQubit
        return (out.value & _mask(firstQubit, second)) >> firstQubit

    def _shots(self, nrTimes: int) -> np.ndarray:
        probs = 1.0 - self.rng.uniform(nrTimes)
        out = np.empty(nrTimes, dtype=np.uint64)
        self._ck(self._lib.qcs_sample(self._h, L.dptr(probs), nrTimes, L.u64ptr(out)))
        return out

    def RepeatedMeasure(self, *args) -> dict:
        """RepeatedMeasure(nrTimes=1000) or RepeatedMeasure(firstQubit, secondQubit, nrTimes=1000)"""
        if len(args) >= 2:
            first, second = args[0], args[1]
            nrTimes = args[2] if len(args) > 2 else 1000
        else:
            first = second = None
            nrTimes = args[0] if args else 1000
        if nrTimes == 0:
            return {}
        if nrTimes == 1:
            v = self.MeasureNoCollapse(first, second) if first is not None else self.MeasureNoCollapse()
            return {v: 1}
        states = self._shots(nrTimes)
        if first is not None:
            states = (states & np.uint64(_mask(first, second))) >> np.uint64(first)
        keys, counts = np.unique(states, return_counts=True)
        return {int(k): int(c) for k, c in zip(keys, counts)}

    RepeatedMeasureUnordered = RepeatedMeasure

    def GetQubitProbability(self, qubit: int) -> float:
        out = C.c_double()
        self._ck(self._lib.qcs_qubit_probability(self._h, qubit, C.byref(out)))
        return out.value

    def GetQubitProbabilityNoAlloc(self, qubit: int) -> float:
        """GetQubitProbability through the library's fixed device array (qcs_qubit_probability_noalloc):
        no device allocation, registers of at most 32 qubits, calls must not overlap on the GPU."""
        out = C.c_double()
        self._ck(self._lib.qcs_qubit_probability_noalloc(self._h, qubit, C.byref(out)))
        return out.value

    def probabilities(self) -> np.ndarray:
        out = np.empty(self.NrBasisStates, dtype=np.float64)
        self._ck(self._lib.qcs_probabilities(self._h, L.dptr(out)))
        return out

    # ---- gates (QubitRegister.h:434-505) ----
    def ApplyGate(self, gate: QuantumGate, qubit: int | None = None, controllingQubit1: int = 0,
                  controllingQubit2: int = 0) -> None:
        if qubit is None:  # ApplyGate(const AppliedGate&) (QubitRegister.h:488-491)
            qubit, controllingQubit1, controllingQubit2 = gate.getQubit1(), gate.getQubit2(), gate.getQubit3()
        m = np.ascontiguousarray(gate.getRawOperatorMatrix(), dtype=np.complex128)
        k = gate.getQubitsNumber()
        self._ck(self._lib.qcs_apply_gate(self._h, m.view(np.float64).ctypes.data_as(C.POINTER(C.c_double)),
                                          k, qubit, controllingQubit1, controllingQubit2, gate.traits()))
        if self.recordGates:
            self.computeGates.append(AppliedGate(m.copy(), qubit, controllingQubit1, controllingQubit2))

    def ApplyGates(self, gates) -> None:
        """ApplyGates(list of AppliedGate) (QubitRegister.h:493-497); also accepts (gate, q0, q1, q2) tuples, or a
        gates.PreparedGates whose records were converted once"""
        from .gates import PreparedGates, records
        if isinstance(gates, PreparedGates):
            tuples, recs = gates.ops, gates.recs
        else:
            tuples = []
            for g in gates:
                if isinstance(g, tuple):
                    tuples.append(g)
                else:
                    tuples.append((g, g.getQubit1(), g.getQubit2(), g.getQubit3()))
            recs = records(tuples)
        self.apply_records(recs)
        if self.recordGates:
            for g, *qs in tuples:
                qs = list(qs) + [0, 0]
                self.computeGates.append(AppliedGate(g.getRawOperatorMatrix().copy(), qs[0], qs[1], qs[2]))

    def apply_records(self, recs: np.ndarray) -> None:
        """apply a qcs_gate array (include/qcs_gpu.h) in one call"""
        recs = np.ascontiguousarray(recs, dtype=L.GATE_DTYPE)
        self._ck(self._lib.qcs_apply_gates(self._h, recs.ctypes.data_as(C.c_void_p), len(recs)))

    def ApplyOperatorMatrix(self, m) -> None:
        """ApplyOperatorMatrix (QubitRegister.h:499-505): a dense 2^n x 2^n operator; a diagonal one (every
        non-zero entry on the diagonal) runs as one multiply per amplitude (qcs_apply_diagonal)"""
        m = np.ascontiguousarray(m, dtype=np.complex128)
        N = self.getNrBasisStates()
        if m.shape != (N, N):
            raise ValueError("the operator must be 2^n x 2^n")
        d = np.ascontiguousarray(np.diagonal(m))
        if np.count_nonzero(m) == np.count_nonzero(d):
            self._ck(self._lib.qcs_apply_diagonal(self._h, d.view(np.float64).ctypes.data_as(C.POINTER(C.c_double))))
        else:
            self._ck(self._lib.qcs_apply_operator_matrix(self._h, m.view(np.float64).ctypes.data_as(C.POINTER(C.c_double))))
        if self.recordGates:
            self.computeGates.append(AppliedGate(m.copy()))

    def ApplyDiagonal(self, d) -> None:
        """amplitude i *= d[i] for the 2^n entries d (qcs_apply_diagonal), without a 2^n x 2^n matrix"""
        d = np.ascontiguousarray(d, dtype=np.complex128)
        if d.shape != (self.getNrBasisStates(),):
            raise ValueError("the diagonal must have 2^n entries")
        self._ck(self._lib.qcs_apply_diagonal(self._h, d.view(np.float64).ctypes.data_as(C.POINTER(C.c_double))))

    def ApplyOperatorOnQubits(self, m, qubits, controls=()) -> None:
        """a dense 2^k x 2^k operator (k <= 10) on the given target qubits (matrix bit j = qubits[j]),
        applied where every control qubit is one: what NQubitsQuantumGate / NQubitsControlledQuantumGate
        do through their 2^n x 2^n extended matrix (qcs_apply_operator_on_qubits)"""
        m = np.ascontiguousarray(m, dtype=np.complex128)
        qs = np.ascontiguousarray(list(qubits), dtype=np.uint32)
        if m.shape != (1 << qs.size, 1 << qs.size):
            raise ValueError("operator size does not match the number of target qubits")
        ctrl = 0
        for c in controls:
            ctrl |= 1 << int(c)
        self._ck(self._lib.qcs_apply_operator_on_qubits(self._h, m.view(np.float64).ctypes.data_as(C.POINTER(C.c_double)),
                                                        qs.size, qs.ctypes.data_as(C.POINTER(C.c_uint32)), ctrl))

    # ---- whole-vector access (QubitRegister.h:507-534) ----
    def getRegisterStorage(self) -> np.ndarray:
        out = np.empty(self.NrBasisStates, dtype=np.complex128)
        self._ck(self._lib.qcs_get_state(self._h, out.view(np.float64).ctypes.data_as(C.POINTER(C.c_double))))
        return out

    def setRegisterStorage(self, vals) -> None:
        vals = np.ascontiguousarray(vals, dtype=np.complex128)
        if vals.size != self.NrBasisStates:
            return
        self.setRegisterStorageFastNoNormalize(vals)
        self.Normalize()

    def setRegisterStorageFastNoNormalize(self, vals) -> None:
        vals = np.ascontiguousarray(vals, dtype=np.complex128)
        self._ck(self._lib.qcs_set_state(self._h, vals.view(np.float64).ctypes.data_as(C.POINTER(C.c_double))))

    def stateFidelity(self, state) -> float:
        state = np.ascontiguousarray(state, dtype=np.complex128)
        if state.size != self.NrBasisStates:
            return 0.0
        out = C.c_double()
        self._ck(self._lib.qcs_fidelity_host(self._h, state.view(np.float64).ctypes.data_as(C.POINTER(C.c_double)),
                                             C.byref(out)))
        return out.value

    # ---- record / replay (QubitRegister.h:536-590) ----
    def ComputeStart(self) -> None:
        self.recordGates = True
        self.computeGates = []

    def ComputeEnd(self) -> None:
        self.recordGates = False

    def ComputeClear(self) -> None:
        self.computeGates = []

    def _replay(self, gates) -> None:
        save, self.recordGates = self.recordGates, False
        run = []
        for g in gates:
            if g.getQubitsNumber() > 3:
                if run:
                    self.ApplyGates(run)
                    run = []
                self.ApplyOperatorMatrix(g.getRawOperatorMatrix())
            else:
                run.append(g)
        if run:
            self.ApplyGates(run)
        self.recordGates = save

    def Compute(self) -> None:
        self._replay(self.computeGates)

    def Uncompute(self) -> None:
        self._replay([AppliedGate(g.getRawOperatorMatrix().conj().T, g.getQubit1(), g.getQubit2(), g.getQubit3())
                      for g in reversed(self.computeGates)])

    # ---- snapshots and expectation (QubitRegister.h:600-674) ----
    def SaveState(self) -> None:
        self._ck(self._lib.qcs_save_state(self._h))

    def RestoreState(self) -> None:
        self._ck(self._lib.qcs_restore_state(self._h))

    def RestoreStateDestructive(self) -> None:
        self._ck(self._lib.qcs_restore_state_destructive(self._h))

    def ExpectationValue(self, gates) -> complex:
        if not gates:
            return complex(1.0, 0.0)
        from .gates import records
        recs = records([(g, g.getQubit1(), g.getQubit2(), g.getQubit3()) for g in gates])
        out = np.zeros(2)
        self._ck(self._lib.qcs_expectation(self._h, recs.ctypes.data_as(C.c_void_p), len(recs), L.dptr(out)))
        return complex(out[0], out[1])

    def Clone(self) -> "QubitRegister":
        c = QubitRegister.__new__(QubitRegister)
        c._lib = self._lib
        c._h = C.c_void_p()
        self._ck(self._lib.qcs_clone(self._h, C.byref(c._h)))
        c.NrQubits, c.NrBasisStates, c.precision = self.NrQubits, self.NrBasisStates, self.precision
        c.rng = Rng(int.from_bytes(os.urandom(8), "little"))
        c.computeGates = list(self.computeGates)
        c.recordGates = self.recordGates
        c._multithreading = self._multithreading
        return c

    # ---- threading knobs (QubitRegisterCalculator.h:1256-1278): kept for API compatibility ----
    def SetMultithreading(self, enable: bool = True) -> None:
        self._multithreading = bool(enable)

    def GetMultithreading(self) -> bool:
        return self._multithreading

    @staticmethod
    def GetNumberOfThreads() -> int:
        return os.cpu_count() or 1


def _mask(first: int, second: int) -> int:
    """measuredPartMask of QubitRegister.h:331-333"""
    return ((1 << (second + 1)) - 1) - ((1 << first) - 1)

