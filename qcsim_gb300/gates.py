"""Gate library mirroring QC::Gates (QCSim/SimpleGates.h, QCSim/QuantumGate.h).

Each gate carries its raw operator matrix (row/column bit 0 = target qubit, bit 1 =
controllingQubit1, bit 2 = controllingQubit2, as in SimpleGates.h:329 and :430) and answers the same
trait questions as the reference's virtuals (SimpleGates.h:27-60).  The register hands both to the
engine, which dispatches on the traits exactly as QubitRegister::ApplyGate does.
"""
from __future__ import annotations

import math

import numpy as np

from . import _lib as L

R2 = 1.0 / math.sqrt(2.0)


def polar(theta: float) -> complex:
    """std::polar(1, theta)"""
    return complex(math.cos(theta), math.sin(theta))


class QuantumGate:
    """QC::Gates::QuantumGate / QuantumGateWithOp (SimpleGates.h:12-132)."""

    code = -1  # CPU-oracle gate code of the reference class this mirrors

    def __init__(self, matrix: np.ndarray):
        self.operatorMat = np.array(matrix, dtype=np.complex128)

    def getRawOperatorMatrix(self) -> np.ndarray:
        return self.operatorMat

    def getQubitsNumber(self) -> int:
        return int(math.log2(self.operatorMat.shape[0]))

    def isControlled(self) -> bool:
        return False

    def isControlQubit(self, qubit: int) -> bool:
        return False

    def isDiagonal(self) -> bool:
        return False

    def isAntidiagonal(self) -> bool:
        return False

    def isSwapGate(self) -> bool:
        return False

    def IsISwapGate(self) -> bool:
        return False

    def IsISwapDagGate(self) -> bool:
        return False

    def traits(self) -> int:
        t = 0
        if self.isDiagonal():
            t |= L.TRAIT_DIAGONAL
        if self.isAntidiagonal():
            t |= L.TRAIT_ANTIDIAGONAL
        if self.isSwapGate():
            t |= L.TRAIT_SWAP
        if self.IsISwapGate():
            t |= L.TRAIT_ISWAP
        if self.IsISwapDagGate():
            t |= L.TRAIT_ISWAPDAG
        if self.isControlled():
            t |= L.TRAIT_CONTROLLED
        if self.isControlQubit(1):
            t |= L.TRAIT_CONTROLQ1
        return t

    def params(self) -> tuple:
        return (0.0, 0.0, 0.0, 0.0)


# ---- one qubit (SingleQubitGate starts from a zero 2x2, SimpleGates.h:140-143) ----
class SingleQubitGate(QuantumGate):
    def __init__(self, matrix=None):
        super().__init__(np.zeros((2, 2)) if matrix is None else matrix)

    def getQubitsNumber(self) -> int:
        return 1


class HadamardGate(SingleQubitGate):  # SimpleGates.h:582-597
    code = 0

    def __init__(self):
        super().__init__([[R2, R2], [R2, -R2]])


class HyGate(SingleQubitGate):  # SimpleGates.h:602-617
    code = 1

    def __init__(self):
        super().__init__([[R2, complex(0, -R2)], [complex(0, R2), -R2]])


class _Diag1(SingleQubitGate):
    def isDiagonal(self) -> bool:
        return True


class SGate(_Diag1):  # SimpleGates.h:620-636
    code = 2

    def __init__(self):
        super().__init__([[1, 0], [0, 1j]])


class SDGGate(_Diag1):  # SimpleGates.h:638-654
    code = 3

    def __init__(self):
        super().__init__([[1, 0], [0, -1j]])


class TGate(_Diag1):  # SimpleGates.h:657-673
    code = 4

    def __init__(self):
        super().__init__([[1, 0], [0, polar(math.pi / 4.0)]])


class TDGGate(_Diag1):  # SimpleGates.h:675-691
    code = 5

    def __init__(self):
        super().__init__([[1, 0], [0, polar(-math.pi / 4.0)]])


class PhaseShiftGate(_Diag1):  # SimpleGates.h:693-714
    code = 6

    def __init__(self, theta: float = 0.0):
        super().__init__([[1, 0], [0, 0]])
        self.SetPhaseShift(theta)

    def SetPhaseShift(self, theta: float) -> None:
        self.theta = theta
        self.operatorMat[1, 1] = polar(theta)

    def params(self):
        return (self.theta, 0.0, 0.0, 0.0)


class PauliXGate(SingleQubitGate):  # SimpleGates.h:717-733
    code = 7

    def __init__(self):
        super().__init__([[0, 1], [1, 0]])

    def isAntidiagonal(self) -> bool:
        return True


class PauliYGate(SingleQubitGate):  # SimpleGates.h:735-751
    code = 8

    def __init__(self):
        super().__init__([[0, -1j], [1j, 0]])

    def isAntidiagonal(self) -> bool:
        return True


class PauliZGate(_Diag1):  # SimpleGates.h:754-770
    code = 9

    def __init__(self):
        super().__init__([[1, 0], [0, -1]])


class SquareRootNOTGate(SingleQubitGate):  # SimpleGates.h:773-786
    code = 10

    def __init__(self):
        super().__init__([[0.5 + 0.5j, 0.5 - 0.5j], [0.5 - 0.5j, 0.5 + 0.5j]])


class SquareRootNOTDagGate(SingleQubitGate):  # SimpleGates.h:788-801
    code = 11

    def __init__(self):
        super().__init__([[0.5 - 0.5j, 0.5 + 0.5j], [0.5 + 0.5j, 0.5 - 0.5j]])


class SplitterGate(SingleQubitGate):  # SimpleGates.h:803-817
    code = 12

    def __init__(self):
        super().__init__([[R2, complex(0, R2)], [complex(0, R2), R2]])


class RotationGate(SingleQubitGate):
    def __init__(self, theta: float = 0.0):
        super().__init__()
        self.SetTheta(theta)

    def params(self):
        return (self.theta, 0.0, 0.0, 0.0)


class RxGate(RotationGate):  # SimpleGates.h:829-849
    code = 13

    def SetTheta(self, theta: float) -> None:
        self.theta = theta
        t2 = theta * 0.5
        c, s = math.cos(t2), math.sin(t2)
        self.operatorMat[:] = [[complex(c, 0), complex(0, -s)], [complex(0, -s), complex(c, 0)]]


class RyGate(RotationGate):  # SimpleGates.h:851-871
    code = 14

    def SetTheta(self, theta: float) -> None:
        self.theta = theta
        t2 = theta * 0.5
        c, s = math.cos(t2), math.sin(t2)
        self.operatorMat[:] = [[c, -s], [s, c]]


class RzGate(RotationGate):  # SimpleGates.h:873-896
    code = 15

    def SetTheta(self, theta: float) -> None:
        self.theta = theta
        t2 = theta * 0.5
        self.operatorMat[:] = [[polar(-t2), 0], [0, polar(t2)]]

    def isDiagonal(self) -> bool:
        return True


def _u_entries(theta, phi, lam, gamma):
    """the four entries UGate / ControlledUGate compute (SimpleGates.h:910-918, QuantumGate.h:284-292)"""
    t2 = theta * 0.5
    c, s = math.cos(t2), math.sin(t2)
    return (polar(gamma) * complex(c, 0.0), -polar(gamma + lam) * s, polar(gamma + phi) * s,
            polar(gamma + phi + lam) * c)


class UGate(SingleQubitGate):  # SimpleGates.h:899-919
    code = 16

    def __init__(self, theta=0.0, phi=0.0, lam=0.0, gamma=0.0):
        super().__init__()
        self.SetParams(theta, phi, lam, gamma)

    def SetParams(self, theta=0.0, phi=0.0, lam=0.0, gamma=0.0):
        self._p = (theta, phi, lam, gamma)
        a, b, c, d = _u_entries(theta, phi, lam, gamma)
        self.operatorMat[:] = [[a, b], [c, d]]

    def params(self):
        return self._p


# ---- two qubits (TwoQubitsGate starts from identity, SimpleGates.h:240-243) ----
class TwoQubitsGate(QuantumGate):
    def __init__(self, matrix=None):
        super().__init__(np.eye(4) if matrix is None else matrix)

    def getQubitsNumber(self) -> int:
        return 2


class SwapGate(TwoQubitsGate):  # QuantumGate.h:10-28
    code = 20

    def __init__(self):
        super().__init__()
        m = self.operatorMat
        m[1, 1] = m[2, 2] = 0
        m[1, 2] = m[2, 1] = 1

    def isSwapGate(self) -> bool:
        return True


class iSwapGate(TwoQubitsGate):  # QuantumGate.h:30-48
    code = 21

    def __init__(self):
        super().__init__()
        m = self.operatorMat
        m[1, 1] = m[2, 2] = 0
        m[1, 2] = m[2, 1] = 1j

    def IsISwapGate(self) -> bool:
        return True


class iSwapDagGate(TwoQubitsGate):  # QuantumGate.h:50-68
    code = 22

    def __init__(self):
        super().__init__()
        m = self.operatorMat
        m[1, 1] = m[2, 2] = 0
        m[1, 2] = m[2, 1] = -1j

    def IsISwapDagGate(self) -> bool:
        return True


class DecrementGate(TwoQubitsGate):  # QuantumGate.h:70-89
    code = 23

    def __init__(self):
        super().__init__(np.zeros((4, 4)))
        m = self.operatorMat
        m[3, 0] = m[0, 1] = m[1, 2] = m[2, 3] = 1


class TwoQubitsControlledGate(TwoQubitsGate):  # QuantumGate.h:91-114
    def isControlled(self) -> bool:
        return True

    def isControlQubit(self, qubit: int) -> bool:
        return qubit == 0

    def SetOperation(self, U) -> None:
        self.operatorMat[2:4, 2:4] = U


class CNOTGate(TwoQubitsControlledGate):  # QuantumGate.h:118-147
    code = 24

    def __init__(self):
        super().__init__()
        m = self.operatorMat
        m[2, 2] = m[3, 3] = 0
        m[2, 3] = m[3, 2] = 1

    def isAntidiagonal(self) -> bool:
        return True


class ControlledYGate(TwoQubitsControlledGate):  # QuantumGate.h:149-168
    code = 25

    def __init__(self):
        super().__init__()
        m = self.operatorMat
        m[2, 2] = m[3, 3] = 0
        m[2, 3] = -1j
        m[3, 2] = 1j

    def isAntidiagonal(self) -> bool:
        return True


class ControlledZGate(TwoQubitsControlledGate):  # QuantumGate.h:170-185
    code = 26

    def __init__(self):
        super().__init__()
        self.operatorMat[3, 3] = -1

    def isDiagonal(self) -> bool:
        return True


class ControlledHadamardGate(TwoQubitsControlledGate):  # QuantumGate.h:187-201
    code = 27

    def __init__(self):
        super().__init__()
        self.SetOperation([[R2, R2], [R2, -R2]])


class ControlledSquareRootNOTGate(TwoQubitsControlledGate):  # QuantumGate.h:203-216
    code = 28

    def __init__(self):
        super().__init__()
        self.SetOperation([[0.5 + 0.5j, 0.5 - 0.5j], [0.5 - 0.5j, 0.5 + 0.5j]])


class ControlledSquareRootNOTDagGate(TwoQubitsControlledGate):  # QuantumGate.h:218-231
    code = 29

    def __init__(self):
        super().__init__()
        self.SetOperation([[0.5 - 0.5j, 0.5 + 0.5j], [0.5 + 0.5j, 0.5 - 0.5j]])


class ControlledPhaseGate(TwoQubitsControlledGate):  # QuantumGate.h:233-249
    code = 30

    def __init__(self):
        super().__init__()
        self.operatorMat[3, 3] = 1j

    def isDiagonal(self) -> bool:
        return True


class ControlledPhaseShiftGate(TwoQubitsControlledGate):  # QuantumGate.h:251-271
    code = 31

    def __init__(self, theta: float = 0.0):
        super().__init__()
        self.SetPhaseShift(theta)

    def SetPhaseShift(self, theta: float) -> None:
        self.theta = theta
        self.operatorMat[3, 3] = polar(theta)

    def isDiagonal(self) -> bool:
        return True

    def params(self):
        return (self.theta, 0.0, 0.0, 0.0)


class ControlledUGate(TwoQubitsControlledGate):  # QuantumGate.h:273-293
    code = 32

    def __init__(self, theta=0.0, phi=0.0, lam=0.0, gamma=0.0):
        super().__init__()
        self.SetParams(theta, phi, lam, gamma)

    def SetParams(self, theta=0.0, phi=0.0, lam=0.0, gamma=0.0):
        self._p = (theta, phi, lam, gamma)
        a, b, c, d = _u_entries(theta, phi, lam, gamma)
        m = self.operatorMat
        m[2, 2], m[2, 3], m[3, 2], m[3, 3] = a, b, c, d

    def params(self):
        return self._p


class ControlledRotationGate(TwoQubitsControlledGate):
    def __init__(self, theta: float = 0.0):
        super().__init__()
        self.SetTheta(theta)

    def params(self):
        return (self.theta, 0.0, 0.0, 0.0)


class ControlledRxGate(ControlledRotationGate):  # QuantumGate.h:305-325
    code = 33

    def SetTheta(self, theta: float) -> None:
        self.theta = theta
        t2 = theta * 0.5
        c, s = math.cos(t2), math.sin(t2)
        self.SetOperation([[complex(c, 0), complex(0, -s)], [complex(0, -s), complex(c, 0)]])


class ControlledRyGate(ControlledRotationGate):  # QuantumGate.h:327-347
    code = 34

    def SetTheta(self, theta: float) -> None:
        self.theta = theta
        t2 = theta * 0.5
        c, s = math.cos(t2), math.sin(t2)
        self.SetOperation([[c, -s], [s, c]])


class ControlledRzGate(ControlledRotationGate):  # QuantumGate.h:349-372
    code = 35

    def SetTheta(self, theta: float) -> None:
        self.theta = theta
        t2 = theta * 0.5
        self.operatorMat[2, 2] = polar(-t2)
        self.operatorMat[3, 3] = polar(t2)

    def isDiagonal(self) -> bool:
        return True


# ---- three qubits (ThreeQubitsGate starts from identity, SimpleGates.h:341-344) ----
class ThreeQubitsGate(QuantumGate):
    def __init__(self, matrix=None):
        super().__init__(np.eye(8) if matrix is None else matrix)

    def getQubitsNumber(self) -> int:
        return 3


class ThreeQubitsControlledGate(ThreeQubitsGate):  # QuantumGate.h:376-399
    def isControlled(self) -> bool:
        return True

    def isControlQubit(self, qubit: int) -> bool:
        return qubit == 0

    def SetOperation(self, U) -> None:
        self.operatorMat[4:8, 4:8] = U


class ToffoliGate(ThreeQubitsControlledGate):  # QuantumGate.h:401-426
    code = 40

    def __init__(self):
        super().__init__()
        m = self.operatorMat
        m[6, 6] = m[7, 7] = 0
        m[6, 7] = m[7, 6] = 1

    def isControlQubit(self, qubit: int) -> bool:
        return qubit <= 1

    def isAntidiagonal(self) -> bool:
        return True


class FredkinGate(ThreeQubitsControlledGate):  # QuantumGate.h:428-447
    code = 41

    def __init__(self):
        super().__init__()
        m = self.operatorMat
        m[5, 5] = m[6, 6] = 0
        m[5, 6] = m[6, 5] = 1

    def isSwapGate(self) -> bool:
        return True


class CCZGate(ThreeQubitsControlledGate):  # QuantumGate.h:449-469
    code = 42

    def __init__(self):
        super().__init__()
        self.operatorMat[7, 7] = -1

    def isControlQubit(self, qubit: int) -> bool:
        return qubit <= 1

    def isDiagonal(self) -> bool:
        return True


class AppliedGate(QuantumGate):
    """QC::Gates::AppliedGate (SimpleGates.h:439-578): a matrix with the qubits it was applied to and
    no trait overrides, used to record and replay gates."""

    def __init__(self, matrix, q1: int = 0, q2: int = 0, q3: int = 0):
        super().__init__(matrix)
        self.q1, self.q2, self.q3 = q1, q2, q3

    @property
    def code(self):  # CPU-oracle code for a matrix-only gate of this size
        return 49 + self.getQubitsNumber()

    def getQubit1(self) -> int:
        return self.q1

    def getQubit2(self) -> int:
        return self.q2

    def getQubit3(self) -> int:
        return self.q3


# name -> class, for circuit descriptions
BY_NAME = {
    "h": HadamardGate, "hy": HyGate, "s": SGate, "sdg": SDGGate, "t": TGate, "tdg": TDGGate,
    "p": PhaseShiftGate, "x": PauliXGate, "y": PauliYGate, "z": PauliZGate, "sx": SquareRootNOTGate,
    "sxdg": SquareRootNOTDagGate, "splitter": SplitterGate, "rx": RxGate, "ry": RyGate, "rz": RzGate,
    "u": UGate, "swap": SwapGate, "iswap": iSwapGate, "iswapdg": iSwapDagGate, "decrement": DecrementGate,
    "cx": CNOTGate, "cy": ControlledYGate, "cz": ControlledZGate, "ch": ControlledHadamardGate,
    "csx": ControlledSquareRootNOTGate, "csxdg": ControlledSquareRootNOTDagGate, "cs": ControlledPhaseGate,
    "cp": ControlledPhaseShiftGate, "cu": ControlledUGate, "crx": ControlledRxGate, "cry": ControlledRyGate,
    "crz": ControlledRzGate, "ccx": ToffoliGate, "cswap": FredkinGate, "ccz": CCZGate,
}
BY_CODE = {cls.code: cls for cls in BY_NAME.values()}

PARAM_COUNT = {PhaseShiftGate: 1, RxGate: 1, RyGate: 1, RzGate: 1, UGate: 4, ControlledPhaseShiftGate: 1,
               ControlledUGate: 4, ControlledRxGate: 1, ControlledRyGate: 1, ControlledRzGate: 1}


def make(name_or_code, *params) -> QuantumGate:
    cls = BY_NAME[name_or_code] if isinstance(name_or_code, str) else BY_CODE[name_or_code]
    n = PARAM_COUNT.get(cls, 0)
    return cls(*params[:n]) if n else cls()


def to_record(gate: QuantumGate, q0: int, q1: int = 0, q2: int = 0, out=None):
    """the qcs_gate record (include/qcs_gpu.h) for ApplyGate(gate, q0, q1, q2)"""
    rec = np.zeros((), dtype=L.GATE_DTYPE) if out is None else out
    m = gate.getRawOperatorMatrix()
    k = gate.getQubitsNumber()
    rec["k"], rec["q0"], rec["q1"], rec["q2"] = k, q0, q1, q2
    rec["traits"] = gate.traits()
    d = 1 << k
    flat = np.ascontiguousarray(m, dtype=np.complex128).reshape(-1).view(np.float64)
    rec["m"][: 2 * d * d] = flat
    rec["m"][2 * d * d:] = 0
    return rec


def records(gates) -> np.ndarray:
    """qcs_gate array from (gate, q0, q1, q2) tuples, the same records to_record makes one by one.  Each distinct
    gate object's matrix, size and traits are read once per call and the columns are filled with whole-array
    writes, so long lists that reuse a few gate objects (oracle expansions, controlled Grover iterations)
    convert quickly."""
    n = len(gates)
    arr = np.zeros(n, dtype=L.GATE_DTYPE)
    if n == 0:
        return arr
    slot: dict[int, int] = {}
    sizes, traits, mats = [], [], []
    inv = np.empty(n, dtype=np.intp)
    qs = []
    for i, g in enumerate(gates):
        gate = g[0]
        j = slot.get(id(gate))
        if j is None:
            j = slot[id(gate)] = len(sizes)
            sizes.append(gate.getQubitsNumber())
            traits.append(gate.traits())
            mats.append(np.ascontiguousarray(gate.getRawOperatorMatrix(), dtype=np.complex128).reshape(-1).view(np.float64))
        inv[i] = j
        qs.append((tuple(g) + (0, 0, 0))[1:4])
    q = np.array(qs, dtype=np.uint32)
    m = np.zeros((len(mats), arr["m"].shape[1]))
    for j, f in enumerate(mats):
        m[j, : f.size] = f
    arr["k"] = np.asarray(sizes, dtype=np.uint32)[inv]
    arr["traits"] = np.asarray(traits, dtype=np.uint32)[inv]
    arr["q0"], arr["q1"], arr["q2"] = q[:, 0], q[:, 1], q[:, 2]
    arr["m"] = m[inv]
    return arr


class PreparedGates:
    """a gate list converted once to engine records, for a circuit applied many times (QubitRegister.ApplyGates
    takes it in place of a list); ops keeps the (gate, q0, q1, q2) tuples"""

    def __init__(self, ops):
        self.ops = [op if isinstance(op, tuple) else (op, op.getQubit1(), op.getQubit2(), op.getQubit3()) for op in ops]
        self.recs = records(self.ops)

    def __len__(self) -> int:
        return len(self.ops)


def cmatrix(m) -> np.ndarray:
    return np.asarray(m, dtype=np.complex128)


__all__ = [n for n in dir() if n[0].isupper() or n in ("make", "to_record", "records", "polar")]
