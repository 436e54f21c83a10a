"""CPU oracle for the dense operator gates -- TEST INFRASTRUCTURE ONLY.

Only tests/ use this module, as the checker of qcs_apply_operator_on_qubits.

extended_operator restates the getOperatorMatrix loops of QCSim's SubAlgo::NQubitsQuantumGate
(NQubitsQuantumGate.h:29-46) and SubAlgo::NQubitsControlledQuantumGate
(NQubitsControlledQuantumGate.h:29-60), with the end qubit of QuantumSubAlgorithmOnSubregister
(QuantumAlgorithm.h:228-231); applying that matrix is QubitRegister::ApplyOperatorMatrix
(QubitRegister.h:499-505).  apply_on_qubits is the same operation for any set of target and control
qubits, written as a tensor contraction; it checks placements the reference's classes cannot express.
"""
from __future__ import annotations

import numpy as np


def operator_qubits(op: np.ndarray) -> int:
    """getOperatorQubitsNumber (NQubitsQuantumGate.h:61-72)"""
    return int(op.shape[0] - 1).bit_length()


def extended_operator(n: int, op: np.ndarray, start: int, ctrl: int | None = None) -> np.ndarray:
    """the 2^n x 2^n matrix the reference builds: entry (i, j) is op((i & mask) >> start, (j & mask) >> start)
    where i and j agree outside mask (the qubits start .. end); controlled, only where the controlling
    qubit is one in both, the identity's entry where it is zero in both, and zero otherwise"""
    k = operator_qubits(op)
    end = max(start, min(n - 1, start + k))
    mask = 0
    for q in range(start, end + 1):
        mask |= 1 << q
    nb = 1 << n
    j = np.arange(nb)
    ext = np.zeros((nb, nb), dtype=np.complex128)
    eye = np.eye(op.shape[0], dtype=np.complex128)
    cbit = 0 if ctrl is None else 1 << ctrl
    for i in range(nb):
        sel = (j | mask) == (i | mask)
        r = (i & mask) >> start
        c = (j[sel] & mask) >> start
        if ctrl is None:
            ext[i, sel] = op[r, c]
            continue
        both_on = (i & cbit) != 0 and ((j[sel] & cbit) != 0)
        both_off = (i & cbit) == 0 and ((j[sel] & cbit) == 0)
        row = np.zeros(c.size, dtype=np.complex128)
        row[both_on] = op[r, c[both_on]]
        row[both_off] = eye[r, c[both_off]]
        ext[i, sel] = row
    return ext


def apply_on_qubits(state: np.ndarray, op: np.ndarray, qubits, controls=()) -> np.ndarray:
    """state with op applied on the target qubits (matrix bit j = qubits[j]) wherever every control
    qubit is one"""
    n = int(state.size).bit_length() - 1
    k = len(qubits)
    psi = state.reshape((2,) * n).copy()  # axis a holds qubit n - 1 - a
    axis = lambda q: n - 1 - q  # noqa: E731
    sub = [slice(None)] * n
    for c in controls:
        sub[axis(c)] = 1
    sub = tuple(sub)
    block = psi[sub]
    # the block keeps the axes of the qubits that are not controls, in the same order
    kept = [q for q in range(n - 1, -1, -1) if q not in set(controls)]
    pos = {q: a for a, q in enumerate(kept)}
    # op as a tensor: output bits (k-1 .. 0), then input bits (k-1 .. 0)
    t = op.reshape((2,) * (2 * k))
    in_axes = [pos[qubits[j]] for j in range(k - 1, -1, -1)]
    out = np.tensordot(t, block, axes=(list(range(k, 2 * k)), in_axes))
    # tensordot puts the k output axes first, then the remaining block axes in order
    rest = [a for a in range(len(kept)) if a not in in_axes]
    order = [0] * len(kept)
    for idx, a in enumerate(in_axes):
        order[a] = idx
    for idx, a in enumerate(rest):
        order[a] = k + idx
    psi[sub] = np.transpose(out, order)
    return psi.reshape(-1)
