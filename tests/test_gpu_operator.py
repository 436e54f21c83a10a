"""The dense operator on chosen qubits (qcs_apply_operator_on_qubits) on the GPU: QCSim's
NQubitsQuantumGate / NQubitsControlledQuantumGate results from tests/golden/nqubits.npz, arbitrary target
and control placements against the oracle's contraction (k = 1 .. 10), both precisions, argument checks.
FP64 tolerance 1e-13 on amplitudes; FP32 2e-6."""
import ctypes as C
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FX = Path(__file__).resolve().parent / "golden" / "nqubits.npz"


@pytest.fixture(scope="module")
def Q():
    import qcsim_gb300
    from qcsim_gb300 import _lib
    try:
        _lib.load()
    except _lib.EngineUnavailable as e:
        pytest.fail(f"engine not built: {e}")
    return qcsim_gb300


def rand_op(rng, k):
    d = 1 << k
    return (rng.standard_normal((d, d)) + 1j * rng.standard_normal((d, d))) / np.sqrt(d)


def rand_state(rng, n):
    v = rng.standard_normal(1 << n) + 1j * rng.standard_normal(1 << n)
    return v / np.linalg.norm(v)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_nqubits_gates_match_reference(Q, precision):
    from qcsim_gb300 import subalgo as A
    fx = np.load(FX)
    tol = 1e-13 if precision == "fp64" else 2e-6
    for i, (n, k, ctrl) in enumerate(fx["cases"]):
        n, k, ctrl = int(n), int(k), int(ctrl)
        reg = Q.QubitRegister(n, seed=1, precision=precision)
        reg.setRegisterStorageFastNoNormalize(fx[f"psi{i}"])
        g = A.NQubitsQuantumGate(n, fx[f"op{i}"], n - k) if ctrl < 0 else A.NQubitsControlledQuantumGate(n, fx[f"op{i}"], n - k, ctrl)
        g.Execute(reg)
        assert np.abs(reg.getRegisterStorage() - fx[f"out{i}"]).max() < tol, (i, n, k, ctrl)
        reg.close()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_operator_on_any_qubits(Q, precision):
    from oracle import nqubits as O
    rng = np.random.default_rng(11 if precision == "fp64" else 12)
    n = 12
    tol = 1e-13 if precision == "fp64" else 2e-6
    for k in range(1, 11):
        for _ in range(2):
            qs = [int(q) for q in rng.permutation(n)[:k]]
            rest = [q for q in range(n) if q not in qs]
            ctrls = [int(q) for q in rng.permutation(rest)[: int(rng.integers(0, min(2, len(rest)) + 1))]]
            op, psi = rand_op(rng, k), rand_state(rng, n)
            reg = Q.QubitRegister(n, seed=1, precision=precision)
            reg.setRegisterStorageFastNoNormalize(psi)
            reg.ApplyOperatorOnQubits(op, qs, ctrls)
            want = O.apply_on_qubits(psi, op, qs, ctrls)
            assert np.abs(reg.getRegisterStorage() - want).max() < tol, (k, qs, ctrls)
            reg.close()


def test_operator_on_larger_register(Q):
    """22 qubits, a 6-qubit operator spread over low, middle and top qubits with one control, on a register
    carrying a pending global factor from single gates"""
    from oracle import nqubits as O
    from qcsim_gb300 import gates as G
    rng = np.random.default_rng(21)
    n = 22
    psi = rand_state(rng, n)
    reg = Q.QubitRegister(n, seed=1)
    reg.setRegisterStorageFastNoNormalize(psi)
    reg.set_passes(False)
    for q in (2, 9, 16):
        reg.ApplyGate(G.RyGate(0.3), q)
    qs, ctrls = [0, 5, 11, 17, 20, 21], [3]
    op = rand_op(rng, 6)
    reg.ApplyOperatorOnQubits(op, qs, ctrls)
    want = psi
    for q in (2, 9, 16):
        want = O.apply_on_qubits(want, G.RyGate(0.3).getRawOperatorMatrix(), [q])
    want = O.apply_on_qubits(want, op, qs, ctrls)
    assert np.abs(reg.getRegisterStorage() - want).max() < 1e-13
    reg.close()


def test_recording_register_keeps_the_extended_matrix(Q):
    """with gate recording on, Execute logs and applies the extended matrix as the reference does; the
    result equals the device path's"""
    from qcsim_gb300 import subalgo as A
    rng = np.random.default_rng(4)
    n, k = 7, 3
    op, psi = rand_op(rng, k), rand_state(rng, n)
    outs = []
    for record in (False, True):
        reg = Q.QubitRegister(n, seed=1)
        reg.setRegisterStorageFastNoNormalize(psi)
        if record:
            reg.ComputeStart()
        A.NQubitsControlledQuantumGate(n, op, n - k, 1).Execute(reg)
        if record:
            reg.ComputeEnd()
            assert len(reg.computeGates) == 1 and reg.computeGates[0].getRawOperatorMatrix().shape == (1 << n, 1 << n)
        outs.append(reg.getRegisterStorage())
        reg.close()
    assert np.abs(outs[0] - outs[1]).max() < 1e-14


def test_operator_argument_checks(Q):
    from qcsim_gb300 import _lib as L
    lib = L.load()
    n = 8
    reg = Q.QubitRegister(n, seed=1)
    reg.setToEqualSuperposition()
    before = reg.getRegisterStorage().copy()

    def call(k, qubits, ctrl):
        m = np.ascontiguousarray(np.eye(1 << max(k, 0), dtype=np.complex128))
        qs = np.ascontiguousarray(qubits, dtype=np.uint32)
        return lib.qcs_apply_operator_on_qubits(reg.handle, m.view(np.float64).ctypes.data_as(C.POINTER(C.c_double)), k,
                                                qs.ctypes.data_as(C.POINTER(C.c_uint32)), ctrl)

    assert call(0, [0], 0) == L.QCS_INVALID_ARGUMENT
    assert call(2, [1, 1], 0) == L.QCS_INVALID_ARGUMENT
    assert call(2, [1, 8], 0) == L.QCS_INVALID_ARGUMENT
    assert call(2, [1, 2], 1 << 2) == L.QCS_INVALID_ARGUMENT
    assert call(2, [1, 2], 1 << 8) == L.QCS_INVALID_ARGUMENT
    assert call(11, list(range(11)), 0) == L.QCS_INVALID_ARGUMENT
    assert np.array_equal(reg.getRegisterStorage(), before)
    reg.close()
