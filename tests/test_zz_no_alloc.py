"""qcs_qubit_probability_noalloc (the qubit probability through the library's fixed device array)
against qcs_qubit_probability, and the property it exists for: the register allocates no scratch.
Collected last so that it also runs after every other GPU test has used the library, and passes when
run alone.  Tolerance 1e-12 for FP64 and FP32 registers alike: both entry points square and sum in
double precision and scale the sum by the pending global factor; they differ only in the order of
their additions."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def Q():
    import qcsim_gb300
    from qcsim_gb300 import _lib
    try:
        _lib.load()
    except _lib.EngineUnavailable as e:
        pytest.fail(f"engine not built: {e}")
    return qcsim_gb300


def prepared(Q, n, precision, seed):
    from qcsim_gb300 import circuits
    reg = Q.QubitRegister(n, precision=precision, seed=seed)
    reg.setRegisterStorage(circuits.random_normal_state(n, seed))
    # rotations leave a pending global factor on the register, which the result must include
    reg.ApplyGates(circuits.layered_circuit(n, 3, seed, p3=0.05, controlled_frac=0.3))
    return reg


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("fp32", 1e-12)])
def test_two_calls_in_a_row_match_allocating_entry_point(Q, precision, tol):
    # sizes from one block (2^13 amplitudes with the bit set) to many blocks, a larger register first
    # so that the smaller one reuses array slots the larger one wrote
    for n, seed in [(22, 3), (14, 4), (26, 5), (1, 6)]:
        reg = prepared(Q, n, precision, seed)
        qubits = sorted({q for q in (0, 1, n // 2, n - 1) if q < n})
        first = [reg.GetQubitProbabilityNoAlloc(q) for q in qubits]
        second = [reg.GetQubitProbabilityNoAlloc(q) for q in qubits]
        want = [reg.GetQubitProbability(q) for q in qubits]
        assert first == second, (n, precision)
        np.testing.assert_allclose(first, want, rtol=0, atol=tol, err_msg=f"n={n} {precision}")
        assert 0.0 < min(first) and max(first) < 1.0
        # a qubit above the register: no amplitude has the bit set, as with the allocating call
        assert reg.GetQubitProbabilityNoAlloc(n + 3) == reg.GetQubitProbability(n + 3) == 0.0


def scratch_bytes(reg) -> tuple[int, int]:
    import ctypes as C
    from qcsim_gb300 import _lib
    dev, pinned = C.c_uint64(), C.c_uint64()
    assert _lib.load().qcs_scratch_bytes(reg.handle, C.byref(dev), C.byref(pinned)) == _lib.QCS_OK
    return dev.value, pinned.value


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_allocates_nothing(Q, precision):
    """on a fresh register whose scratch nothing has touched, the call leaves the register without
    scratch, while the allocating entry point then allocates it"""
    from qcsim_gb300 import circuits
    n = 20
    reg = Q.QubitRegister(n, precision=precision, seed=2)
    reg.setToEqualSuperposition()
    reg.ApplyGates(circuits.layered_circuit(n, 2, 7))
    assert scratch_bytes(reg) == (0, 0)
    p = [reg.GetQubitProbabilityNoAlloc(q) for q in (0, 5, n - 1)]
    assert scratch_bytes(reg) == (0, 0)
    want = [reg.GetQubitProbability(q) for q in (0, 5, n - 1)]
    assert scratch_bytes(reg)[0] > 0
    np.testing.assert_allclose(p, want, rtol=0, atol=1e-12)
    reg.close()


def test_basis_state_exact(Q):
    reg = Q.QubitRegister(20, seed=1)
    reg.setToBasisState(0b1010_0000_0000_0000_0101)
    got = [reg.GetQubitProbabilityNoAlloc(q) for q in range(20)]
    want = [float((0b1010_0000_0000_0000_0101 >> q) & 1) for q in range(20)]
    assert got == want


def test_rejects_registers_above_its_array(Q):
    from qcsim_gb300 import _lib
    reg = Q.QubitRegister(33, precision="fp32", seed=1)  # 2^33 amplitudes, 64 GiB
    with pytest.raises(_lib.QcsError, match="at most 32 qubits"):
        reg.GetQubitProbabilityNoAlloc(0)
    assert reg.GetQubitProbability(0) == 0.0  # the allocating entry point still serves it
    del reg
