"""Edge cases of the engine on the GPU: empty gate lists and shot counts, one-qubit registers, a one-qubit QFT,
a dense operator on every qubit of the register, zero Trotter steps, one-qubit sub-register measurements.
Expected values are QCSim's (QubitRegister.h:227-237 for zero and one shot) or the oracle's."""
import math

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


def rand_state(n, seed):
    r = np.random.default_rng(seed)
    v = r.standard_normal(1 << n) + 1j * r.standard_normal(1 << n)
    return v / np.linalg.norm(v)


@pytest.mark.parametrize("n,precision", [(3, "fp64"), (16, "fp64"), (16, "fp32")])
def test_empty_inputs(Q, n, precision):
    from qcsim_gb300 import gates as G
    v = rand_state(n, 1)
    reg = Q.QubitRegister(n, seed=1, precision=precision)
    reg.setRegisterStorageFastNoNormalize(v)
    before = reg.getRegisterStorage().copy()
    reg.ApplyGates([])
    reg.apply_records(G.records([]))
    assert np.array_equal(reg.getRegisterStorage(), before)
    assert reg.RepeatedMeasure(0) == {} and reg.RepeatedMeasure(0, n - 1, 0) == {}
    one = reg.RepeatedMeasure(1)
    assert len(one) == 1 and sum(one.values()) == 1
    assert np.array_equal(reg.getRegisterStorage(), before)  # no collapse
    reg.close()


def test_one_qubit_register(Q):
    from oracle import bind as B
    from qcsim_gb300 import subalgo as A, gates as G
    for precision, tol in (("fp64", 1e-15), ("fp32", 1e-7)):
        reg = Q.QubitRegister(1, seed=3, precision=precision)
        reg.ApplyGate(G.HadamardGate(), 0)
        reg.ApplyGate(G.RzGate(0.7), 0)
        ref = B.OracleRegister(1)
        ref.set_state(np.array([1, 0], dtype=np.complex128))
        ref.apply([(G.HadamardGate(), 0), (G.RzGate(0.7), 0)])
        assert np.abs(reg.getRegisterStorage() - ref.state()).max() < tol
        assert abs(reg.GetQubitProbability(0) - 0.5) < tol
        A.QuantumFourierTransform(1).QFT(reg)  # a one-qubit QFT is a Hadamard
        ref.apply([(G.HadamardGate(), 0)])
        assert np.abs(reg.getRegisterStorage() - ref.state()).max() < tol
        counts = reg.RepeatedMeasure(2000)
        assert set(counts) <= {0, 1} and sum(counts.values()) == 2000
        assert reg.MeasureAll() in (0, 1)
        reg.close()


def test_operator_on_every_qubit(Q):
    """a dense operator over the whole register equals ApplyOperatorMatrix with the same matrix"""
    rng = np.random.default_rng(5)
    n = 6
    u = np.linalg.qr(rng.standard_normal((64, 64)) + 1j * rng.standard_normal((64, 64)))[0]
    v = rand_state(n, 2)
    a = Q.QubitRegister(n, seed=1)
    a.setRegisterStorageFastNoNormalize(v)
    a.ApplyOperatorOnQubits(u, list(range(n)))
    b = Q.QubitRegister(n, seed=1)
    b.setRegisterStorageFastNoNormalize(v)
    b.ApplyOperatorMatrix(u)
    assert np.abs(a.getRegisterStorage() - u @ v).max() < 1e-13
    assert np.abs(a.getRegisterStorage() - b.getRegisterStorage()).max() < 1e-13
    a.close()
    b.close()


def test_zero_trotter_steps(Q):
    from qcsim_gb300.schrodinger import SchrodingerSimulation
    sim = SchrodingerSimulation(14, 0.01, 0.1, 0)
    sim.setGaussian(4096, 30.0, 5.0)
    before = sim.getRegisterStorage().copy()
    sim.Execute()
    assert np.abs(sim.getRegisterStorage() - before).max() < 1e-15
    sim.close()


def test_one_qubit_sub_register_measurement(Q):
    """Measure(q, q) returns that qubit's value and collapses only it"""
    from qcsim_gb300 import gates as G
    n = 5
    reg = Q.QubitRegister(n, seed=12)
    reg.ApplyGates([(G.HadamardGate(), q) for q in range(n)])
    m = reg.Measure(2, 2)
    assert m in (0, 1)
    st = reg.getRegisterStorage()
    on = np.array([((i >> 2) & 1) == m for i in range(1 << n)])
    assert np.abs(st[~on]).max() == 0
    assert np.abs(np.abs(st[on]) - 1 / math.sqrt(1 << (n - 1))).max() < 1e-14
    reg.close()
