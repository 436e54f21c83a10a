"""QCSim's algorithms over the engine, through the Python mirror of their classes: phase estimation
(PhaseEstimation.h, with its controlled powers of U as NQubitsControlledQuantumGate on the device) and
Grover's search with the diagonal oracle matrix (GroverAlgorithm.h).  The pre-measurement states are
compared with a statevector computed by the oracle's contraction on the host (1e-12), and the measured
answers with the checks of QCSim's own tests (PhaseEstimationTests.cpp:71-125: estimate within 0.05)."""
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


def host_hadamards(v, qubits):
    from oracle import nqubits as O
    h = np.array([[1, 1], [1, -1]], dtype=np.complex128) / math.sqrt(2)
    for q in qubits:
        v = O.apply_on_qubits(v, h, [q])
    return v


def host_phase_estimation(U, N, L):
    """the circuit of PhaseEstimation::ExecuteWithoutMeasurement, before the IQFT"""
    from oracle import nqubits as O
    v = np.zeros(1 << N, dtype=np.complex128)
    v[1 << L] = 1
    v = host_hadamards(v, range(L))
    cg = U.copy()
    k = int(U.shape[0] - 1).bit_length()
    for ctrl in range(L - 1, 0, -1):
        v = O.apply_on_qubits(v, cg, list(range(L, L + k)), [ctrl])
        cg = cg @ cg
    return O.apply_on_qubits(v, cg, list(range(L, L + k)), [0])


@pytest.mark.parametrize("phase", [1 / 4, 1 / 3, 1 / 2, 2 / 3, 3 / 4])
def test_phase_estimation(Q, phase):
    from qcsim_gb300 import algorithms as A, gates as G
    U = G.PhaseShiftGate(phase * 2 * math.pi).getRawOperatorMatrix()
    pe = A.PhaseEstimation(U, 4, 3)
    reg = Q.QubitRegister(4, seed=7)
    reg.setToQubitState(3)
    counts = pe.ExecuteWithMultipleMeasurements(reg, 10000)
    ranked = sorted(counts.items(), key=lambda kv: -kv[1])
    mx, cnt = ranked[0]
    assert abs(mx / 8 - phase) <= 0.05, (phase, ranked[:3])
    second = ranked[1][0] if len(ranked) > 1 else -1
    assert abs(pe.getPhase(mx, second, cnt / 10000) - phase) < 0.05
    # the state before the measurements
    reg2 = Q.QubitRegister(4, seed=7)
    pe.ExecuteWithoutMeasurement(reg2)
    want = host_phase_estimation(np.asarray(U), 4, 3)
    from oracle import bind as B
    ref = B.OracleRegister(4)
    ref.set_state(want)
    B.oracle().qo_qft(ref.h, 0, 2, 1, 0)
    assert np.abs(reg2.getRegisterStorage() - ref.state()).max() < 1e-12
    reg.close()
    reg2.close()


@pytest.mark.parametrize("n,marked", [(6, 45), (10, 613), (11, 1777)])
def test_grover(Q, n, marked):
    from qcsim_gb300 import algorithms as A
    g = A.GroverAlgorithm(n, seed=3)
    g.setCorrectQuestionState(marked)
    g.ExecuteWithoutMeasurement()
    got = g.getRegisterStorage()
    v = np.full(1 << n, 1 / math.sqrt(1 << n), dtype=np.complex128)
    for _ in range(int(math.floor(math.pi / 4 * math.sqrt(1 << n) + 0.5))):
        v[marked] *= -1
        v = host_hadamards(v, range(n))
        v[0] *= -1
        v = host_hadamards(v, range(n))
    assert np.abs(got - v).max() < 1e-12
    assert abs(got[marked]) ** 2 > 0.99
    counts = g.RepeatedMeasure(1000)
    assert max(counts, key=counts.get) == marked
    g.close()


@pytest.mark.parametrize("carry", [False, True])
def test_draper_adders(Q, carry):
    """every pair of 3-bit inputs (AdderTests.cpp:270-340 draws random ones): the register ends in the basis
    state a | (a + b) << 3, the sum mod 8 without the carry qubit, the full 4-bit sum with it"""
    from qcsim_gb300 import algorithms as A
    n = 3
    adder = A.DraperAdderWithCarry(n, seed=5) if carry else A.DraperAdder(n, seed=5)
    for a in range(8):
        for b in range(8):
            adder.setToBasisState(a | (b << n))
            adder.ExecuteWithoutMeasurement()
            s = a + b if carry else (a + b) % 8
            want = a | (s << n)
            state = adder.getRegisterStorage()
            assert abs(abs(state[want]) - 1) < 1e-12, (a, b, carry)
            assert adder.Measure() == want
    adder.close()


def test_bernstein_vazirani(Q):
    """the measured value is the hidden string, with probability 1 (BernsteinVazirani.h:83-91)"""
    from qcsim_gb300 import algorithms as A
    rng = np.random.default_rng(17)
    for n in (4, 9):
        bv = A.BernsteinVaziraniAlgorithm(n, seed=2)
        for s in [0, (1 << n) - 1] + [int(x) for x in rng.integers(0, 1 << n, 6)]:
            bv.setString(s)
            assert bv.Execute() == s
            assert abs(bv.getBasisStateProbability(s) - 1) < 1e-12
        bv.close()


@pytest.mark.parametrize("sign", [False, True])
def test_three_qubit_codes(Q, sign):
    """ErrorCorrectionTests.cpp:25-80 (flip) and its sign counterpart: for random states and every error
    position, the syndrome names the flipped qubit and qubit 0 carries the original state (fidelity of
    the collapsed register with alpha|m> + beta|m+1>, m = syndrome << 1)"""
    from qcsim_gb300 import algorithms as A
    rng = np.random.default_rng(23 + sign)
    code = A.ErrorCorrection3QubitsSign(seed=4) if sign else A.ErrorCorrection3QubitsFlip(seed=4)
    for _ in range(6):
        a, b = complex(*rng.uniform(-1, 1, 2)), complex(*rng.uniform(-1, 1, 2))
        nrm = math.sqrt(abs(a) ** 2 + abs(b) ** 2)
        a, b = a / nrm, b / nrm
        for q in range(4):
            code.SetState(a, b)
            code.SetErrorQubit(q)
            res = code.Execute()
            assert res == {0: 3, 1: 1, 2: 2, 3: 0}[q], (q, res)
            want = np.zeros(8, dtype=np.complex128)
            want[res << 1], want[(res << 1) | 1] = a, b
            assert code.stateFidelity(want) > 1 - 1e-12
    code.close()


def host_shor_state(C, N, L, a):
    """PhaseEstimation.h:129-145 on the host: f register = 1, Hadamards on x, the controlled multiplications
    (the reference's 2^N x 2^N matrices, built here from their definition), then the oracle's IQFT"""
    from oracle import bind as B
    v = np.zeros(1 << N, dtype=np.complex128)
    v[1 << L] = 1
    v = host_hadamards(v, range(L))
    an = a
    for l in range(L):
        out = np.zeros_like(v)
        for k in range(1 << N):
            x, f = k & ((1 << L) - 1), k >> L
            if (x >> l) & 1 and f < C:
                out[(((an % C) * f) % C) << L | x] += v[k]
            else:
                out[k] += v[k]
        v = out
        an = (an * an) & 0xFFFFFFFFFFFFFFFF
    ref = B.OracleRegister(N)
    ref.set_state(v)
    B.oracle().qo_qft(ref.h, 0, L - 1, 1, 1)
    return ref.state()


@pytest.mark.parametrize("C,N,L,a", [(15, 7, 3, 7), (15, 7, 3, 2), (21, 9, 4, 5)])
def test_shor_period_finding(Q, C, N, L, a):
    """the pre-measurement state against the host; measured x values are multiples of 2^L / r (r = the order of
    a mod C, when r divides 2^L)"""
    from qcsim_gb300 import algorithms as A
    shor = A.ShorAlgorithm(C, N, L, seed=11)
    shor.setA(a)
    shor.phaseEstimation.ExecuteWithoutMeasurement(shor.reg)
    assert np.abs(shor.getRegisterStorage() - host_shor_state(C, N, L, a)).max() < 1e-12
    r = next(k for k in range(1, C) if pow(a, k, C) == 1)
    if (1 << L) % r == 0:
        counts = shor.reg.RepeatedMeasure(2000)
        xs = {s & ((1 << L) - 1) for s in counts}
        assert xs <= {m * ((1 << L) // r) for m in range(r)}, (xs, r)
    shor.close()


def test_shor_factorizes_15(Q):
    """Tests.cpp:76-88: 15 = 5 x 3"""
    from qcsim_gb300 import algorithms as A
    found = False
    for seed in range(5):
        shor = A.ShorAlgorithm(15, 7, 3, seed=seed, factor_seed=seed)
        used, p1, p2 = shor.factorize()
        shor.close()
        assert sorted((p1, p2)) == [3, 5], (used, p1, p2)
        found = found or used
    assert found


def test_vqe_energy_estimate_and_search(Q):
    """VQETests.cpp:9-65: H = 3X - 2Y + Z on one qubit (ground energy -sqrt(14)); the sampled energy of a point
    agrees with the exact expectation of the same circuit, and the Nelder-Mead search ends below -3"""
    from qcsim_gb300 import vqe as V
    rng = np.random.default_rng(31)
    solver = V.VariationalQuantumEigensolver(1, seed=9)
    for op, c in (("X", 3.0), ("Y", -2.0), ("Z", 1.0)):
        t = V.PauliStringVQE(1)
        t.setOperatorForQubit(0, op)
        t.setCoefficient(c)
        solver.AddTerm(t)
    th, ph = 1.1, 2.3
    # exact <H> of RZ(ph) RY(th)|0>: Bloch vector (sin th cos ph, sin th sin ph, cos th)
    exact = 3 * math.sin(th) * math.cos(ph) - 2 * math.sin(th) * math.sin(ph) + math.cos(th)
    est = solver.EstimateEnergy([th, ph], 40000)
    assert abs(est - exact) < 0.1, (est, exact)
    theta, phi, radius = rng.uniform() * math.pi / 2, rng.uniform() * math.pi, 0.35
    R = rng.uniform() * 2 * math.pi / 3
    solver.SetVertices([[theta + radius * math.cos(R + v * 2 * math.pi / 3), phi + radius * math.sin(R + v * 2 * math.pi / 3)]
                        for v in range(3)])
    solver.Execute()
    assert solver.GetMinEnergy() < -3.0, solver.GetMinEnergy()
    assert len(solver.GetMinVertex()) == 2
    solver.close()
