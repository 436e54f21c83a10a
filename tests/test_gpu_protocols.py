"""QCSim's oracle algorithms, teleportation family and quantum counting over the engine, through the Python
mirror of their classes, with the checks of QCSim's own tests: Deutsch-Jozsa (DeutschJozsaTests.cpp),
Simon (SimonAlgorithm.h:167-248), superdense coding (Tests.cpp:279-301), teleportation and entanglement
swapping (TeleportationTests.cpp, approxEqual at 1e-10), quantum counting (Tests.cpp:619-663), the
statevector expectation values (Tests.cpp:665-723), the CHSH inequality (Tests.cpp:303-330) and BB84
(Tests.cpp:474-520), the distributed CNOTs (DistributedTests.cpp), the nine-qubit Shor code
(ErrorCorrectionTests.cpp:150-205), the qubit adders (AdderTests.cpp:9-150), the paradoxes (ParadoxesTests.cpp)
and coin flipping (GamesTests.cpp:9-26).  The counting circuit's final state is also compared with the CPU
oracle (1e-12)."""
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


@pytest.mark.parametrize("N", [2, 3, 5, 9])
def test_deutsch_jozsa(Q, N):
    from qcsim_gb300 import algorithms as A
    FT = A.DeutschJozsaAlgorithm.FunctionType
    dj = A.DeutschJozsaAlgorithm(N, seed=N, function_seed=N)
    for i in range(15):
        ft = FT.constantZero if i < 5 else FT.constantOne if i < 10 else FT.balanced
        dj.setFunction(ft)
        assert dj.WasConstantResult(dj.Execute()) == (ft != FT.balanced), (N, i)
    dj.close()


@pytest.mark.parametrize("N", [2, 3, 4])
def test_simon(Q, N):
    from qcsim_gb300 import algorithms as A
    simon = A.SimonAlgorithm(N, seed=7, function_seed=N)
    for s in range(1 << N):
        simon.setString(s)
        assert simon.f.checkFunction()
        assert simon.Execute() == s, (N, s)
    simon.close()


def test_superdense_coding(Q):
    from qcsim_gb300 import teleportation as T
    coding = T.SuperdenseCoding(seed=3)
    for bit1 in (False, True):
        for bit2 in (False, True):
            for _ in range(3):
                coding.SetBits(bit1, bit2)
                got = coding.Execute()
                assert (bool(got & 1), bool(got & 2)) == (bit1, bit2)
    coding.close()


def _random_qubit_state(rng):
    a = complex(*rng.uniform(-1, 1, 2))
    b = complex(*rng.uniform(-1, 1, 2))
    n = np.sqrt(abs(a) ** 2 + abs(b) ** 2)
    return a / n, b / n


def test_teleportation(Q):
    """TeleportationTests (TeleportationTests.cpp:120-170): basis states arrive as measured; a generic state
    arrives on qubit 2 next to the two measured bits, with explicit and with coherent correction"""
    from qcsim_gb300 import teleportation as T
    rng = np.random.default_rng(5)
    qt = T.QuantumTeleportationRealization(seed=11)
    for i in range(12):
        up = bool(i % 2)
        qt.SetState(0, 1) if up else qt.SetState(1, 0)
        assert qt.Execute() == int(up)
    for i in range(16):
        alpha, beta = _random_qubit_state(rng)
        qt.SetState(alpha, beta)
        bits = qt.Teleport(i >= 8)
        assert abs(qt.getBasisStateAmplitude(bits) - alpha) < 1e-10
        assert abs(qt.getBasisStateAmplitude(4 | bits) - beta) < 1e-10
    qt.close()


def test_teleport_sub_algorithm(Q):
    """TeleportTests (TeleportationTests.cpp:9-72): QC::SubAlgo::Teleport over a bare register"""
    from qcsim_gb300 import QubitRegister
    from qcsim_gb300 import teleportation as T
    rng = np.random.default_rng(6)
    tp = T.Teleport()
    reg = QubitRegister(3, seed=13)
    for i in range(10):
        reg.setToBasisState(i % 2)
        tp.Execute(reg)
        assert reg.MeasureQubit(2) == i % 2
    for _ in range(16):
        alpha, beta = _random_qubit_state(rng)
        reg.Clear()
        reg.setRawAmplitude(0, alpha)
        reg.setRawAmplitude(1, beta)
        reg.Normalize()
        bits = tp.Execute(reg)
        assert abs(reg.getBasisStateAmplitude(bits) - alpha) < 1e-10
        assert abs(reg.getBasisStateAmplitude(4 | bits) - beta) < 1e-10
    reg.close()


def test_entanglement_swapping(Q):
    """EntanglementSwappingTests (TeleportationTests.cpp:74-118): the Bell pair sent on (0, 2) ends on (4, 5)"""
    from qcsim_gb300 import QubitRegister
    from qcsim_gb300 import teleportation as T
    es = T.EntanglementSwapping(seed=17)
    bell = T.BellState()
    reg = QubitRegister(2, seed=1)
    for i in range(16):
        s1, s2 = bool(i & 1), bool(i & 2)
        bell.setBellState(reg, 0, 1, s1, s2)
        es.SetBellStateToBeSent(s1, s2)
        meas = es.Teleport(i >= 8)
        v = es.getRegisterStorage()
        expect = reg.getRegisterStorage()
        for state in range(64):
            want = expect[state >> 4] if (state & 0xF) == meas else 0
            assert abs(v[state] - want) < 1e-10, (i, state)
    es.close()
    reg.close()


def test_quantum_counting_state_matches_oracle(Q):
    """the 14-qubit counting register (6 precision, 4 Grover qubits, 5 marked states) after the controlled
    Grover iterations and the inverse QFT, against the CPU oracle"""
    from oracle import bind as B
    from qcsim_gb300 import counting as C
    qc = C.QuantumCountingAlgorithm(6, 4, seed=2)
    qc.SetMarkedStates([1, 4, 7, 10, 13])
    ref = B.OracleRegister(14)
    ref.apply(qc.circuit())
    assert B.oracle().qo_qft(ref.h, 0, 5, 1, 0) == 0
    qc.ExecuteWithoutMeasurement()
    assert np.max(np.abs(qc.getRegisterStorage() - ref.state())) < 1e-12
    qc.close()


def test_quantum_counting(Q):
    """CountingTests (Tests.cpp:619-663): for 0..16 marked states of 4 Grover qubits, the most measured value of
    the 6 precision qubits (10000 shots) gives the number of marked states"""
    from qcsim_gb300 import counting as C
    rng = np.random.default_rng(9)
    for marked in range(17):
        qc = C.QuantumCountingAlgorithm(6, 4, seed=marked)
        qc.SetMarkedStates(rng.permutation(16)[:marked].tolist())
        res = qc.ExecuteWithMultipleMeasurements(10000)
        state = max(res.items(), key=lambda kv: kv[1])[0]
        assert qc.GetCountForState(state) == marked, (marked, res)
        qc.close()


def test_expectation_values_statevector(Q):
    """checkExpectationValuesStatevector (Tests.cpp:665-723): <I> = 1, <Z0> = 1, -1 after X, 0 after H, <Z1> = 0"""
    from qcsim_gb300 import gates as G
    reg = Q.QubitRegister(3, seed=1)
    z0 = [G.AppliedGate(G.PauliZGate().getRawOperatorMatrix(), 0)]
    assert abs(reg.ExpectationValue([]) - 1.0) <= 1e-6
    assert abs(reg.ExpectationValue(z0) - 1.0) <= 1e-6
    reg.ApplyGate(G.PauliXGate(), 0)
    assert abs(reg.ExpectationValue(z0) + 1.0) <= 1e-6
    reg.ApplyGate(G.HadamardGate(), 0)
    assert abs(reg.ExpectationValue(z0)) <= 1e-6
    reg.setToBasisState(0)
    reg.ApplyGate(G.HadamardGate(), 1)
    assert abs(reg.ExpectationValue([G.AppliedGate(G.PauliZGate().getRawOperatorMatrix(), 1)])) <= 1e-6
    reg.close()


@pytest.mark.parametrize("separate", [False, True])
def test_chsh_inequality(Q, separate):
    """BellInequalitiesTests (Tests.cpp:303-330): the CHSH value exceeds 2 and lies within 0.1 of 2 sqrt(2)
    (20000 checks per run here, 100000 in the reference)"""
    from qcsim_gb300 import measurement_basis as M
    chsh = M.CheckCHSHInequality(seed=21 + separate, choice_seed=5)
    for _ in range(20000):
        chsh.Check(separate)
    v = chsh.getValue()
    assert v > 2.0 and abs(v - 2.0 * np.sqrt(2.0)) <= 0.1, v
    chsh.close()


def test_bb84(Q):
    """QuantumCryptograpyTests (Tests.cpp:474-520): without eavesdropping the compared bits match and so do the
    keys; with an eavesdropper on every bit or on random bits the comparison fails"""
    from qcsim_gb300 import measurement_basis as M
    bb84 = M.BB84Protocol(seed=3, choice_seed=4)
    for i in range(30):
        eavesdrop = i > 9
        bb84.setEavesdropping(eavesdrop)
        bb84.setRandomEavesdropping(i > 19)
        match = bb84.Execute()
        assert bool(match) != eavesdrop, i
        if match:
            assert bb84.compareKeys() and len(bb84.getReceivedKey()) > 64
    bb84.close()


def _two_qubit_state(rng):
    v = rng.uniform(-1, 1, 4) + 1j * rng.uniform(-1, 1, 4)
    return v / np.linalg.norm(v)


def test_distributed_cnot(Q):
    """distributedCNOTTest (DistributedTests.cpp:8-100): the control on qubit 0 and target on qubit 3 end as
    after a local CNOT, next to the measured Bell-pair qubits"""
    from qcsim_gb300 import distributed as D
    rng = np.random.default_rng(8)
    dc = D.DistributedCNOT(seed=5)
    for _ in range(16):
        a = _two_qubit_state(rng)  # index bit 0 = control, bit 1 = target
        dc.Clear()
        for idx, amp in zip((0, 1, 8, 9), a):
            dc.setRawAmplitude(idx, amp)
        dc.Normalize()
        m = dc.Execute() << 1
        want = a[[0, 3, 2, 1]]  # CNOT(target <- control)
        got = [dc.getBasisStateAmplitude(s) for s in (m, m | 1, 8 | m, 8 | m | 1)]
        assert np.abs(np.array(got) - want).max() < 1e-10
    dc.close()


def test_teleported_cnot(Q):
    """teleportedCNOTTest (DistributedTests.cpp:102-190): target on qubit 0, control on qubit 5, the CNOT's
    result on qubits 2 (target) and 3 (control) next to the measured bits"""
    from qcsim_gb300 import distributed as D
    rng = np.random.default_rng(9)
    tc = D.TeleportedCNOT(seed=6)
    for _ in range(16):
        a = _two_qubit_state(rng)  # index bit 0 = target, bit 1 = control
        tc.Clear()
        for idx, amp in zip((0, 1, 0x20, 0x21), a):
            tc.setRawAmplitude(idx, amp)
        tc.Normalize()
        m = tc.Execute()
        want = a[[0, 1, 3, 2]]
        v = tc.getRegisterStorage()
        assert np.abs(np.array([v[(i << 2) | m] for i in range(4)]) - want).max() < 1e-10
    tc.close()


def _check_shor_code(make, rng, states=4):
    """ShorCodeTests (ErrorCorrectionTests.cpp:150-205): every error type on every qubit is corrected; the
    measurement of qubits 1-8 is non-zero exactly when an error was applied, and qubit 0 carries the state"""
    code = make()
    ET = type(code).ErrorType
    for _ in range(states):
        a, b = rng.uniform(-1, 1, 2) + 1j * rng.uniform(-1, 1, 2)
        n = np.sqrt(abs(a) ** 2 + abs(b) ** 2)
        a, b = a / n, b / n
        for q in range(10):
            code.SetErrorQubit(q)
            for c in range(3):
                code.SetState(a, b)
                code.setErrorType(ET.none if q == 9 else ET(c))
                res = code.Execute()
                assert (res != 0) == (q != 9), (q, c, res)
                v = code.getRegisterStorage()
                assert abs(np.conj(a) * v[res << 1] + np.conj(b) * v[(res << 1) | 1]) ** 2 >= 0.99999, (q, c)
                if q == 9:
                    break
    code.close()


def _check_qubit_adders(make_reg, make_adder, rng):
    """quantumHalfAdderTests / quantumFullAdderTests / NQubitsAdderTests (AdderTests.cpp:9-150)"""
    from qcsim_gb300 import algorithms as Al
    reg = make_reg(3)
    half = Al.TwoQubitsHalfAdder(0, 1, 2)
    for x in range(4):
        reg.setToBasisState(x)
        assert half.Execute(reg) == 0
        res = reg.MeasureAll()
        assert res & 1 == x & 1 and res >> 1 == (x & 1) + (x >> 1)
    reg = make_reg(4)
    full = Al.TwoQubitsFullAdder(0, 1, 2, 3)
    for x in range(4):
        reg.setToBasisState(x)
        assert full.Execute(reg) == 0
        res = reg.MeasureAll()
        assert res & 3 == x and res >> 2 == (x & 1) + (x >> 1)
    assert Al.TwoQubitsHalfAdder(0, 0, 2).Execute(reg) == 2 and Al.TwoQubitsFullAdder(0, 1, 2, 9).Execute(reg) == 1
    adder = make_adder()
    for _ in range(10):
        n1, n2 = (int(v) for v in rng.integers(0, 8, 2))
        adder.setToBasisState((n2 << 3) | n1)
        res = adder.Execute()
        assert res & 0x3F == (n2 << 3) | n1 and res >> 6 == n1 + n2
    adder.close()


def test_shor_code(Q):
    from qcsim_gb300 import algorithms as A
    _check_shor_code(lambda: A.ShorCode(seed=2), np.random.default_rng(13))


def test_qubit_adders(Q):
    from qcsim_gb300 import algorithms as A
    _check_qubit_adders(lambda n: Q.QubitRegister(n, seed=1), lambda: A.NQubitsAdderAlgorithm(3, seed=3),
                        np.random.default_rng(14))


def _check_paradoxes(P, hardy_step=0.1):
    """ParadoxesTests (ParadoxesTests.cpp) and CoinFlippingTests (GamesTests.cpp:9-26): the eraser's four and two
    outcomes within 5 % of their expected counts, the bomb's efficiency and Hardy's gamma within 0.08 of the
    formulas, and the coin always back on heads"""
    import math
    er = P.QuantumEraser(seed=1)
    m = er.ExecuteWithMultipleMeasurements(100000)
    assert all(abs(m.get(k, 0) - 25000) <= 1250 for k in range(4)), m
    er.setEraser()
    m = er.ExecuteWithMultipleMeasurements(100000)
    assert abs(m.get(0, 0) - 50000) <= 2500 and abs(m.get(3, 0) - 50000) <= 2500
    assert m.get(1, 0) == 0 and m.get(2, 0) == 0
    er.close()
    bomb = P.GeneralElitzurVaidmanBomb(4, seed=2)
    for stages in range(1, 5):
        bomb.setStages(stages)
        theta = 0.05 * math.pi
        while theta < 0.9 * math.pi:
            bomb.setTheta(theta)
            m = bomb.ExecuteWithMultipleMeasurements(10000)
            result = m.get(0, 0) / (10000 - m.get(1, 0))
            assert abs(result - bomb.TheoreticalEfficiency()) <= 0.08, (stages, theta)
            theta += 0.05 * math.pi
    bomb.close()
    hardy = P.HardyParadox(seed=3)
    t0 = hardy_step * math.pi
    while t0 < math.pi - hardy_step * math.pi:
        hardy.setTheta0(t0)
        t1 = hardy_step * math.pi
        while t1 < math.pi - hardy_step * math.pi:
            hardy.setTheta1(t1)
            m = hardy.ExecuteWithMultipleMeasurements(100000)
            p = [m.get(k, 0) / 100000 for k in range(4)]
            assert abs(p[0] / sum(p) - hardy.TheoreticalGamma()) <= 0.08, (t0, t1)
            t1 += hardy_step * math.pi
        t0 += hardy_step * math.pi
    hardy.close()
    coin = P.CoinFlipping(seed=4, choice_seed=5)
    assert all(coin.Execute() == 0 for _ in range(100))
    coin.close()


def test_paradoxes_and_coin_flipping(Q):
    """the reference's Hardy sweep steps both angles by 0.025 pi"""
    from qcsim_gb300 import paradoxes as P
    _check_paradoxes(P, hardy_step=0.025)


def _check_gate_oracles(O):
    """DeutschWithGatesTests (DeutschJozsaTests.cpp:8-47) and its N-qubit form, the Bernstein-Vazirani and Simon
    algorithms with gate-built oracles (SimonWithGatesTests, Tests.cpp:522-560): the same answers as with the
    oracle matrices"""
    FT = O.DeutschJozsaAlgorithmWithGatesOracle.FunctionType
    for N in (2, 3, 5, 6):
        dj = O.DeutschJozsaAlgorithmWithGatesOracle(N, seed=N, function_seed=N)
        for i in range(9):
            ft = FT.constantZero if i < 3 else FT.constantOne if i < 6 else FT.balanced
            dj.setFunction(ft)
            assert dj.WasConstantResult(dj.Execute()) == (ft != FT.balanced), (N, i)
        dj.close()
    for N in (2, 3, 5):
        bv = O.BernsteinVaziraniAlgorithmWithGatesOracle(N, seed=N)
        for s in range(1 << N):
            bv.setString(s)
            assert bv.Execute() == s, (N, s)
        bv.close()
    for N in (2, 3, 4):
        simon = O.SimonAlgorithmWithGatesOracle(N, seed=N, function_seed=N)
        for s in range(1 << N):
            simon.setString(s)
            assert simon.Execute() == s, (N, s)
        simon.close()


def test_gate_built_oracles(Q):
    from qcsim_gb300 import oracles as O
    _check_gate_oracles(O)


def test_magic_square(Q):
    """MagicSquareTests (GamesTests.cpp:28-45): the quantum strategy wins every play"""
    from qcsim_gb300 import paradoxes as P
    game = P.MagicSquare(seed=6, choice_seed=7)
    assert game.Execute() == game.getNrPlays()
    for a in (1, 2, 3):
        for b in (1, 2, 3):
            won, ra, rb = game.Play(a, b)
            assert won and bin(ra).count("1") % 2 == 0 and bin(rb).count("1") % 2 == 1
    game.close()


def _check_qmeans(make, shots):
    """QMeansClustering2DTests (QMLTests.cpp:26-120): three clusters of 15 points around (0, 0), (3, 3) and
    (1.5, 2); clustering converges, and no point measures a larger swap-test overlap with another centroid than
    with its own (within 4 standard deviations of the shot noise; the reference uses 10^6 shots and no margin)"""
    from qcsim_gb300 import qml as M
    rng = np.random.default_rng(15)
    data = [M.DataPoint(cx + rng.uniform(-1.5, 1.5), cy + rng.uniform(-1.5, 1.5))
            for cx, cy in ((0.0, 0.0), (3.0, 3.0), (1.5, 2.0)) for _ in range(15)]
    data = [data[i] for i in rng.permutation(len(data))]
    qm = make()
    qm.setData(data)
    assert qm.Cluster(3, shots)
    pts, cents = qm.getData(), qm.getCentroids()
    assert sorted((p.x, p.y) for p in pts) == sorted((p.x, p.y) for p in data)
    margin = 4 * np.sqrt(shots) / 2
    for p in pts:
        qm.SetDataPoint1(p)
        qm.SetDataPoint2(cents[p.cluster])
        own = qm.ExecuteWithMultipleMeasurements(shots).get(0, 0)
        for c, cent in enumerate(cents):
            if c != p.cluster:
                qm.SetDataPoint2(cent)
                assert qm.ExecuteWithMultipleMeasurements(shots).get(0, 0) <= own + margin
    qm.close()


def test_qmeans_clustering(Q):
    from qcsim_gb300 import qml as M
    _check_qmeans(lambda: M.QMeansClustering2D(seed=1, choice_seed=2), 100000)


def _check_pauli_simulation(S, cases=10):
    """PauliSimulationTests (SimulationTests.cpp:21-80): 3 qubits, 1-5 random Pauli-string terms with
    coefficients -U(0.1, 10), t = 1 / (2 pi) in 100 Trotter steps; fidelity >= 0.999 with exp(-i t H)|0>"""
    import math
    rng = np.random.default_rng(21)
    t = 1.0 / (2.0 * math.pi)
    for _ in range(cases):
        sim = S.PauliDecomposedHamiltonianSimulation(3, t, 100, seed=1)
        sim.setToBasisState(0)
        term = S.PauliStringSimulation()
        for _ in range(int(rng.integers(1, 6))):
            for q in range(3):
                term.setOperatorForQubit(q, int(rng.integers(0, 3)))
            sim.AddTerm(-rng.uniform(0.1, 10.0), term)
        ex = sim.getEvolutionOperator(t) @ sim.getRegisterStorage()
        sim.setToBasisState(0)
        sim.Execute()
        v = sim.getRegisterStorage()
        assert abs(np.vdot(ex, v)) ** 2 >= 0.999
        sim.close()


def test_pauli_hamiltonian_simulation(Q):
    from qcsim_gb300 import pauli_simulation as S
    _check_pauli_simulation(S)


def _check_pauli_golden(S, tol):
    """the mirror's Trotter evolution against QCSim's own PauliDecomposedHamiltonianSimulation::Execute on the
    same inputs (tests/golden/pauli.npz, made by tests/golden/make_pauli.py from the compiled reference)"""
    from pathlib import Path
    g = np.load(Path(__file__).resolve().parent / "golden" / "pauli.npz")
    for i, (n, nt) in enumerate(g["cases"]):
        sim = S.PauliDecomposedHamiltonianSimulation(int(n), float(g["times"][i]), int(g["steps"][i]), seed=1)
        sim.setRegisterStorage(g[f"psi{i}"])
        for ops, c in zip(g[f"ops{i}"], g[f"coeffs{i}"]):
            term = S.PauliStringSimulation(0.0, int(n))
            for q, op in enumerate(ops):
                term.setOperatorForQubit(q, int(op))
            sim.AddTerm(float(c), term)
        sim.Execute()
        assert np.abs(sim.getRegisterStorage() - g[f"out{i}"]).max() <= tol, i
        sim.close()


def test_pauli_simulation_matches_reference(Q):
    from qcsim_gb300 import pauli_simulation as S
    _check_pauli_golden(S, 1e-12)


def _check_oracles_golden(O, make_reg, tol):
    """the mirror's gate-built oracles against QCSim's own OracleWithGates / OracleWithGatesSimpleFunction
    Execute on the same states and function tables (tests/golden/oracles.npz, made by tests/golden/make_oracles.py
    from the compiled reference)"""
    from pathlib import Path
    g = np.load(Path(__file__).resolve().parent / "golden" / "oracles.npz")
    for i, (n, start, end, target, anc, simple) in enumerate(g["cases"].tolist()):
        values = g[f"table{i}"].tolist()
        cls = O.OracleWithGatesSimpleFunction if simple else O.OracleWithGates
        oracle = cls(n, start, end, target, anc)
        oracle.setFunction(lambda x, v=values: v[x])
        reg = make_reg(n)
        reg.setRegisterStorage(g[f"psi{i}"])
        oracle.Execute(reg)
        assert np.abs(reg.getRegisterStorage() - g[f"out{i}"]).max() <= tol, i
        reg.close()


def test_gate_built_oracles_match_reference(Q):
    from qcsim_gb300 import oracles as O
    _check_oracles_golden(O, lambda n: Q.QubitRegister(n, seed=1), 1e-12)


def _check_algorithms_golden(A, make_reg, tol):
    """the mirrors' pre-measurement states against QCSim's own Grover search, Draper adders, phase estimation,
    VQE ansatz, Shor's period finding and quantum counting
    (tests/golden/algorithms.npz, made by tests/golden/make_algorithms.py from the compiled reference)"""
    from pathlib import Path
    g = np.load(Path(__file__).resolve().parent / "golden" / "algorithms.npz")
    for i, (n, marked) in enumerate(g["grover"].tolist()):
        gr = A.GroverAlgorithm(n, seed=1)
        gr.setCorrectQuestionState(marked)
        gr.ExecuteWithoutMeasurement()
        assert np.abs(gr.getRegisterStorage() - g[f"grover{i}"]).max() <= tol, ("grover", i)
        gr.close()
    for i, (N, carry) in enumerate(g["draper"].tolist()):
        ad = (A.DraperAdderWithCarry if carry else A.DraperAdder)(N, seed=1)
        ad.setRegisterStorage(g[f"draper_in{i}"])
        ad.ExecuteWithoutMeasurement()
        assert np.abs(ad.getRegisterStorage() - g[f"draper{i}"]).max() <= tol, ("draper", i)
        ad.close()
    for i, (k, N, L) in enumerate(g["phase"].tolist()):
        pe = A.PhaseEstimation(g[f"phase_u{i}"], N, L)
        reg = make_reg(N)
        reg.setRegisterStorage(g[f"phase_in{i}"])
        pe.ExecuteWithoutMeasurement(reg)
        assert np.abs(reg.getRegisterStorage() - g[f"phase{i}"]).max() <= tol, ("phase", i)
        reg.close()
    from qcsim_gb300 import vqe as V
    for i, (n, npar) in enumerate(g["vqe"].tolist()):
        term = V.PauliStringVQE(n)
        for q, op in enumerate(g[f"vqe_ops{i}"].tolist()):
            term.setOperatorForQubit(q, int(op))
        reg = make_reg(n)
        reg.setToBasisState(0)
        term.Ansatz(reg, g[f"vqe_params{i}"].tolist())
        term.Execute(reg)
        assert np.abs(reg.getRegisterStorage() - g[f"vqe{i}"]).max() <= tol, ("vqe", i)
        reg.close()
    for i, (c, a, n, L) in enumerate(g["shor"].tolist()):
        fx = A.Fx(L, n - L, c)
        fx.setParam(a)
        reg = make_reg(n)
        A.ShorPhaseEstimation(fx, n, L).ExecuteWithoutMeasurement(reg)
        assert np.abs(reg.getRegisterStorage() - g[f"shor{i}"]).max() <= tol, ("shor", i)
        reg.close()
    from qcsim_gb300 import counting as CT
    for i, (P, Gq) in enumerate(g["counting"].tolist()):
        qc = CT.QuantumCountingAlgorithm(P, Gq, seed=1)
        qc.SetMarkedStates(g[f"counting_marked{i}"].tolist())
        qc.ExecuteWithoutMeasurement()
        assert np.abs(qc.getRegisterStorage() - g[f"counting{i}"]).max() <= tol, ("counting", i)
        qc.close()


def test_algorithms_match_reference(Q):
    from qcsim_gb300 import algorithms as A
    _check_algorithms_golden(A, lambda n: Q.QubitRegister(n, seed=1), 1e-12)
