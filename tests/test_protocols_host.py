"""The small-protocol mirrors run end to end on the CPU, no GPU: each algorithm's register is replaced by a
stand-in over the oracle (tests/oracle_register.py), so the host logic (gate order, mid-circuit measurement
handling, classical corrections, bookkeeping) is checked against QCSim's own test conditions.  The same
checks run over the engine in test_gpu_protocols.py."""
import numpy as np
import pytest

from oracle_register import OracleBackedRegister
from qcsim_gb300 import algorithms as A


@pytest.fixture
def on_oracle(monkeypatch):
    monkeypatch.setattr(A, "QubitRegister", OracleBackedRegister)


def test_deutsch_jozsa_and_simon(on_oracle):
    FT = A.DeutschJozsaAlgorithm.FunctionType
    for N in (2, 4):
        dj = A.DeutschJozsaAlgorithm(N, seed=N, function_seed=N)
        for ft in (FT.constantZero, FT.constantOne, FT.balanced, FT.balanced):
            dj.setFunction(ft)
            assert dj.WasConstantResult(dj.Execute()) == (ft != FT.balanced)
    simon = A.SimonAlgorithm(3, seed=1, function_seed=3)
    for s in (0, 3, 5):
        simon.setString(s)
        assert simon.Execute() == s


def test_teleportation_family(on_oracle):
    from qcsim_gb300 import teleportation as T
    rng = np.random.default_rng(2)
    qt = T.QuantumTeleportationRealization(seed=1)
    for explicit in (False, True):
        for _ in range(4):
            a, b = rng.standard_normal(2) + 1j * rng.standard_normal(2)
            n = np.sqrt(abs(a) ** 2 + abs(b) ** 2)
            qt.SetState(a / n, b / n)
            bits = qt.Teleport(explicit)
            assert abs(qt.getBasisStateAmplitude(bits) - a / n) < 1e-12
            assert abs(qt.getBasisStateAmplitude(4 | bits) - b / n) < 1e-12
    reg = OracleBackedRegister(3, seed=4)
    tp = T.Teleport()
    for v in (0, 1, 1, 0):
        reg.setToBasisState(v)
        tp.Execute(reg)
        assert reg.MeasureQubit(2) == v
    es = T.EntanglementSwapping(seed=3)
    ref = OracleBackedRegister(2, seed=0)
    for i in range(4):
        T.BellState().setBellState(ref, 0, 1, bool(i & 1), bool(i & 2))
        es.SetBellStateToBeSent(bool(i & 1), bool(i & 2))
        meas = es.Teleport(bool(i & 1))
        v, want = es.getRegisterStorage(), ref.getRegisterStorage()
        assert all(abs(v[s] - (want[s >> 4] if (s & 15) == meas else 0)) < 1e-12 for s in range(64))
    coding = T.SuperdenseCoding(seed=5)
    for b1 in (False, True):
        for b2 in (False, True):
            coding.SetBits(b1, b2)
            got = coding.Execute()
            assert (bool(got & 1), bool(got & 2)) == (b1, b2)


def test_distributed_cnots(on_oracle):
    from qcsim_gb300 import distributed as D
    rng = np.random.default_rng(7)
    dc, tc = D.DistributedCNOT(seed=1), D.TeleportedCNOT(seed=2)
    for _ in range(6):
        a = rng.standard_normal(4) + 1j * rng.standard_normal(4)
        a /= np.linalg.norm(a)
        dc.Clear()
        for idx, amp in zip((0, 1, 8, 9), a):
            dc.setRawAmplitude(idx, amp)
        dc.Normalize()
        m = dc.Execute() << 1
        got = [dc.getBasisStateAmplitude(s) for s in (m, m | 1, 8 | m, 8 | m | 1)]
        assert np.abs(np.array(got) - a[[0, 3, 2, 1]]).max() < 1e-12
        tc.Clear()
        for idx, amp in zip((0, 1, 0x20, 0x21), a):
            tc.setRawAmplitude(idx, amp)
        tc.Normalize()
        m = tc.Execute()
        v = tc.getRegisterStorage()
        assert np.abs(np.array([v[(i << 2) | m] for i in range(4)]) - a[[0, 1, 3, 2]]).max() < 1e-12


def test_chsh_and_bb84(on_oracle):
    from qcsim_gb300 import measurement_basis as M
    chsh = M.CheckCHSHInequality(seed=3, choice_seed=4)
    for separate in (False, True):
        chsh.ResetStatistics()
        for _ in range(4000):
            chsh.Check(separate)
        v = chsh.getValue()
        assert v > 2.0 and abs(v - 2 * np.sqrt(2)) < 0.2, v
    bb84 = M.BB84Protocol(seed=5, nrBits=256, choice_seed=6)
    for eavesdrop, rand in ((False, False), (True, False), (True, True)):
        bb84.setEavesdropping(eavesdrop)
        bb84.setRandomEavesdropping(rand)
        match = bb84.Execute()
        assert bool(match) != eavesdrop
        if match:
            assert bb84.compareKeys() and bb84.getReceivedKey() == bb84.getSentKey()


def test_quantum_counting_execute(on_oracle):
    """Execute end to end (circuit, inverse QFT on the precision qubits through the QFT mirror, measurement)"""
    from qcsim_gb300 import counting as C
    qc = C.QuantumCountingAlgorithm(5, 2, seed=1)
    for marked in ([], [1], [0, 3], [0, 1, 2, 3]):
        qc.SetMarkedStates(marked)
        res = qc.ExecuteWithMultipleMeasurements(2000)
        state = max(res.items(), key=lambda kv: kv[1])[0]
        assert qc.GetCountForState(state) == len(marked)


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
    reg = make_reg(3)
    half = A.TwoQubitsHalfAdder(0, 1, 2)
    for x in range(4):
        reg.setToBasisState(x)
        assert half.Execute(reg) == 0
        res = reg.MeasureAll()
        assert res & 1 == x & 1 and res >> 1 == (x & 1) + (x >> 1)
    reg = make_reg(4)
    full = A.TwoQubitsFullAdder(0, 1, 2, 3)
    for x in range(4):
        reg.setToBasisState(x)
        assert full.Execute(reg) == 0
        res = reg.MeasureAll()
        assert res & 3 == x and res >> 2 == (x & 1) + (x >> 1)
    assert A.TwoQubitsHalfAdder(0, 0, 2).Execute(reg) == 2 and A.TwoQubitsFullAdder(0, 1, 2, 9).Execute(reg) == 1
    adder = make_adder()
    for _ in range(10):
        n1, n2 = (int(v) for v in rng.integers(0, 8, 2))
        adder.setToBasisState((n2 << 3) | n1)
        res = adder.Execute()
        assert res & 0x3F == (n2 << 3) | n1 and res >> 6 == n1 + n2
    adder.close()


def test_shor_code_and_adders(on_oracle):
    rng = np.random.default_rng(12)
    _check_shor_code(lambda: A.ShorCode(seed=2), rng, states=2)
    _check_qubit_adders(lambda n: OracleBackedRegister(n, seed=1), lambda: A.NQubitsAdderAlgorithm(3, seed=3), rng)


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


def test_paradoxes_and_coin_flipping(on_oracle):
    from qcsim_gb300 import paradoxes as P
    _check_paradoxes(P, hardy_step=0.1)


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


def test_gate_built_oracles(on_oracle):
    from qcsim_gb300 import oracles as O
    _check_gate_oracles(O)


def test_n_controlled_gates_with_ancilla():
    """NControlledGateWithAncilla.h:23-75: with 1 to 7 controls, two NOTs added as controlled gates flip their
    targets exactly when every control is set, and the ancillas return to 0"""
    from qcsim_gb300 import counting as C
    from qcsim_gb300 import gates as G
    from qcsim_gb300 import oracles as O
    x = G.PauliXGate().getRawOperatorMatrix()
    for nc in range(1, 8):
        g = O.NControlledGatesWithAncilla()
        g.SetControlQubits(range(nc))
        g.SetStartAncillaQubits(nc + 2)
        assert g.AddGate(G.AppliedGate(x, nc)) and g.AddGate(G.AppliedGate(x, nc + 1))
        seq = C.GateSequence()
        g.Execute(seq)
        for c in range(1 << nc):
            bits = c
            for gate, t, c1, c2 in seq.ops:
                k = gate.getQubitsNumber()
                if (k == 3 and (bits >> c1) & (bits >> c2) & 1) or (k == 2 and (bits >> c1) & 1):
                    bits ^= 1 << t
            assert bits >> (nc + 2) == 0, (nc, c)
            full = c == (1 << nc) - 1
            assert (bits >> nc) & 3 == (3 if full else 0), (nc, c)


def test_magic_square(on_oracle):
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


def test_qmeans_clustering(on_oracle):
    from qcsim_gb300 import qml as M
    _check_qmeans(lambda: M.QMeansClustering2D(seed=1, choice_seed=2), 4000)


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


def test_pauli_hamiltonian_simulation(on_oracle):
    from qcsim_gb300 import pauli_simulation as S
    _check_pauli_simulation(S, cases=4)


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


def test_pauli_simulation_matches_reference(on_oracle):
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


def test_gate_built_oracles_match_reference():
    from qcsim_gb300 import oracles as O
    _check_oracles_golden(O, lambda n: OracleBackedRegister(n, seed=1), 1e-12)


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


def test_algorithms_match_reference(on_oracle):
    _check_algorithms_golden(A, lambda n: OracleBackedRegister(n, seed=1), 1e-12)
