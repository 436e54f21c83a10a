"""Parity of the GPU engine (libqcs_gpu.so through the C ABI) with the CPU oracle and with QCSim's own
outputs (tests/golden).  FP64 tolerance: 1e-12 max amplitude error; measurement outcomes identical
under the same random stream.  FP32 registers: 2e-6 max amplitude error per gate sequence here."""
import itertools

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12


@pytest.fixture(scope="module")
def Q():
    import qcsim_gb300
    from qcsim_gb300 import _lib
    try:
        _lib.load()
    except _lib.EngineUnavailable as e:
        pytest.fail(f"engine not built: {e}")
    return qcsim_gb300


def oracle_state(n, ops, init=None):
    from oracle import bind as B
    reg = B.OracleRegister(n)
    if init is not None:
        reg.set_state(init)
    reg.apply(ops)
    return reg.state()


def rand_state(n, seed):
    r = np.random.default_rng(seed)
    v = r.standard_normal(1 << n) + 1j * r.standard_normal(1 << n)
    return v / np.linalg.norm(v)


def test_every_gate_every_placement(Q):
    """each gate class on every ordered qubit placement of a 5-qubit register"""
    from qcsim_gb300 import gates as G
    n = 5
    init = rand_state(n, 1)
    reg = Q.QubitRegister(n, seed=1)
    worst = 0.0
    for code in sorted(G.BY_CODE):
        g = G.make(code, 0.9, -0.4, 1.3, 0.2)
        k = g.getQubitsNumber()
        for qs in itertools.permutations(range(n), k):
            qs = list(qs) + [0] * (3 - k)
            reg.setRegisterStorageFastNoNormalize(init)
            reg.ApplyGate(g, *qs)
            got = reg.getRegisterStorage()
            want = oracle_state(n, [(g, *qs)], init)
            worst = max(worst, np.abs(got - want).max())
            assert np.abs(got - want).max() <= TOL, (code, qs)
    assert worst <= TOL


def test_matrix_only_gates(Q):
    """AppliedGate (no traits) takes the dense 2x2 / 4x4 / 8x8 paths"""
    from qcsim_gb300 import gates as G
    n = 6
    r = np.random.default_rng(3)
    init = rand_state(n, 2)
    reg = Q.QubitRegister(n, seed=1)
    for k in (1, 2, 3):
        for qs in list(itertools.permutations(range(n), k))[::3]:
            a = r.standard_normal((1 << k, 1 << k)) + 1j * r.standard_normal((1 << k, 1 << k))
            u, _ = np.linalg.qr(a)
            qs = list(qs) + [0] * (3 - k)
            g = G.AppliedGate(u, *qs)
            reg.setRegisterStorageFastNoNormalize(init)
            reg.ApplyGate(g)
            assert np.abs(reg.getRegisterStorage() - oracle_state(n, [(g, *qs)], init)).max() <= TOL


def test_golden_random_circuits(Q, golden):
    from test_oracle_golden import split_recs
    from qcsim_gb300 import _lib as L, gates as G
    import ctypes as C
    from oracle import bind as B
    off = 0
    for n, recs in split_recs(golden):
        ref = golden["circ_states"][off:off + (1 << n)]
        off += 1 << n
        # rebuild the gate objects from codes/params (the engine gets matrices + traits)
        ops = []
        for r in recs:
            code = int(r["code"])
            if code >= 50:
                k = code - 49
                d = 1 << k
                m = r["m"][: 2 * d * d].view(np.complex128).reshape(d, d)
                g = G.AppliedGate(m, int(r["q0"]), int(r["q1"]), int(r["q2"]))
            else:
                g = G.make(code, *r["p"])
            ops.append((g, int(r["q0"]), int(r["q1"]), int(r["q2"])))
        reg = Q.QubitRegister(n, seed=1)
        for op in ops:
            reg.ApplyGate(*op)
        assert np.abs(reg.getRegisterStorage() - ref).max() <= TOL
        reg2 = Q.QubitRegister(n, seed=1)
        reg2.ApplyGates(ops)
        assert np.abs(reg2.getRegisterStorage() - ref).max() <= TOL
    _ = (L, C, B)


def test_layered_12_golden(Q, golden):
    from qcsim_gb300 import circuits
    ops = circuits.layered_circuit(12, 10, seed=4, p3=0.05)
    reg = Q.QubitRegister(12, seed=7)
    reg.ApplyGates(ops)
    assert np.abs(reg.getRegisterStorage() - golden["l12_state"]).max() <= TOL
    qp = np.array([reg.GetQubitProbability(q) for q in range(12)])
    assert np.abs(qp - golden["l12_qprob"]).max() <= TOL
    hist = reg.RepeatedMeasure(1024)
    assert np.array_equal(np.array(sorted(hist.items()), dtype=np.uint64), golden["l12_hist"])
    assert reg.MeasureAll() == golden["l12_measure_all"][0]
    st = reg.getRegisterStorage()
    assert st[int(golden["l12_measure_all"][0])] == 1 and np.count_nonzero(st) == 1


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_layered_20_parity(Q, golden, seed):
    """the 20-qubit layered workload (depth 40): full state vs the oracle, probe amplitudes, qubit
    probabilities and 1024 seeded shots vs the reference"""
    from qcsim_gb300 import circuits
    ops = circuits.layered_circuit(20, 40, seed=seed)
    reg = Q.QubitRegister(20, seed=seed)
    reg.ApplyGates(ops)
    st = reg.getRegisterStorage()
    assert np.abs(st - oracle_state(20, ops)).max() <= TOL
    assert np.abs(st[golden["c0_probe_idx"]] - golden["c0_amp"][seed - 1]).max() <= TOL
    qp = np.array([reg.GetQubitProbability(q) for q in range(20)])
    assert np.abs(qp - golden["c0_qprob"][seed - 1]).max() <= 1e-12
    off = int(np.sum(golden["c0_hist_len"][: seed - 1]))
    want = golden["c0_hist"][off:off + golden["c0_hist_len"][seed - 1]]
    got = np.array(sorted(reg.RepeatedMeasure(1024).items()), dtype=np.uint64)
    assert np.array_equal(got, want)


def test_measurement_kats(Q, golden):
    for (s, op, v), after in zip(golden["kat_rows"], golden["kat_after"]):
        reg = Q.QubitRegister(2, seed=1000 + int(s))
        reg.setToBasisState(0)
        reg.setRawAmplitude(0, 0.5)
        reg.setRawAmplitude(1, -0.5j)
        reg.setRawAmplitude(3, 1 / np.sqrt(2))
        reg.Normalize()
        got = [lambda: reg.MeasureQubit(0), lambda: reg.MeasureQubit(1), lambda: reg.Measure(0, 1),
               reg.MeasureAll, reg.MeasureNoCollapse][int(op)]()
        assert got == v
        assert np.abs(reg.getRegisterStorage() - after).max() <= 1e-15


def test_subregister_measurements(Q, golden):
    for (a, b, v), after in zip(golden["sub_rows"], golden["sub_after"]):
        a, b = int(a), int(b)
        reg = Q.QubitRegister(10, seed=31 + a * 10 + b)
        reg.setRegisterStorageFastNoNormalize(golden["sub_state"])
        assert reg.Measure(a, b) == v
        assert np.abs(reg.getRegisterStorage() - after).max() <= 1e-14
    for a, b in ((0, 0), (3, 5), (2, 9), (9, 9), (0, 9)):
        rows = golden["sub_hist"][(golden["sub_hist"][:, 0] == a) & (golden["sub_hist"][:, 1] == b)]
        reg = Q.QubitRegister(10, seed=77 + a * 10 + b)
        reg.setRegisterStorageFastNoNormalize(golden["sub_state"])
        h = reg.RepeatedMeasure(a, b, 500)
        assert np.array_equal(np.array(sorted(h.items()), dtype=np.uint64), rows[:, 2:])


def test_scan_edges(Q, golden):
    for row in golden["edge_rows"]:
        s = int(row[0])
        reg = Q.QubitRegister(10, seed=500 + s)
        reg.setRegisterStorageFastNoNormalize(golden["edge_state"])
        assert reg.MeasureNoCollapse() == row[2]
        h = reg.RepeatedMeasure(64)
        assert np.array_equal(np.array([k for k in sorted(h) for _ in range(h[k])], dtype=np.uint64), row[3:])
        reg.setRegisterStorageFastNoNormalize(golden["edge_state"])
        assert reg.MeasureAll() == row[1]


def test_qft(Q, golden):
    from qcsim_gb300 import subalgo
    for cfg, inp, outp in zip(golden["qft_cfg"], golden["qft_in"], golden["qft_out"]):
        n, s0, e0, inv, sw = (int(x) for x in cfg)
        reg = Q.QubitRegister(n, seed=1)
        reg.setRegisterStorageFastNoNormalize(inp[: 1 << n])
        qft = subalgo.QuantumFourierTransform(n, s0, e0)
        (qft.IQFT if inv else qft.QFT)(reg, bool(sw))
        assert np.abs(reg.getRegisterStorage() - outp[: 1 << n]).max() <= TOL


@pytest.mark.parametrize("n", [12, 18])
def test_qft_random_state(Q, n):
    from qcsim_gb300 import circuits, subalgo
    v = circuits.random_normal_state(n, 5)
    reg = Q.QubitRegister(n, seed=1)
    reg.setRegisterStorageFastNoNormalize(v)
    subalgo.QuantumFourierTransform(n).QFT(reg)
    want = oracle_state(n, circuits.qft_circuit(0, n - 1), v)
    assert np.abs(reg.getRegisterStorage() - want).max() <= TOL
    # QFT then IQFT returns the input
    subalgo.QuantumFourierTransform(n).IQFT(reg)
    assert np.abs(reg.getRegisterStorage() - v).max() <= 1e-11


def test_qaoa(Q, golden):
    from qcsim_gb300 import circuits
    insts = circuits.qaoa_instances(4, seed=8, nmin=6, nmax=10, p=2)
    for inst, st, en in zip(insts, golden["qaoa_states"], golden["qaoa_energy"]):
        n = inst["n"]
        reg = Q.QubitRegister(n, seed=1)
        reg.ApplyGates(circuits.qaoa_circuit(inst))
        got = reg.getRegisterStorage()
        assert np.abs(got - st[: 1 << n]).max() <= TOL
        e_exact = float(np.dot(reg.probabilities(), en[: 1 << n]))
        assert abs(e_exact - float(np.dot(np.abs(st[: 1 << n]) ** 2, en[: 1 << n]))) <= 1e-12


def test_expectation_and_replay(Q, golden):
    from qcsim_gb300 import gates as G
    from test_gpu_parity import _ops_from_recs
    ops = _ops_from_recs(golden["exp_recs"])
    pre = _ops_from_recs(golden["exp_pre"])
    reg = Q.QubitRegister(6, seed=1)
    reg.ApplyGates(ops)
    v = reg.ExpectationValue([g for (g, *_) in pre])
    assert abs(v - complex(*golden["exp_value"])) <= 1e-13
    assert np.abs(reg.getRegisterStorage() - golden["exp_state_after"]).max() <= TOL
    assert reg.ExpectationValue([]) == 1.0
    for mode, want in ((1, golden["replay_states"][0]), (2, golden["replay_states"][1])):
        r2 = Q.QubitRegister(6, seed=1)
        r2.ComputeStart()
        for op in ops:
            r2.ApplyGate(*op)
        r2.ComputeEnd()
        (r2.Compute if mode == 1 else r2.Uncompute)()
        assert np.abs(r2.getRegisterStorage() - want).max() <= TOL
    _ = G


def _ops_from_recs(recs):
    from qcsim_gb300 import gates as G
    ops = []
    for r in recs:
        code = int(r["code"])
        if code >= 50:
            d = 1 << (code - 49)
            g = G.AppliedGate(r["m"][: 2 * d * d].view(np.complex128).reshape(d, d), int(r["q0"]), int(r["q1"]), int(r["q2"]))
        else:
            g = G.make(code, *r["p"])
        ops.append((g, int(r["q0"]), int(r["q1"]), int(r["q2"])))
    return ops


def test_invalid_arguments(Q):
    from qcsim_gb300 import gates as G
    reg = Q.QubitRegister(3, seed=1)
    for args, msg in (((G.HadamardGate(), 3), "Qubit number is too high"),
                      ((G.CNOTGate(), 1, 1), "Qubit and controlling qubit are the same"),
                      ((G.CNOTGate(), 1, 5), "Controlling qubit number is too high"),
                      ((G.ToffoliGate(), 0, 1, 1), "Qubits must be different"),
                      ((G.ToffoliGate(), 0, 1, 7), "Controlling qubit number is too high")):
        with pytest.raises(ValueError, match=msg):
            reg.ApplyGate(*args)


def test_state_api(Q):
    n = 8
    reg = Q.QubitRegister(n, seed=3)
    assert reg.getBasisStateAmplitude(0) == 1
    reg.setToQubitState(3)
    assert reg.getBasisStateProbability(8) == 1
    reg.setToQubitState(99)  # out of range: no-op
    assert reg.getBasisStateProbability(8) == 1
    reg.setToCatState()
    st = reg.getRegisterStorage()
    assert st[0] == st[-1] == 1 / np.sqrt(2)
    reg.setToEqualSuperposition()
    assert np.allclose(reg.getRegisterStorage(), 1 / 16)
    assert reg.getBasisStateAmplitude(1 << n) == 0
    v = rand_state(n, 9) * 3.0
    reg.setRegisterStorage(v)
    assert abs(np.linalg.norm(reg.getRegisterStorage()) - 1) < 1e-14
    reg.setRegisterStorageFastNoNormalize(v)
    reg.AdjustPhaseAndNormalize()
    want = v / v[0]
    want /= np.linalg.norm(want)
    assert np.abs(reg.getRegisterStorage() - want).max() < 1e-14
    assert abs(reg.stateFidelity(want) - 1) < 1e-13
    reg.SaveState()
    reg.ApplyGate(Q.gates.HadamardGate(), 2)
    c = reg.Clone()
    reg.RestoreState()
    assert np.abs(reg.getRegisterStorage() - want).max() < 1e-14
    c.RestoreStateDestructive()
    assert np.abs(c.getRegisterStorage() - want).max() < 1e-14
    m = np.linalg.qr(np.random.default_rng(1).standard_normal((256, 256)))[0].astype(np.complex128)
    reg.ApplyOperatorMatrix(m)
    assert np.abs(reg.getRegisterStorage() - m @ want).max() < 1e-13
    reg.Clear()
    assert not reg.getRegisterStorage().any()


def test_fp32_register(Q):
    from qcsim_gb300 import circuits
    n = 14
    ops = circuits.layered_circuit(n, 8, seed=2, p3=0.05)
    reg = Q.QubitRegister(n, seed=1, precision="fp32")
    reg.ApplyGates(ops)
    want = oracle_state(n, ops)
    got = reg.getRegisterStorage()
    assert np.abs(got - want).max() < 2e-6
    # fidelity of the renormalised FP32 state (the FP32 path renormalises in FP64)
    got = got / np.linalg.norm(got)
    assert 1 - abs(np.vdot(want, got)) ** 2 < 1e-9


@pytest.mark.parametrize("n,precision", [(14, "fp64"), (16, "fp64"), (15, "fp32"), (17, "fp32")])
def test_passes_match_per_gate(Q, n, precision):
    """gate lists run as shared-memory passes give the per-gate results (every gate class, random
    placements, matrix-only gates, long runs of diagonal gates on non-tile qubits)"""
    from qcsim_gb300 import circuits, gates as G
    r = np.random.default_rng(n)
    codes = sorted(G.BY_CODE)
    ops = []
    for _ in range(300):
        g = G.make(int(r.choice(codes)), *r.uniform(0, 2 * np.pi, 4))
        qs = [int(x) for x in r.choice(n, size=3, replace=False)]
        ops.append((g, *qs))
    for k in (1, 2, 3):
        a = r.standard_normal((1 << k, 1 << k)) + 1j * r.standard_normal((1 << k, 1 << k))
        u, _ = np.linalg.qr(a)
        qs = [int(x) for x in r.choice(n, size=3, replace=False)]
        ops.append((G.AppliedGate(u, *qs), *qs))
    ops += circuits.qft_circuit(0, n - 1)
    init = rand_state(n, 4)
    a = Q.QubitRegister(n, seed=1, precision=precision)
    a.setRegisterStorageFastNoNormalize(init)
    a.ApplyGates(ops)
    b = Q.QubitRegister(n, seed=1, precision=precision)
    b.set_passes(False)
    b.setRegisterStorageFastNoNormalize(init)
    b.ApplyGates(ops)
    sa, sb = a.getRegisterStorage(), b.getRegisterStorage()
    want = oracle_state(n, ops, init)
    tol = TOL if precision == "fp64" else 5e-5
    assert np.abs(sa - want).max() <= tol
    assert np.abs(sb - want).max() <= tol
    assert np.abs(sa - sb).max() <= (1e-14 if precision == "fp64" else 1e-6)


def test_qft_passes(Q):
    from qcsim_gb300 import circuits, subalgo
    n = 20
    v = circuits.random_normal_state(n, 11)
    reg = Q.QubitRegister(n, seed=1)
    reg.setRegisterStorageFastNoNormalize(v)
    subalgo.QuantumFourierTransform(n).QFT(reg)
    got = reg.getRegisterStorage()
    # QFT|v> is the unitary DFT with e^{+2 pi i jk / N}: N * ifft(v) / sqrt(N) (the bit-reversing swaps included)
    want = np.fft.ifft(v) * np.sqrt(v.size)
    assert np.abs(got - want).max() <= TOL
    assert np.abs(got - oracle_state(n, circuits.qft_circuit(0, n - 1), v)).max() <= TOL


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("start,end", [(0, 17), (2, 15), (1, 17), (0, 8), (9, 17)])
def test_qft_phase_rows(Q, start, end, precision):
    """QFT / IQFT on a sub-register of an 18-qubit register (shared-memory passes, each target's run of
    controlled phases applied as one row; FP32 registers too, whose gate lists are otherwise fused)
    against the oracle's gate-by-gate sequence"""
    from qcsim_gb300 import circuits, subalgo
    n = 18
    tol = TOL if precision == "fp64" else 2e-6
    v = circuits.random_normal_state(n, 21 + start + end)
    for inverse in (False, True):
        for do_swap in (False, True):
            reg = Q.QubitRegister(n, seed=1, precision=precision)
            reg.setRegisterStorageFastNoNormalize(v)
            qft = subalgo.QuantumFourierTransform(n, start, end)
            (qft.IQFT if inverse else qft.QFT)(reg, do_swap)
            want = oracle_state(n, circuits.qft_circuit(start, end, inverse=inverse, do_swap=do_swap), v)
            assert np.abs(reg.getRegisterStorage() - want).max() <= tol, (inverse, do_swap)


@pytest.mark.parametrize("n,max_q", [(10, 5), (16, 5), (18, 3), (20, 4)])
def test_fused_fp32(Q, n, max_q):
    """the FP32 fused path (blocks of <= max_q qubits, one dense matrix each) against the FP64 oracle:
    fidelity of the renormalised state within 1e-9, max amplitude error within 2e-6"""
    from qcsim_gb300 import circuits
    ops = circuits.layered_circuit(n, 10, seed=n, p3=0.05)
    reg = Q.QubitRegister(n, seed=1, precision="fp32")
    reg.set_fusion(1, max_q)
    reg.ApplyGates(ops)
    got = reg.getRegisterStorage()
    want = oracle_state(n, ops)
    assert np.abs(got - want).max() < 2e-6
    got = got / np.linalg.norm(got)
    assert 1 - abs(np.vdot(want, got)) ** 2 < 1e-9


@pytest.mark.parametrize("n,max_q,controlled", [(14, 5, 0.0), (16, 4, 0.1), (18, 5, 0.1), (20, 5, 0.0)])
def test_fused_fp32_tensor_cores(Q, n, max_q, controlled):
    """4- and 5-qubit fused blocks as 3xTF32 tensor-core products (tcgen05) against the FP64 oracle and
    against the same blocks as FP32 FMAs on the CUDA cores: fidelity of the renormalised state within
    1e-9, max amplitude error within 2e-6"""
    from qcsim_gb300 import circuits
    ops = circuits.layered_circuit(n, 8, seed=100 + n, p3=0.05, controlled_frac=controlled)
    init = circuits.random_normal_state(n, n)
    want = oracle_state(n, ops, init)
    states = {}
    for tc in (True, False):
        reg = Q.QubitRegister(n, seed=1, precision="fp32")
        reg.set_fusion(1, max_q)
        reg.set_tensor_cores(tc)
        reg.setRegisterStorageFastNoNormalize(init)
        reg.profile(True)
        reg.ApplyGates(ops)
        prof = reg.read_profile()
        assert ("tile_pass_tc" in prof) == tc, prof
        got = reg.getRegisterStorage()
        assert np.abs(got - want).max() < 2e-6, tc
        got = got / np.linalg.norm(got)
        assert 1 - abs(np.vdot(want, got)) ** 2 < 1e-9, tc
        states[tc] = got
    assert np.abs(states[True] - states[False]).max() < 2e-6


def test_fused_fp64(Q):
    """fusion on an FP64 register (blocks of <= 4 qubits) stays within the FP64 tolerance"""
    from qcsim_gb300 import circuits, gates as G
    n = 17
    r = np.random.default_rng(2)
    ops = circuits.layered_circuit(n, 6, seed=5, p3=0.1, controlled_frac=0.1)
    for code in sorted(G.BY_CODE):
        g = G.make(code, *r.uniform(0, 2 * np.pi, 4))
        ops.append((g, *[int(x) for x in r.choice(n, size=3, replace=False)]))
    reg = Q.QubitRegister(n, seed=1)
    reg.set_fusion(1, 4)
    reg.ApplyGates(ops)
    assert np.abs(reg.getRegisterStorage() - oracle_state(n, ops)).max() <= 1e-12


@pytest.mark.parametrize("n,precision,depth", [(30, "fp64", 3), (33, "fp32", 2)])
def test_full_size_round_trips(Q, n, precision, depth):
    """the configurations' full sizes (30 qubits FP64 = 16 GiB; 33 qubits FP32 = 64 GiB, fused path with
    tensor-core blocks) through size-independent properties: QFT|0> is the uniform state, a layered
    circuit followed by its inverse and the inverse QFT return |0>"""
    from qcsim_gb300 import circuits, subalgo
    tol = 1e-10 if precision == "fp64" else 2e-4
    reg = Q.QubitRegister(n, seed=1, precision=precision)
    qft = subalgo.QuantumFourierTransform(n)
    qft.QFT(reg)
    u = 2.0 ** (-n / 2)
    for idx in (0, 1, (1 << n) - 1, 0x2AAAAAAA & ((1 << n) - 1)):
        assert abs(reg.getBasisStateAmplitude(idx) - u) < tol * u * 50
    for q in (0, n // 2, n - 1):
        assert abs(reg.GetQubitProbability(q) - 0.5) < tol
    ops = circuits.layered_circuit(n, depth, seed=77, p3=0.05)
    reg.ApplyGates(ops)
    inv = [(type(g)(*(-x for x in g.params()[:1])) if hasattr(g, "theta") else g, *q) for (g, *q) in reversed(ops)]
    reg.ApplyGates(inv)
    qft.IQFT(reg)
    assert abs(reg.getBasisStateAmplitude(0) - 1) < tol
    reg.close()


def test_larger_register_properties(Q):
    """24 qubits: unitary circuits keep the norm; an inverse circuit returns the start state"""
    from qcsim_gb300 import circuits
    n = 24
    ops = circuits.layered_circuit(n, 6, seed=9, p3=0.05)
    reg = Q.QubitRegister(n, seed=1)
    reg.ApplyGates(ops)
    p = reg.probabilities()
    assert abs(p.sum() - 1) < 1e-12
    inv =[(type(g)(*(-x for x in g.params()[:1])) if hasattr(g, "theta") else g, *q) for (g, *q) in reversed(ops)]
    reg.ApplyGates(inv)
    assert abs(reg.getBasisStateAmplitude(0) - 1) < 1e-11


@pytest.mark.parametrize("other_precision", ["fp64", "fp32"])
def test_compare_applies_pending_factors(Q, other_precision):
    """qcs_compare against amplitudes read back on the host: one register carries a pending global
    factor (Hadamards and rotations applied one at a time, whose real factors stay on the host), the other
    runs the same gates as one list; fidelity and max amplitude difference match the host figures"""
    import ctypes as C
    from qcsim_gb300 import _lib as L, gates as G
    n = 14
    ops = [(G.HadamardGate(), q) for q in range(n)] + [(G.RxGate(0.3 + 0.1 * q), q) for q in range(n)]
    ops += [(G.CNOTGate(), q, (q + 5) % n) for q in range(n)] + [(G.RyGate(-0.7), q) for q in range(0, n, 3)]
    a = Q.QubitRegister(n, seed=1)
    a.set_passes(False)
    for g, *qs in ops:
        a.ApplyGate(g, *qs)
    b = Q.QubitRegister(n, seed=1, precision=other_precision)
    b.ApplyGates(ops)
    lib = L.load()
    f, d = C.c_double(), C.c_double()
    L.check(lib.qcs_compare(a.handle, b.handle, C.byref(f), C.byref(d)), a.handle)
    va, vb = a.getRegisterStorage(), b.getRegisterStorage().astype(np.complex128)
    tol = 1e-13 if other_precision == "fp64" else 1e-6
    assert abs(d.value - np.abs(va - vb).max()) < tol
    assert abs(f.value - abs(np.vdot(va, vb)) ** 2 / (np.vdot(va, va).real * np.vdot(vb, vb).real)) < 1e-12
    assert d.value < (1e-12 if other_precision == "fp64" else 1e-5)
    a.close()
    b.close()


def test_pass_fp_op_count(Q):
    """the profile's floating-point instruction count of a shared-memory pass follows the gate forms: a
    factored rotation is one FMA per real component of each amplitude (2 per amplitude), a phase one
    complex product on half the amplitudes (2 per amplitude), a CNOT none"""
    from qcsim_gb300 import gates as G
    n = 16
    N = 1 << n
    reg = Q.QubitRegister(n, seed=1)
    reg.ApplyGates([(G.HadamardGate(), q) for q in range(n)])  # planning warm-up
    reg.profile(True)
    reg.read_profile()
    reg.ApplyGates([(G.RxGate(0.3), 3), (G.RzGate(0.2), 5), (G.CNOTGate(), 1, 7), (G.RyGate(0.4), 14)])
    prof = reg.read_profile(fp_ops=True)
    assert set(prof) == {"tile_pass"}, prof
    launches, _, _, ops = prof["tile_pass"]
    assert launches == 1 and ops == 6 * N, (launches, ops)
    reg.close()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_tile_factors(Q, precision):
    """diagonal gates whose target and controls all lie outside a pass's tile scale each tile by one factor:
    a pass with two or more of them applies their product as it stores the tile (TileFactor operations).
    Here one pass holds H on qubits 0-11 and phases (RZ and P) on qubits 12-17, a CP with a non-tile control
    and a CZ (a sign flip: a factor too where both its qubits lie outside the tile); unfused, so that FP32
    runs the same light pass.  The result matches the oracle, and the profile counts one complex product
    per amplitude for all the non-tile phases together"""
    from qcsim_gb300 import gates as G
    n = 18
    N = 1 << n
    tile = 12 if precision == "fp64" else 13  # H fixes qubits 0-11; the planner fills the tile from the bottom
    r = np.random.default_rng(5)
    ops = [(G.HadamardGate(), q) for q in range(12)]
    for q in range(12, 18):
        ops.append((G.RzGate(float(r.uniform(0, 2 * np.pi))), q))
        ops.append((G.PhaseShiftGate(float(r.uniform(0, 2 * np.pi))), q))
    ops += [(G.ControlledPhaseShiftGate(0.7), 15, 13), (G.ControlledZGate(), 16, 12)]
    init = rand_state(n, 9)
    reg = Q.QubitRegister(n, seed=1, precision=precision)
    reg.set_fusion(0)
    reg.setRegisterStorageFastNoNormalize(init)
    reg.ApplyGates(ops)  # planning warm-up
    reg.setRegisterStorageFastNoNormalize(init)
    reg.profile(True)
    reg.read_profile()
    reg.ApplyGates(ops)
    prof = reg.read_profile(fp_ops=True)
    got = reg.getRegisterStorage()
    want = oracle_state(n, ops, init)
    assert np.abs(got - want).max() <= (TOL if precision == "fp64" else 2e-6)
    launches, _, _, fp = prof["tile_pass"]
    # 12 factored rotations (2 per amplitude), each phase on a tile qubit one complex product on half the
    # amplitudes (2 per amplitude), and the factor product on every tile where it is not one
    local_phases = 2 * (tile - 12)
    factors = 2 * (18 - tile)
    cz = 0.75 if tile == 12 else 1.0  # the CZ's control (qubit 12) is a tile qubit in the 13-qubit tile
    want_fp = N * (2 * 12 + 2 * local_phases + 4 * (1 - 0.5 ** factors * 0.75 * cz))
    assert launches == 1 and abs(fp - want_fp) <= 1e-9 * want_fp, (launches, fp, want_fp)
    reg.close()


@pytest.mark.parametrize("batched", [False, True])
def test_fp32_long_factored_sequences(Q, batched):
    """600 Hadamards on one qubit of an FP32 register (each leaves a factor 1/sqrt(2) pending): the
    pending factor is folded before the stored values leave FP32's range, and H^600 = identity"""
    from qcsim_gb300 import gates as G
    n = 16
    rng = np.random.default_rng(3)
    v = rng.standard_normal(1 << n) + 1j * rng.standard_normal(1 << n)
    v /= np.linalg.norm(v)
    reg = Q.QubitRegister(n, seed=1, precision="fp32")
    reg.setRegisterStorageFastNoNormalize(v)
    ops = [(G.HadamardGate(), 3)] * 600
    if batched:
        reg.ApplyGates(ops)
    else:
        for g, q in ops:
            reg.ApplyGate(g, q)
    got = reg.getRegisterStorage()
    assert np.all(np.isfinite(got.view(np.float32)))
    assert np.abs(got - v).max() < 1e-5
    reg.close()


@pytest.mark.parametrize("n,precision", [(34, "fp64"), (35, "fp32")])
def test_largest_registers(Q, n, precision):
    """the largest register of each precision that HBM holds (2^n amplitudes = 256 GiB): gates through the
    pass planner (tiles with 22-23 fixed qubits), then exact qubit probabilities"""
    import torch
    from qcsim_gb300 import gates as G
    free, _ = torch.cuda.mem_get_info()
    need = (1 << n) * (16 if precision == "fp64" else 8)
    if free < need + (4 << 30):
        pytest.skip(f"{free / 2**30:.0f} GiB free, {need / 2**30:.0f} GiB needed")
    reg = Q.QubitRegister(n, seed=1, precision=precision)
    top = n - 1
    reg.ApplyGates([(G.HadamardGate(), top), (G.HadamardGate(), 0), (G.CNOTGate(), 17, top), (G.PauliXGate(), 9)])
    tol = 1e-12 if precision == "fp64" else 1e-6
    assert abs(reg.GetQubitProbability(top) - 0.5) < tol
    assert abs(reg.GetQubitProbability(17) - 0.5) < tol
    assert abs(reg.GetQubitProbability(0) - 0.5) < tol
    assert abs(reg.GetQubitProbability(9) - 1.0) < tol
    assert reg.GetQubitProbability(5) < tol
    assert abs(reg.getBasisStateAmplitude((1 << top) | (1 << 17) | (1 << 9)) - 0.5) < tol
    reg.close()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_one_qubit_transforms(Q, precision):
    """OneQubitGateTransform, HadamardTransform and XTransform (HadamardTransform.h:9-41) on sub-ranges
    [start, end] of a random state, against the oracle applying the reference's loop gate by gate;
    end beyond the register is clamped to n - 1 as QuantumSubAlgorithmOnSubregister does
    (QuantumAlgorithm.h:228-231).  FP64 1e-12, FP32 2e-6."""
    from qcsim_gb300 import gates as G, subalgo as S
    tol = TOL if precision == "fp64" else 2e-6
    for n in (7, 16):  # 16 qubits: the gate lists go through the shared-memory passes
        init = rand_state(n, n)
        reg = Q.QubitRegister(n, seed=1, precision=precision)
        ry = G.RyGate(0.83)
        for cls, gate, start, end in ((S.HadamardTransform, None, 0, S.INT_MAX), (S.XTransform, None, 2, n - 3),
                                      (S.OneQubitGateTransform, ry, 1, n + 5), (S.HadamardTransform, None, n - 1, n - 1),
                                      (S.OneQubitGateTransform, G.TGate(), 3, 3)):
            t = cls(n, start, end) if gate is None else cls(n, start, end, gate=gate)
            g = t.gate
            reg.setRegisterStorageFastNoNormalize(init)
            t.Execute(reg)
            ops = [(g, q) for q in range(t.getStartQubit(), t.getEndQubit() + 1)]
            err = float(np.abs(reg.getRegisterStorage() - oracle_state(n, ops, init)).max())
            assert err <= tol, (cls.__name__, start, end, err)
        reg.close()


def test_one_qubit_transform_rejects_bad_ranges(Q):
    """the C ABI rejects start > end, end >= n and a missing matrix before building the gate list, and
    leaves the state unchanged"""
    import ctypes as C
    from qcsim_gb300 import _lib as L, gates as G
    lib = L.load()
    n = 6
    reg = Q.QubitRegister(n, seed=1)
    init = rand_state(n, 3)
    reg.setRegisterStorageFastNoNormalize(init)
    m = np.ascontiguousarray(G.HadamardGate().getRawOperatorMatrix(), dtype=np.complex128)
    pm = m.view(np.float64).ctypes.data_as(C.POINTER(C.c_double))
    tr = G.HadamardGate().traits()
    for start, end in ((3, 2), (0, n), (0, 0xFFFFFFFF), (n, n)):
        assert lib.qcs_one_qubit_transform(reg.handle, pm, tr, start, end) == L.QCS_INVALID_ARGUMENT
    assert lib.qcs_one_qubit_transform(reg.handle, None, tr, 0, 1) == L.QCS_INVALID_ARGUMENT
    assert np.abs(reg.getRegisterStorage() - init).max() == 0.0
    reg.close()
