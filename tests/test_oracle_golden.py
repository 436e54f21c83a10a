"""Pin the CPU oracle to QCSim's own outputs (tests/golden/golden.npz, made by the compiled reference).

The oracle restates QubitRegister / QubitRegisterCalculator; these tests require it to reproduce the
reference's fixtures: amplitudes to 1e-13, measurement outcomes exactly.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import bind as B
from qcsim_gb300 import circuits
from qcsim_gb300.rng import Mt19937_64

TOL = 1e-13


def split_recs(g):
    out, off = [], 0
    for n, ln in zip(g["circ_n"], g["circ_len"]):
        out.append((int(n), g["circ_recs"][off:off + ln]))
        off += ln
    return out


def uniforms(seed, n):
    m = Mt19937_64(seed)
    return np.array([m.uniform() for _ in range(n)])


def test_rng_stream(golden, oracle_lib):
    for row, seed in zip(golden["rng_uniforms"], (1, 7, 123456789)):
        g = oracle_lib.qo_rng_create(seed)
        got = np.array([oracle_lib.qo_rng_uniform(g) for _ in range(row.size)])
        oracle_lib.qo_rng_destroy(g)
        assert np.array_equal(got, row)
        assert np.array_equal(uniforms(seed, row.size), row)


def test_gate_matrices(golden, oracle_lib):
    p = golden["gate_params"].copy()
    for code, m, k, t in zip(golden["gate_codes"], golden["gate_mats"], golden["gate_k"], golden["gate_traits"]):
        got = np.zeros(128)
        kk, tt = C.c_uint32(), C.c_uint32()
        assert oracle_lib.qo_gate_matrix(int(code), B.dp(p), B.dp(np.zeros(128)), B.dp(got), C.byref(kk), C.byref(tt)) == 0
        d = 1 << int(k)
        assert kk.value == k and tt.value == t, code
        assert np.array_equal(got[: 2 * d * d], m[: 2 * d * d]), code


def test_random_circuits(golden, oracle_lib):
    off = 0
    for n, recs in split_recs(golden):
        ref = golden["circ_states"][off:off + (1 << n)]
        off += 1 << n
        reg = B.OracleRegister(n)
        reg.apply(recs)
        assert np.abs(reg.state() - ref).max() <= TOL


def test_layered_12(golden, oracle_lib):
    reg = B.OracleRegister(12)
    reg.apply(golden["l12_recs"])
    st = reg.state()
    assert np.abs(st - golden["l12_state"]).max() <= TOL
    qp = [oracle_lib.qo_qubit_probability(reg.h, q) for q in range(12)]
    assert np.abs(np.array(qp) - golden["l12_qprob"]).max() <= TOL
    u = uniforms(7, 1025)
    shots = reg.sample(1.0 - u[:1024])
    keys, cnt = np.unique(shots, return_counts=True)
    assert np.array_equal(np.stack([keys, cnt.astype(np.uint64)], 1), golden["l12_hist"])
    assert oracle_lib.qo_measure_all(reg.h, 1.0 - u[1024]) == golden["l12_measure_all"][0]


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_layered_20(golden, oracle_lib, seed):
    reg = B.OracleRegister(20)
    reg.apply(circuits.layered_circuit(20, 40, seed=seed))
    st = reg.state()
    assert np.abs(st[golden["c0_probe_idx"]] - golden["c0_amp"][seed - 1]).max() <= TOL
    qp = np.array([oracle_lib.qo_qubit_probability(reg.h, q) for q in range(20)])
    assert np.abs(qp - golden["c0_qprob"][seed - 1]).max() <= 1e-12
    off = int(np.sum(golden["c0_hist_len"][: seed - 1]))
    hist = golden["c0_hist"][off:off + golden["c0_hist_len"][seed - 1]]
    shots = reg.sample(1.0 - uniforms(seed, 1024))
    keys, cnt = np.unique(shots, return_counts=True)
    assert np.array_equal(np.stack([keys, cnt.astype(np.uint64)], 1), hist)


def test_measurement_kats(golden, oracle_lib):
    """MeasurementsTests.cpp:34-167 state; outcomes and collapsed states for 16 seeds x 5 measures"""
    for (s, op, v), after in zip(golden["kat_rows"], golden["kat_after"]):
        reg = B.OracleRegister(2)
        reg.set_state(golden["kat_state"])
        oracle_lib.qo_normalize(reg.h)
        prob = 1.0 - uniforms(1000 + int(s), 1)[0]
        if op == 0:
            got = oracle_lib.qo_measure(reg.h, 0, 0, prob)
        elif op == 1:
            got = oracle_lib.qo_measure(reg.h, 1, 1, prob)
        elif op == 2:
            got = oracle_lib.qo_measure(reg.h, 0, 1, prob)
        elif op == 3:
            got = oracle_lib.qo_measure_all(reg.h, prob)
        else:
            got = oracle_lib.qo_measure_no_collapse(reg.h, prob)
        assert got == v
        assert np.abs(reg.state() - after).max() <= 1e-15


def test_subregister(golden, oracle_lib):
    for (a, b, v), after in zip(golden["sub_rows"], golden["sub_after"]):
        a, b = int(a), int(b)
        reg = B.OracleRegister(10)
        reg.set_state(golden["sub_state"])
        got = oracle_lib.qo_measure(reg.h, a, b, 1.0 - uniforms(31 + a * 10 + b, 1)[0])
        assert got == v
        assert np.abs(reg.state() - after).max() <= 1e-14
    for a, b in ((0, 0), (3, 5), (2, 9), (9, 9), (0, 9)):
        rows = golden["sub_hist"][(golden["sub_hist"][:, 0] == a) & (golden["sub_hist"][:, 1] == b)]
        reg = B.OracleRegister(10)
        reg.set_state(golden["sub_state"])
        shots = reg.sample(1.0 - uniforms(77 + a * 10 + b, 500))
        mask = ((1 << (b + 1)) - 1) - ((1 << a) - 1)
        sub = (shots & np.uint64(mask)) >> np.uint64(a)
        keys, cnt = np.unique(sub, return_counts=True)
        assert np.array_equal(keys, rows[:, 2]) and np.array_equal(cnt, rows[:, 3])


def test_scan_edges(golden, oracle_lib):
    """total probability 0.81: MeasureNoCollapse falls back to 0, MeasureAll to the last state and
    RepeatedMeasure to the table size (all as the reference)"""
    for row in golden["edge_rows"]:
        s = int(row[0])
        u = uniforms(500 + s, 66)
        reg = B.OracleRegister(10)
        reg.set_state(golden["edge_state"])
        assert oracle_lib.qo_measure_no_collapse(reg.h, 1.0 - u[0]) == row[2]
        shots = np.sort(reg.sample(1.0 - u[1:65]))
        assert np.array_equal(shots, row[3:])
        reg.set_state(golden["edge_state"])
        assert oracle_lib.qo_measure_all(reg.h, 1.0 - u[65]) == row[1]
    assert np.any(golden["edge_rows"][:, 3:] == 1024)  # some shots past the table


def test_qft(golden, oracle_lib):
    for cfg, inp, outp in zip(golden["qft_cfg"], golden["qft_in"], golden["qft_out"]):
        n, s0, e0, inv, sw = (int(x) for x in cfg)
        reg = B.OracleRegister(n)
        reg.set_state(inp[: 1 << n])
        assert oracle_lib.qo_qft(reg.h, s0, e0, inv, sw) == 0
        assert np.abs(reg.state() - outp[: 1 << n]).max() <= TOL


def test_qft_sign():
    """QFT|1> = 2^{-n/2} sum_k e^{+2 pi i k / 2^n} |k> for the reference's gate sequence"""
    n = 5
    reg = B.OracleRegister(n)
    st = np.zeros(1 << n, dtype=np.complex128)
    st[1] = 1
    reg.set_state(st)
    reg.lib.qo_qft(reg.h, 0, n - 1, 0, 1)
    k = np.arange(1 << n)
    assert np.abs(reg.state() - np.exp(2j * np.pi * k / (1 << n)) / np.sqrt(1 << n)).max() < 1e-14


def test_qaoa(golden, oracle_lib):
    insts = circuits.qaoa_instances(4, seed=8, nmin=6, nmax=10, p=2)
    for inst, n, st, en in zip(insts, golden["qaoa_n"], golden["qaoa_states"], golden["qaoa_energy"]):
        assert inst["n"] == n
        e = np.array(inst["edges"], dtype=np.uint32).reshape(-1)
        J, hv = np.array(inst["J"]), np.array(inst["h"])
        gm, bt = np.array(inst["gammas"]), np.array(inst["betas"])
        reg = B.OracleRegister(n)
        pu32 = e.ctypes.data_as(C.POINTER(C.c_uint32))
        assert oracle_lib.qo_qaoa_exec(reg.h, len(inst["edges"]), pu32, B.dp(J), B.dp(hv), len(gm), B.dp(gm), B.dp(bt)) == 0
        assert np.abs(reg.state() - st[: 1 << n]).max() <= TOL
        got = [oracle_lib.qo_ising_energy(n, len(inst["edges"]), pu32, B.dp(J), B.dp(hv), x) for x in range(1 << n)]
        assert np.abs(np.array(got) - en[: 1 << n]).max() <= 1e-12
        # the numpy energy table used by the engine tests agrees
        assert np.abs(circuits.ising_energies(inst) - en[: 1 << n]).max() <= 1e-12
        # and the circuit as a gate list reproduces the state
        reg2 = B.OracleRegister(n)
        reg2.apply(circuits.qaoa_circuit(inst))
        assert np.abs(reg2.state() - st[: 1 << n]).max() <= TOL


def test_expectation_and_replay(golden, oracle_lib):
    reg = B.OracleRegister(6)
    reg.apply(golden["exp_recs"])
    before = reg.state()
    reg.apply(golden["exp_pre"])
    val = np.vdot(before, reg.state())
    assert abs(val - complex(*golden["exp_value"])) <= 1e-13
    assert np.abs(before - golden["exp_state_after"]).max() <= TOL
    # Compute applies the recorded gates again (as matrix-only gates), Uncompute undoes them
    from qcsim_gb300 import gates as G
    ops = golden["exp_recs"]
    regc = B.OracleRegister(6)
    regc.apply(ops)
    matrix_only = []
    for r in ops:
        m = np.zeros(128)
        kk, tt = C.c_uint32(), C.c_uint32()
        oracle_lib.qo_gate_matrix(int(r["code"]), B.dp(r["p"].copy()), B.dp(r["m"].copy()), B.dp(m), C.byref(kk), C.byref(tt))
        d = 1 << kk.value
        mat = m[: 2 * d * d].view(np.complex128).reshape(d, d)
        matrix_only.append((G.AppliedGate(mat, int(r["q0"]), int(r["q1"]), int(r["q2"])), int(r["q0"]), int(r["q1"]), int(r["q2"])))
    regc.apply(matrix_only)
    assert np.abs(regc.state() - golden["replay_states"][0]).max() <= TOL
    regu = B.OracleRegister(6)
    regu.apply(ops)
    regu.apply([(G.AppliedGate(g.getRawOperatorMatrix().conj().T, a, b, c), a, b, c) for (g, a, b, c) in reversed(matrix_only)])
    assert np.abs(regu.state() - golden["replay_states"][1]).max() <= TOL


def test_invalid_arguments(oracle_lib):
    from qcsim_gb300 import gates as G
    reg = B.OracleRegister(3)
    for ops, msg in (([(G.HadamardGate(), 3, 0, 0)], "Qubit number is too high"),
                     ([(G.CNOTGate(), 1, 1, 0)], "Qubit and controlling qubit are the same"),
                     ([(G.CNOTGate(), 1, 5, 0)], "Controlling qubit number is too high"),
                     ([(G.ToffoliGate(), 0, 1, 1)], "Qubits must be different")):
        with pytest.raises(ValueError, match=msg):
            reg.apply(ops)


@pytest.mark.skipif(not B.REF_LIB.exists(), reason="the compiled reference (make -C oracle ref) is not built")
@pytest.mark.parametrize("generator,fixture", [("make_golden", "golden"), ("make_oracles", "oracles"),
                                               ("make_pauli", "pauli"), ("make_nqubits", "nqubits")])
def test_compiled_reference_reproduces_fixtures(generator, fixture):
    """the committed fixtures are what the generators make from QCSim's own register, compiled here:
    integer outputs (shots, histograms, record fields) exactly, floating-point ones to 1e-13 (OpenMP
    reduction order of the probability sums; LAPACK's last bits in the random unitaries on other hosts)"""
    import importlib
    import sys
    from pathlib import Path
    golden_dir = Path(__file__).resolve().parent / "golden"
    if str(golden_dir) not in sys.path:
        sys.path.insert(0, str(golden_dir))
    out = importlib.import_module(generator).generate(B.ref())
    want = np.load(golden_dir / f"{fixture}.npz")
    assert set(out) == set(want.files)
    def same(name, a, b):
        assert a.shape == b.shape, name
        if a.dtype.names:
            for f in a.dtype.names:
                same(f"{name}.{f}", a[f], b[f])
        elif a.dtype.kind in "iu":
            assert np.array_equal(a, b), name
        elif a.size:
            assert float(np.abs(a - b).max()) <= 1e-13, name

    for k, a in out.items():
        same(k, np.asarray(a), want[k])
