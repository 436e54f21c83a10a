"""The dense operator gates on the CPU: the oracle's restatement of NQubitsQuantumGate /
NQubitsControlledQuantumGate and the Python mirror classes reproduce QCSim's own extended matrices and
Execute results (tests/golden/nqubits.npz, made by the compiled reference), and the contraction form
used for arbitrary placements agrees with them."""
import numpy as np
import pytest

from oracle import nqubits as O
from qcsim_gb300 import subalgo as A

ROOT_GOLDEN = __import__("pathlib").Path(__file__).resolve().parent / "golden" / "nqubits.npz"


@pytest.fixture(scope="module")
def fx():
    return np.load(ROOT_GOLDEN)


def cases(fx):
    for i, (n, k, ctrl) in enumerate(fx["cases"]):
        yield i, int(n), int(k), int(ctrl)


def test_extended_matrices_match_reference(fx):
    seen = 0
    for i, n, k, ctrl in cases(fx):
        if f"ext{i}" not in fx.files:
            continue
        op, ext = fx[f"op{i}"], fx[f"ext{i}"]
        c = None if ctrl < 0 else ctrl
        assert np.array_equal(O.extended_operator(n, op, n - k, c), ext), i
        g = A.NQubitsQuantumGate(n, op, n - k) if c is None else A.NQubitsControlledQuantumGate(n, op, n - k, c)
        assert np.array_equal(g.getOperatorMatrix(), ext), i
        seen += 1
    assert seen >= 6


def test_execute_results_match_reference(fx):
    for i, n, k, ctrl in cases(fx):
        op, psi, out = fx[f"op{i}"], fx[f"psi{i}"], fx[f"out{i}"]
        ctrls = [] if ctrl < 0 else [ctrl]
        got = O.apply_on_qubits(psi, op, list(range(n - k, n)), ctrls)
        assert np.abs(got - out).max() < 1e-14, i
        if n <= 6:
            assert np.abs(O.extended_operator(n, op, n - k, None if ctrl < 0 else ctrl) @ psi - out).max() < 1e-14, i


def test_contraction_against_brute_force():
    rng = np.random.default_rng(5)
    n = 6
    for _ in range(25):
        k = int(rng.integers(1, 5))
        qs = [int(q) for q in rng.permutation(n)[:k]]
        rest = [q for q in range(n) if q not in qs]
        ctrls = [int(q) for q in rng.permutation(rest)[: int(rng.integers(0, min(3, len(rest)) + 1))]]
        op = rng.standard_normal((1 << k, 1 << k)) + 1j * rng.standard_normal((1 << k, 1 << k))
        psi = rng.standard_normal(1 << n) + 1j * rng.standard_normal(1 << n)
        want = psi.copy()
        for i in range(1 << n):
            if all((i >> c) & 1 for c in ctrls):
                r = sum(((i >> q) & 1) << j for j, q in enumerate(qs))
                base = i & ~sum(1 << q for q in qs)
                want[i] = sum(op[r, c] * psi[base | sum(((c >> j) & 1) << q for j, q in enumerate(qs))] for c in range(1 << k))
        assert np.abs(O.apply_on_qubits(psi, op, qs, ctrls) - want).max() < 1e-12, (qs, ctrls)


def test_mirror_placement_checks():
    op = np.eye(4)
    with pytest.raises(ValueError):
        A.NQubitsQuantumGate(3, op, 2)  # qubits 2, 3 of a 3-qubit register
    with pytest.raises(ValueError):
        A.NQubitsControlledQuantumGate(4, op, 1, 2)  # control among the targets
    with pytest.raises(ValueError):
        A.NQubitsQuantumGate(4, np.eye(3))  # not 2^k x 2^k
    g = A.NQubitsControlledQuantumGate(5, op, 3, 0)
    assert g.targets() == [3, 4] and g.controls() == [0] and g.getRawOperatorQubitsNumber() == 2
