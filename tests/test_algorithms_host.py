"""Host-side parts of the algorithm mirrors, no GPU: Shor's classical steps (gcd, continued fraction,
convergents: ShorAlgorithm.h:214-258), VQE's Nelder-Mead geometry and vertex ranking (VQE.h:383-452), the
Bernstein-Vazirani oracle (BernsteinVazirani.h:16-57) and the Grover oracle (GroverAlgorithm.h:16-40)."""
from fractions import Fraction

import numpy as np

from qcsim_gb300 import algorithms as A
from qcsim_gb300 import vqe as V


def test_shor_classical_steps():
    S = A.ShorAlgorithm
    assert S.gcd(15, 6) == 3 and S.gcd(21, 5) == 1 and S.gcd(0, 7) == 7
    # 3/8 = [0; 2, 1, 2]; in floating point 1 / (2/3) = 1.5000000000000004, so the expansion goes on as
    # [0, 2, 1, 1, 1] (the reference's C++ takes the same IEEE steps); its last convergent is still 3/8
    assert S.continuedFraction(3 / 8, 3) == [0, 2, 1]
    nums, dens = S.getFractions(S.continuedFraction(3 / 8, 8))
    assert S.continuedFraction(3 / 8, 8) == [0, 2, 1, 1, 1]
    assert dens == [1, 2, 3, 5, 8] and nums == [0, 1, 1, 2, 3]
    assert Fraction(nums[-1], dens[-1]) == Fraction(3, 8)
    # a measured x / 2^L near s / r gives r among the convergents' denominators
    for r, L in ((4, 3), (6, 9)):
        x = round(5 / r * 2 ** L) % 2 ** L
        _, d = S.getFractions(S.continuedFraction(x / 2 ** L, L))
        assert any(r % q == 0 or q % r == 0 for q in d[1:] if q)


def test_vqe_nelder_mead_geometry():
    VQE = V.VariationalQuantumEigensolver
    pts = [[0.0, 0.0], [2.0, 0.0], [0.0, 4.0]]
    assert VQE.Centroid(pts) == [2 / 3, 4 / 3]
    assert VQE.Centroid(pts, 2) == [1.0, 0.0]
    assert VQE.ReflectionPoint([1.0, 1.0], [3.0, 0.0], 2.0) == [5.0, -1.0]
    assert VQE.ReflectionPoint([1.0, 1.0], [3.0, 0.0], 0.5) == [2.0, 0.5]
    solver = object.__new__(VQE)
    solver.vertexEnergies = [0.5, 3.0, -1.0, 2.0]
    minE, maxE, maxE2, minI, maxI, maxI2 = solver.GetMinMaxEnergy()
    assert (minE, minI, maxE, maxI) == (-1.0, 2, 3.0, 1)
    assert (maxE2, maxI2) == (0.5, 0)  # the reference tracks the previous maximum only (VQE.h:436-451)
    solver.vertices = [[0.0], [1.0], [2.0], [3.0]]
    assert solver.GetMinEnergy() == -1.0 and solver.GetMinVertex() == [2.0]


def test_oracles():
    o = A.BernsteinVaziraniOracle()
    o.setString(0b1101)
    m = o.getOperatorMatrix(5)
    for x in range(32):
        assert m[x, x] == (-1 if bin(x & 0b1101).count("1") % 2 else 1)
    assert np.count_nonzero(m - np.diag(np.diag(m))) == 0
    g = A.GroverOracle()
    g.setCorrectQuestionState(5)
    gm = g.getOperatorMatrix(3)
    assert gm[5, 5] == -1 and np.trace(gm) == 6


class _HostRegister:
    """stands in for the engine register where only the register's size is read"""

    def __init__(self, N, *a, **kw):
        self.N = N

    def getNrQubits(self):
        return self.N

    def getNrBasisStates(self):
        return 1 << self.N


def _host_algorithm(monkeypatch, cls, *args, **kw):
    def init(self, N=3, addseed=0, **_):
        self.reg = _HostRegister(N)
    monkeypatch.setattr(A.QuantumAlgorithm, "__init__", init)
    return cls(*args, **kw)


def _is_permutation(u):
    return (np.count_nonzero(u) == u.shape[0] and np.all(np.abs(u).sum(axis=0) == 1)
            and np.all(np.abs(u).sum(axis=1) == 1))


def test_simon_function_and_oracle(monkeypatch):
    """SimonFunction (SimonAlgorithm.h:15-97) is one-to-one for s = 0 and two-to-one with f(x) = f(x ^ s)
    otherwise; the oracle (SimonAlgorithm.h:104-136) maps |x>|y> to |x>|y ^ f(x)>"""
    for N in (2, 3, 4):
        for s in range(1 << N):
            f = A.SimonFunction(np.random.default_rng(s))
            f.setString(s, N)
            assert f.checkFunction()
            if s:
                assert all(f(x) == f(x ^ s) for x in range(1 << N))
    simon = _host_algorithm(monkeypatch, A.SimonAlgorithm, 3, function_seed=4)
    simon.setString(0b101)
    u = simon.OracleOp
    assert _is_permutation(u)
    for bra in range(64):
        x, y = bra & 7, bra >> 3
        assert u[x | ((y ^ int(simon.f(x))) << 3), bra] == 1


def test_deutsch_jozsa_oracle(monkeypatch):
    """DeutschJozsa.h:54-72, :104-129: balanced functions take the value 1 on half the inputs; the oracle maps
    |y>|x> to |y + f(x)>|x> with y the top qubit"""
    dj = _host_algorithm(monkeypatch, A.DeutschJozsaAlgorithm, 5, function_seed=2)
    FT = A.DeutschJozsaAlgorithm.FunctionType
    for ft, ones in ((FT.constantZero, 0), (FT.constantOne, 16), (FT.balanced, 8)):
        dj.setFunction(ft)
        fx = dj.f(np.arange(16))
        assert int(fx.sum()) == ones
        u = dj.getOracleMatrix()
        assert _is_permutation(u)
        for bra in range(32):
            assert u[(bra & 15) | (((bra >> 4) ^ int(fx[bra & 15])) << 4), bra] == 1
    assert dj.WasConstantResult(16) and not dj.WasConstantResult(3)


def test_n_controlled_not_with_ancilla():
    """NControlledNotWithAncilla.h:27-100: the target flips exactly when every control is set, and the
    ancillas are returned to 0 (the recorded ancilla computation is undone)"""
    from qcsim_gb300 import counting as Q
    for nc in range(1, 8):
        controls = list(range(nc))
        target, anc0 = nc, nc + 1
        g = Q.NControlledNotWithAncilla()
        g.SetControlQubits(controls)
        g.SetTargetQubit(target)
        g.SetStartAncillaQubits(anc0)
        seq = Q.GateSequence()
        g.Execute(seq)
        for c in range(1 << nc):
            bits = c
            for gate, t, c1, c2 in seq.ops:
                if gate.getQubitsNumber() == 3:
                    if (bits >> c1) & (bits >> c2) & 1:
                        bits ^= 1 << t
                elif (bits >> c1) & 1:
                    bits ^= 1 << t
            assert bits >> anc0 == 0, (nc, c)
            assert (bits >> target) & 1 == (c == (1 << nc) - 1), (nc, c)


def test_quantum_counting_circuit_on_the_oracle(monkeypatch):
    """QuantumCountingAlgorithm.h:104-179 and CountingTests (Tests.cpp:619-663) at 3 Grover qubits and 6
    precision qubits: the gate list plus the inverse QFT (no swaps) on the CPU oracle; the most probable
    precision value gives the number of marked states, and the ancillas end in |0>"""
    from oracle import bind as B
    from qcsim_gb300 import counting as Q
    P, Gq = 6, 3
    n = P + 2 * Gq
    rng = np.random.default_rng(11)
    for marked in range(0, (1 << Gq) + 1):
        qc = _host_algorithm(monkeypatch, Q.QuantumCountingAlgorithm, P, Gq)
        qc.SetMarkedStates(rng.permutation(1 << Gq)[:marked].tolist())
        ref = B.OracleRegister(n)
        ref.apply(qc.circuit())
        assert B.oracle().qo_qft(ref.h, 0, P - 1, 1, 0) == 0
        p = np.abs(ref.state()) ** 2
        assert p[np.arange(p.size) >> (P + Gq) != 0].sum() < 1e-20
        px = np.bincount(np.arange(p.size) & ((1 << P) - 1), weights=p)
        assert qc.GetCountForState(int(np.argmax(px))) == marked


def test_operator_basis_change():
    """MeasurementBasis::switchToOperatorBasis (Utils.h:143-205): the unitary diagonalises the operator with the
    larger eigenvalue first; Z gives the identity, -Z the swap, and switchBack the adjoint"""
    from qcsim_gb300.measurement_basis import MeasurementBasis as MB
    z = np.diag([1.0, -1.0]).astype(np.complex128)
    x = np.array([[0, 1], [1, 0]], dtype=np.complex128)
    y = np.array([[0, -1j], [1j, 0]])
    assert np.array_equal(MB.operatorBasisMatrix(z), np.eye(2))
    assert np.array_equal(MB.operatorBasisMatrix(-z), np.array([[0, 1], [1, 0]]))
    rng = np.random.default_rng(3)
    ops = [x, y, (-z - x) / np.sqrt(2), (z - x) / np.sqrt(2)]
    for _ in range(20):
        a, b = rng.standard_normal(2)
        c = complex(*rng.standard_normal(2))
        ops.append(np.array([[a, c], [np.conj(c), b]]))
    for op in ops:
        U = MB.operatorBasisMatrix(op)
        assert np.abs(U @ U.conj().T - np.eye(2)).max() < 1e-14
        d = U @ op @ U.conj().T
        ev = np.linalg.eigvalsh(op)
        assert abs(d[0, 1]) < 1e-12 and abs(d[1, 0]) < 1e-12
        assert abs(d[0, 0] - ev[1]) < 1e-12 and abs(d[1, 1] - ev[0]) < 1e-12
        assert np.array_equal(MB.operatorBasisMatrix(op, True), U.conj().T)
