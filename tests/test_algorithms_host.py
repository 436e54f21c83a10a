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
