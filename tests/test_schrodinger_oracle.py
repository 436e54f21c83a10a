"""The Schrodinger split-operator workload on the CPU: the oracle's restatement of
SchrodingerSimulation::Execute (QFT steps through the pinned oracle QFT) agrees with an independent
host-DFT evolution, and the engine mirror builds the same operator diagonals."""
import math

import numpy as np
import pytest

from oracle import schrodinger as S


@pytest.mark.parametrize("n,pot", [(8, "barrier"), (9, "step"), (10, "free")])
def test_qft_evolution_matches_host_dft(oracle_lib, n, pot):
    nb = 1 << n
    V = {"barrier": S.barrier(n, 30.0, nb // 16), "step": S.step_right(n, 15.0), "free": np.zeros(nb)}[pot]
    psi0 = S.gaussian(n, 0.1, nb // 4, 6.0, 12.0)
    a = S.evolve(psi0, n, 0.005, 0.1, V, 12)
    b = S.classical_fft_evolve(psi0, n, 0.005, 0.1, V, 12)
    assert np.abs(a - b).max() < 1e-12
    assert abs(np.linalg.norm(a) - 1) < 1e-12


def test_mirror_operator_diagonals():
    """the engine mirror's vectorised Init equals the reference-order scalar restatement"""
    from qcsim_gb300.schrodinger import _polar
    n, dt, dx = 10, 0.007, 0.05
    V = S.barrier(n, 25.0, 40)
    pot, kin = S.operators(n, dt, dx, V)
    half_x = 0.5 * dx * ((1 << n) - 1.0)
    x = dx * np.arange(1 << n) - half_x
    assert np.abs(_polar(-V * dt) - pot).max() < 1e-15
    assert np.abs(_polar(-0.5 * x * x * dt) - kin).max() < 1e-15
    # the walls (1e150) and large kinetic angles reduce exactly
    assert np.array_equal(_polar(-V * dt)[[0, -1]], pot[[0, -1]])
    big = np.array([1e9, -3.7e12, 2.5e15, 1e150])
    assert np.array_equal(_polar(big), np.array([complex(math.cos(t), math.sin(t)) for t in big]))
