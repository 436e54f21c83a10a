"""Host-side checks of the Ising model and QAOA sub-algorithm mirror (qcsim_gb300.ising), no GPU: the model's
energies against the oracle's (IsingModel.h:106-179), the circuit of Exec against the oracle's QAOA circuit
(IsingModel.h:485-567, pinned to the compiled reference), and the optimiser of Execute (IsingModel.h:220-273,
580-636) on a stand-in register over the CPU oracle with QCSim's IsingTests.cpp settings."""
import ctypes as C

import numpy as np
import pytest

from oracle import bind as B
from qcsim_gb300 import circuits
from qcsim_gb300 import ising as I


class OracleBackedRegister:
    """the register members the QAOA sub-algorithm calls, over the CPU oracle, with seeded multinomial
    sampling in place of the register's RepeatedMeasure"""

    def __init__(self, n, seed):
        self.n = n
        self.r = B.OracleRegister(n)
        self.rng = np.random.default_rng(seed)

    def getNrQubits(self):
        return self.n

    def setToBasisState(self, s):
        v = np.zeros(1 << self.n, dtype=np.complex128)
        v[s] = 1
        self.r.set_state(v)

    def ApplyGates(self, ops):
        self.r.apply(ops)

    def RepeatedMeasure(self, shots):
        p = np.abs(self.r.state()) ** 2
        counts = self.rng.multinomial(shots, p / p.sum())
        return {int(i): int(c) for i, c in enumerate(counts) if c}


def _model(inst):
    m = I.IsingModel()
    m.Set([(i, j, J) for (i, j), J in zip(inst["edges"], inst["J"])], inst["h"])
    return m


def test_model_energies_match_the_oracle():
    lib = B.oracle()
    for inst in circuits.qaoa_instances(4, seed=8, nmin=6, nmax=10, p=2):
        m = _model(inst)
        n = inst["n"]
        e = np.array(inst["edges"], dtype=np.uint32).reshape(-1)
        pu = e.ctypes.data_as(C.POINTER(C.c_uint32))
        J, h = np.array(inst["J"]), np.array(inst["h"])
        want = np.array([lib.qo_ising_energy(n, len(inst["edges"]), pu, B.dp(J), B.dp(h), x) for x in range(1 << n)])
        assert np.abs(m.Energies() - want).max() <= 1e-12
        assert all(abs(m.Energy(x) - want[x]) <= 1e-12 for x in range(0, 1 << n, 7))
        assert m.GetMinEnergyState() == int(np.argmin(want))
        assert int(np.argmin(want)) in m.GetMinEnergyStates()


def test_min_energy_states_with_ties():
    """the max-cut graph of MaxCutTest (IsingTests.cpp:45-93): a degenerate ground state, found as a set"""
    m = I.IsingModel()
    m.Set([(0, 1, -1), (0, 2, -1), (0, 5, -1), (1, 2, -1), (1, 3, -1), (2, 3, -1), (2, 4, -1), (3, 5, -1)], [0.0] * 6)
    e = m.Energies()
    states = m.GetMinEnergyStates()
    assert states == set(np.flatnonzero(np.abs(e - e.min()) <= 1e-9).tolist())
    assert len(states) >= 2 and all((63 ^ s) in states for s in states)  # flipping every spin keeps the cut


def test_exec_circuit_matches_the_oracle():
    lib = B.oracle()
    for inst in circuits.qaoa_instances(3, seed=5, nmin=6, nmax=8, p=3):
        q = I.QAOAIsingSubalgorithm()
        q.Set([(i, j, J) for (i, j), J in zip(inst["edges"], inst["J"])], inst["h"])
        n = inst["n"]
        reg = OracleBackedRegister(n, 0)
        q.Exec(reg, inst["gammas"], inst["betas"])
        ref = B.OracleRegister(n)
        e = np.array(inst["edges"], dtype=np.uint32).reshape(-1)
        J, h = np.array(inst["J"]), np.array(inst["h"])
        g, b = np.array(inst["gammas"]), np.array(inst["betas"])
        assert lib.qo_qaoa_exec(ref.h, len(inst["edges"]), e.ctypes.data_as(C.POINTER(C.c_uint32)), B.dp(J), B.dp(h),
                                len(g), B.dp(g), B.dp(b)) == 0
        assert np.abs(reg.r.state() - ref.state()).max() <= 1e-12


@pytest.mark.parametrize("seed", [1, 2])
def test_optimiser_ising_model(seed):
    """IsingModelTest (IsingTests.cpp:6-43): three spins, p = 3, fixed starts, better mixing; the state
    returned is the ground state"""
    q = I.QAOAIsingSubalgorithm()
    q.Set([(0, 1, 1.5), (1, 2, 2), (0, 2, -3)], [1.25, 3.25, -2.5])
    q.SetP(3)
    q.SetGammaStart(1)
    q.SetBetaStart(3)
    q.SetGammaStart(0.3, 1)
    q.SetBetaStart(1, 1)
    q.SetMixing(True)
    state = q.Execute(OracleBackedRegister(3, seed))
    assert len(q.history) >= 1
    assert state == q.GetMinEnergyState()


@pytest.mark.parametrize("seed", [1, 2])
def test_optimiser_max_cut(seed):
    """MaxCutTest (IsingTests.cpp:45-93): six vertices, p = 2; the state returned is a maximum cut"""
    q = I.QAOAIsingSubalgorithm()
    q.Set([(0, 1, -1), (0, 2, -1), (0, 5, -1), (1, 2, -1), (1, 3, -1), (2, 3, -1), (2, 4, -1), (3, 5, -1)], [0.0] * 6)
    q.SetP(2)
    q.SetGammaStart(6)
    q.SetBetaStart(0.7)
    q.SetGammaStart(4.2, 1)
    q.SetBetaStart(0.5, 1)
    state = q.Execute(OracleBackedRegister(6, seed))
    assert state in q.GetMinEnergyStates()
