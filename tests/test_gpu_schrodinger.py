"""The Schrodinger split-operator workload on the GPU (qcs_schrodinger_evolve through the
SchrodingerSimulation mirror) and diagonal operators (qcs_apply_diagonal), against the oracle:
the restated Execute on small registers, the host-DFT evolution on larger ones.  FP64 tolerance 1e-11
on amplitudes after the steps; FP32 1e-5."""
import numpy as np
import pytest

from oracle import schrodinger as S

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


def simulation(n, dt, dx, steps, precision="fp64"):
    from qcsim_gb300.schrodinger import SchrodingerSimulation
    return SchrodingerSimulation(n, dt, dx, steps, precision=precision)


def test_execute_matches_restated_reference(Q, oracle_lib):
    """10 qubits (one kernel per gate): a Gaussian packet on a barrier, 20 steps"""
    n, dt, dx, steps = 10, 0.005, 0.1, 20
    sim = simulation(n, dt, dx, steps)
    sim.setGaussian(256, 6.0, 12.0)
    sim.setConstantPotentialInTheMiddle(30.0, 48)
    psi0 = sim.getRegisterStorage().copy()
    sim.Execute()
    want = S.evolve(psi0, n, dt, dx, sim.potential, steps)
    assert np.abs(sim.getRegisterStorage() - want).max() < 1e-12
    sim.close()


@pytest.mark.parametrize("n,steps,precision", [(16, 12, "fp64"), (20, 6, "fp64"), (18, 10, "fp32")])
def test_execute_matches_host_dft(Q, n, steps, precision):
    """shared-memory passes with the diagonals inside the transforms' passes: no launch of their own"""
    dt, dx = 0.002, 0.05
    nb = 1 << n
    sim = simulation(n, dt, dx, steps, precision)
    sim.setGaussian(nb // 4, 40.0, 20.0)
    sim.setConstantPotentialToRight(8.0)
    psi0 = sim.getRegisterStorage().astype(np.complex128)
    sim.reg.profile(True)
    sim.reg.read_profile()
    sim.Execute()
    prof = sim.reg.read_profile()
    assert prof and all(k.startswith("tile_pass") for k in prof), prof
    got = sim.getRegisterStorage().astype(np.complex128)
    want = S.classical_fft_evolve(psi0, n, dt, dx, sim.potential, steps)
    tol = 1e-11 if precision == "fp64" else 1e-5
    assert np.abs(got - want).max() < tol
    assert abs(np.linalg.norm(got) - 1) < (1e-12 if precision == "fp64" else 1e-5)
    sim.close()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_diagonal_operator(Q, precision):
    rng = np.random.default_rng(8)
    n = 9
    N = 1 << n
    v = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    v /= np.linalg.norm(v)
    d = np.exp(1j * rng.uniform(0, 2 * np.pi, N)) * rng.uniform(0.5, 1.5, N)
    tol = 1e-15 if precision == "fp64" else 1e-6
    reg = Q.QubitRegister(n, seed=1, precision=precision)
    reg.setRegisterStorageFastNoNormalize(v)
    reg.ApplyDiagonal(d)
    assert np.abs(reg.getRegisterStorage() - d * v).max() < tol
    # ApplyOperatorMatrix of a diagonal matrix takes the same route, a dense one the dense product
    reg.setRegisterStorageFastNoNormalize(v)
    reg.profile(True)
    reg.read_profile()
    reg.ApplyOperatorMatrix(np.diag(d))
    assert "table_diag" in reg.read_profile()
    assert np.abs(reg.getRegisterStorage() - d * v).max() < tol
    m = np.diag(d)
    m[3, 5] = 0.25
    reg.setRegisterStorageFastNoNormalize(v)
    reg.ApplyOperatorMatrix(m)
    assert np.abs(reg.getRegisterStorage() - m @ v).max() < (1e-14 if precision == "fp64" else 1e-6)
    reg.close()
