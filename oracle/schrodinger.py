"""CPU oracle for the Schrodinger split-operator workload -- TEST INFRASTRUCTURE ONLY.

Only tests/ and bench.py's CPU leg use this module, as the checker or the timed CPU baseline.

QCSim's QuantumSimulation::SchrodingerSimulation (Schrodinger.h) cannot be compiled here: it includes
FFT.h, which needs FFTW (fftw3.h), and Eigen's unsupported modules, none of which are installed.  This
module restates its Execute / Init / setGaussian / potential setters in plain numpy loops, each citing
the reference lines.  The two transforms of every step are the oracle's QFT (qcs_oracle.cpp: qo_qft),
which is pinned to the reference's own QFT sub-algorithm by tests/golden/golden.npz, and the
diagonal operators are the element-wise products the reference's dense diagonal matrices amount to.
classical_fft_evolve is an independent host-DFT form of the same evolution (numpy's FFT in place of the
QFT, the convention mapped below); it plays the part of the reference's solveWithClassicalFFT
(Schrodinger.h:240-284).
"""
from __future__ import annotations

import math

import numpy as np

from . import bind as B


def operators(n: int, dt: float, dx: float, potential: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """Init (Schrodinger.h:291-315): the diagonals of potentialOp = polar(1, -V_i dt) and kineticOp =
    polar(1, -x_i^2 dt / 2), x_i = dx i - dx (2^n - 1) / 2"""
    nb = 1 << n
    half_x = 0.5 * dx * (nb - 1.0)
    kin = np.empty(nb, dtype=np.complex128)
    pot = np.empty(nb, dtype=np.complex128)
    for i in range(nb):
        x = dx * i - half_x
        kin[i] = complex(math.cos(-0.5 * x * x * dt), math.sin(-0.5 * x * x * dt))
        pot[i] = complex(math.cos(-potential[i] * dt), math.sin(-potential[i] * dt))
    return pot, kin


def gaussian(n: int, dx: float, pos: int, stdev: float, k: float) -> np.ndarray:
    """setGaussian (Schrodinger.h:106-136): a * exp(-e^2 / 2 + i k x) on points 1 .. 2^n - 2, normalised"""
    nb = 1 << n
    stdev *= dx
    a = 1.0 / (stdev * math.sqrt(2.0 * math.pi))
    half_x = 0.5 * dx * (nb - 1.0)
    m = dx * pos - half_x
    v = np.zeros(nb, dtype=np.complex128)
    for i in range(1, nb - 1):
        x = dx * i - half_x
        e = (x - m) / stdev
        v[i] = a * complex(math.exp(-0.5 * e * e) * math.cos(k * x), math.exp(-0.5 * e * e) * math.sin(k * x))
    return v / np.linalg.norm(v)


def barrier(n: int, val: float, halfwidth: int) -> np.ndarray:
    """setConstantPotentialInTheMiddle (Schrodinger.h:76-88)"""
    nb = 1 << n
    v = np.zeros(nb)
    for i in range(max(1, nb // 2 - halfwidth), min(nb - 1, nb // 2 + halfwidth)):
        v[i] = val
    v[0] = v[nb - 1] = 1e150
    return v


def step_right(n: int, val: float) -> np.ndarray:
    """setConstantPotentialToRight (Schrodinger.h:91-102)"""
    nb = 1 << n
    v = np.zeros(nb)
    v[nb // 2:] = val
    v[0] = 1e15
    v[nb - 1] = 1e150
    return v


def evolve(state: np.ndarray, n: int, dt: float, dx: float, potential: np.ndarray, steps: int) -> np.ndarray:
    """Execute (Schrodinger.h:32-45) from a given start state: normalise, then per step the potential
    diagonal, the IQFT of the whole register with its swaps, the kinetic diagonal and the QFT"""
    pot, kin = operators(n, dt, dx, potential)
    return evolve_with(state / np.linalg.norm(state), n, pot, kin, steps)


def evolve_with(psi: np.ndarray, n: int, pot: np.ndarray, kin: np.ndarray, steps: int) -> np.ndarray:
    """the steps of Execute (Schrodinger.h:36-42) with the operators' diagonals given"""
    reg = B.OracleRegister(n)
    for _ in range(steps):
        reg.set_state(psi * pot)
        B.oracle().qo_qft(reg.h, 0, n - 1, 1, 1)
        reg.set_state(reg.state() * kin)
        B.oracle().qo_qft(reg.h, 0, n - 1, 0, 1)
        psi = reg.state()
    return psi


def classical_fft_evolve(state: np.ndarray, n: int, dt: float, dx: float, potential: np.ndarray, steps: int) -> np.ndarray:
    """the same steps with numpy's FFT: the register's QFT (with swaps) is the unitary DFT with kernel
    exp(+2 pi i j k / 2^n), i.e. sqrt(2^n) * ifft, and its IQFT is fft / sqrt(2^n)"""
    pot, kin = operators(n, dt, dx, potential)
    r = math.sqrt(1 << n)
    psi = state / np.linalg.norm(state)
    for _ in range(steps):
        psi = np.fft.fft(psi * pot) / r
        psi = np.fft.ifft(psi * kin) * r
    return psi
