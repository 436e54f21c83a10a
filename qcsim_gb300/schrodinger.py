"""QCSim's QuantumSimulation::SchrodingerSimulation (Schrodinger.h:19-361) over the engine: a particle in
a 1D box of 2^N grid points evolved by the Suzuki-Trotter split operator, with the momentum-space step
done by the quantum Fourier transform.

Execute (Schrodinger.h:32-45) runs as one engine call, qcs_schrodinger_evolve.  The potential and
kinetic operators are diagonal (Init, Schrodinger.h:291-315).  They go to the device once, as their
2^N diagonal entries; the reference multiplies 2^N x 2^N matrices instead (ApplyOperatorMatrix,
:335-347).  On the device the diagonals run inside the shared-memory passes of the IQFT and QFT.

The reference's finite-difference and FFTW solvers (solveWithFiniteDifferences*, solveWithClassicalFFT,
:147-288) are host-side cross-checks of the quantum evolution and are not part of the engine.
"""
from __future__ import annotations

import ctypes as C
import math
import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np

from .subalgo import QuantumAlgorithm


def _polar(t: np.ndarray) -> np.ndarray:
    """cos t + i sin t, as std::polar(1, t); numpy's float64 cos and sin reduce arguments of any size
    exactly (the kinetic angles reach 1e12 and the walls 1e150).  Large arrays are split over host
    threads (numpy's ufuncs release the interpreter lock)."""
    t = np.ascontiguousarray(t, dtype=np.float64)
    out = np.empty(t.shape, dtype=np.complex128)
    parts = out.view(np.float64).reshape(-1, 2)

    def fill(lo: int, hi: int) -> None:
        np.cos(t[lo:hi], out=parts[lo:hi, 0])
        np.sin(t[lo:hi], out=parts[lo:hi, 1])

    chunk = 1 << 20
    if t.size <= chunk:
        fill(0, t.size)
    else:
        with ThreadPoolExecutor(max_workers=min(32, os.cpu_count() or 1)) as ex:
            list(ex.map(lambda lo: fill(lo, min(t.size, lo + chunk)), range(0, t.size, chunk)))
    return out


class SchrodingerSimulation(QuantumAlgorithm):
    """SchrodingerSimulation(N, dt, dx, nrSteps, addSeed) with the reference's setters and initial states"""

    def __init__(self, N: int = 8, dt: float = 0.1, dx: float = 0.1, nrSteps: int = 50, addSeed: bool = False, *,
                 precision: str = "fp64"):
        super().__init__(N, int(addSeed), precision=precision)
        self.deltat = dt
        self.steps = nrSteps
        self.deltax = dx
        self.potential = np.zeros(self.getNrBasisStates())
        self.setToBasisState(0)

    def Execute(self) -> int:
        potential_op, kinetic_op = self.Init()
        self.reg._ck(self.reg._lib.qcs_schrodinger_evolve(self.reg.handle, potential_op.view(np.float64).ctypes.data_as(C.POINTER(C.c_double)),
                                                          kinetic_op.view(np.float64).ctypes.data_as(C.POINTER(C.c_double)), self.steps))
        return 0

    def getPotential(self, pos: int) -> float:
        return float(self.potential[pos]) if 0 <= pos < self.potential.size else 0.0

    def setPotential(self, pos: int, val: float) -> None:
        if 0 <= pos < self.potential.size:
            self.potential[pos] = val

    def getDeltax(self) -> float:
        return self.deltax

    def setDeltax(self, v: float) -> None:
        self.deltax = v

    def setSimulationTimeInterval(self, dt: float) -> None:
        self.deltat = dt

    def setNrSteps(self, nrSteps: int) -> None:
        self.steps = nrSteps

    def setConstantPotentialInTheMiddle(self, val: float, halfwidth: int) -> None:
        """a square barrier (val > 0) or well in the middle, walls at both ends (Schrodinger.h:76-88)"""
        n = self.getNrBasisStates()
        half = n // 2
        lo, hi = max(1, half - halfwidth), min(n - 1, half + halfwidth)
        if lo < hi:
            self.potential[lo:hi] = val
        self.setPotential(0, 1e150)
        self.setPotential(n - 1, 1e150)

    def setConstantPotentialToRight(self, val: float) -> None:
        """a step from the middle on, walls at both ends (Schrodinger.h:91-102)"""
        n = self.getNrBasisStates()
        self.potential[n // 2:] = val
        self.setPotential(0, 1e15)
        self.setPotential(n - 1, 1e150)

    def setGaussian(self, pos: int, stdev: float, k: float) -> None:
        """a normalised Gaussian wave packet centred on grid point pos, moving with wave number k; the end
        points stay zero (Schrodinger.h:106-136)"""
        n = self.getNrBasisStates()
        stdev *= self.deltax
        a = 1.0 / (stdev * math.sqrt(2.0 * math.pi))
        half_x = 0.5 * self.deltax * (n - 1.0)
        m = self.deltax * pos - half_x
        v = np.zeros(n, dtype=np.complex128)
        x = self.deltax * np.arange(1, n - 1) - half_x
        e = (x - m) / stdev
        g = np.exp(-0.5 * e * e)
        v[1:n - 1] = a * (g * np.cos(k * x) + 1j * (g * np.sin(k * x)))
        self.reg.setRegisterStorageFastNoNormalize(v)
        self.Normalize()

    def Init(self) -> tuple[np.ndarray, np.ndarray]:
        """normalise the start state; the potential and kinetic operators' diagonals, exp(-i V(x_i) dt) and
        exp(-i x_i^2 dt / 2) with x_i = dx i - dx (2^N - 1) / 2 (Schrodinger.h:291-315)"""
        self.Normalize()
        n = self.getNrBasisStates()
        half_x = 0.5 * self.deltax * (n - 1.0)
        x = self.deltax * np.arange(n) - half_x
        return _polar(-self.potential * self.deltat), _polar(-0.5 * x * x * self.deltat)

    def close(self) -> None:
        self.reg.close()
