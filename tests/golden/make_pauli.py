"""Generate tests/golden/pauli.npz from QCSim's own Pauli-Hamiltonian simulation (the compiled reference).

Run in a checkout that has the QCSim sources (oracle/Makefile target `ref` builds oracle/_ref/libqcsref.so from them):

    make -C oracle ref && python tests/golden/make_pauli.py

Each case is QuantumSimulation::PauliDecomposedHamiltonianSimulation (PauliStringSimulation.h:105-219) on n qubits from
a random normalised state, with random Pauli-string terms (codes 0 = Z, 1 = X, 2 = Y per qubit) and coefficients, run
through Execute for the given time and Trotter steps; the fixture holds the inputs and the reference's final state.
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import bind as B  # noqa: E402

OUT = Path(__file__).resolve().parent / "pauli.npz"

# (n, number of terms, simulation time, steps)
CASES = [(3, 1, 0.159, 100), (3, 5, 0.159, 100), (4, 3, 0.5, 20), (5, 4, 0.3, 7), (6, 6, 0.2, 3)]


def pd(a: np.ndarray):
    return a.view(np.float64).ctypes.data_as(C.POINTER(C.c_double))


def generate(lib=None) -> dict[str, np.ndarray]:
    """every fixture array, produced through ref_driver.cpp's entry points in `lib` (default: the
    compiled reference, B.ref(); B.ref_dropin() runs the same driver over the GPU drop-in register)"""
    lib = lib if lib is not None else B.ref()
    rng = np.random.default_rng(20261205)
    out = {"cases": np.array([c[:2] for c in CASES], dtype=np.int64), "times": np.array([c[2] for c in CASES]),
           "steps": np.array([c[3] for c in CASES], dtype=np.int64)}
    for i, (n, nt, t, steps) in enumerate(CASES):
        psi = rng.standard_normal(1 << n) + 1j * rng.standard_normal(1 << n)
        psi = np.ascontiguousarray(psi / np.linalg.norm(psi))
        ops = np.ascontiguousarray(rng.integers(0, 3, (nt, n)).astype(np.uint8))
        coeffs = np.ascontiguousarray(-rng.uniform(0.1, 10.0, nt))
        res = np.zeros(1 << n, dtype=np.complex128)
        st = lib.qr_pauli_simulation(n, pd(psi), nt, ops.ctypes.data_as(C.c_void_p), coeffs.ctypes.data_as(C.POINTER(C.c_double)),
                                     t, steps, pd(res))
        assert st == 0
        out[f"psi{i}"], out[f"ops{i}"], out[f"coeffs{i}"], out[f"out{i}"] = psi, ops, coeffs, res
    return out


def main() -> None:
    np.savez_compressed(OUT, **generate())
    print("wrote", OUT, OUT.stat().st_size, "bytes")


if __name__ == "__main__":
    main()
