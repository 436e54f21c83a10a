"""Generate tests/golden/algorithms.npz from QCSim's own Grover search, Draper adders and phase estimation (the
compiled reference).

Run in a checkout that has the QCSim sources (oracle/Makefile target `ref` builds oracle/_ref/libqcsref.so from them):

    make -C oracle ref && python tests/golden/make_algorithms.py

Each case is the state after the class's ExecuteWithoutMeasurement (GroverAlgorithm.h:89-98, DraperAdder.h:38-57 and
:88-112, PhaseEstimation.h:195-215): Grover from its equal superposition with the given marked state; the adders from
a random normalised superposition of inputs; phase estimation of a random unitary on the function register; VQE's
PauliStringVQE Ansatz followed by Execute (VQE.h:33-114) from |0> with random parameters and operators; Shor's
period finding, ShorPhaseEstimation of Shor::Fx (PhaseEstimation.h:100-149, ShorAlgorithm.h:54-104); and quantum
counting's pre-measurement state (QuantumCountingAlgorithm.h:104-128), read after its non-collapsing sampling.
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import bind as B  # noqa: E402

OUT = Path(__file__).resolve().parent / "algorithms.npz"

GROVER = [(3, 5), (5, 17), (7, 100), (9, 300)]  # (qubits, marked state)
DRAPER = [(2, 0), (3, 0), (4, 0), (2, 1), (3, 1), (4, 1)]  # (N, with carry)
PHASE = [(1, 4, 3), (2, 7, 5), (3, 8, 5)]  # (operator qubits k, register qubits N, precision qubits L), k = N - L
VQE = [(1, 2), (2, 4), (3, 9), (4, 14), (5, 30)]  # (qubits, parameters): the ansatz's single layer and CNOT-ring layers
# (C, a, register qubits N, x qubits L); a^(2^(L-1)) must fit in 64 bits, since Fx squares in 64-bit arithmetic and
# asserts that each modular multiplier is unitary (ShorAlgorithm.h:62-101)
SHOR = [(15, 7, 7, 3), (15, 2, 7, 3), (15, 11, 7, 3), (21, 2, 11, 6)]
COUNTING = [(3, 1, [5]), (4, 2, [0, 3]), (5, 3, [1, 2, 6, 7]), (6, 4, [0, 4, 9, 13, 15])]  # (P, G, marked states)


def pd(a: np.ndarray):
    return a.view(np.float64).ctypes.data_as(C.POINTER(C.c_double))


def unit(rng, n: int) -> np.ndarray:
    v = rng.standard_normal(1 << n) + 1j * rng.standard_normal(1 << n)
    return np.ascontiguousarray(v / np.linalg.norm(v))


def generate(lib=None, max_shor_qubits: int = 64) -> dict[str, np.ndarray]:
    """every fixture array, produced through ref_driver.cpp's entry points in `lib` (default: the
    compiled reference, B.ref(); B.ref_dropin() runs the same driver over the GPU drop-in register).
    Shor cases on more than max_shor_qubits register qubits are left out: Fx builds its 2^N x 2^N
    modular-multiplication operators as dense host matrices (the 11-qubit case spends about two minutes
    in host matrix products, whichever register runs it)."""
    lib = lib if lib is not None else B.ref()
    rng = np.random.default_rng(20261207)
    out = {"grover": np.array(GROVER, dtype=np.int64), "draper": np.array(DRAPER, dtype=np.int64),
           "phase": np.array(PHASE, dtype=np.int64), "vqe": np.array(VQE, dtype=np.int64),
           "shor": np.array(SHOR, dtype=np.int64), "counting": np.array([c[:2] for c in COUNTING], dtype=np.int64)}
    for i, (n, marked) in enumerate(GROVER):
        res = np.zeros(1 << n, dtype=np.complex128)
        assert lib.qr_grover(n, marked, pd(res)) == 0
        out[f"grover{i}"] = res
    for i, (N, carry) in enumerate(DRAPER):
        psi = unit(rng, 2 * N + carry)
        res = np.zeros_like(psi)
        assert lib.qr_draper(N, carry, pd(psi), pd(res)) == 0
        out[f"draper_in{i}"], out[f"draper{i}"] = psi, res
    for i, (k, N, L) in enumerate(PHASE):
        d = 1 << k
        u, _ = np.linalg.qr(rng.standard_normal((d, d)) + 1j * rng.standard_normal((d, d)))
        u = np.ascontiguousarray(u)
        psi = unit(rng, N)
        res = np.zeros_like(psi)
        assert lib.qr_phase_estimation(pd(u), k, N, L, pd(psi), pd(res)) == 0
        out[f"phase_u{i}"], out[f"phase_in{i}"], out[f"phase{i}"] = u, psi, res
    for i, (n, npar) in enumerate(VQE):
        ops = np.ascontiguousarray(rng.integers(0, 3, n).astype(np.uint8))
        params = np.ascontiguousarray(rng.uniform(-np.pi, np.pi, npar))
        res = np.zeros(1 << n, dtype=np.complex128)
        assert lib.qr_vqe_term(n, ops.ctypes.data_as(C.c_void_p), npar, params.ctypes.data_as(C.POINTER(C.c_double)),
                               pd(res)) == 0
        out[f"vqe_ops{i}"], out[f"vqe_params{i}"], out[f"vqe{i}"] = ops, params, res
    for i, (c, a, n, L) in enumerate(SHOR):
        if n > max_shor_qubits:
            continue
        res = np.zeros(1 << n, dtype=np.complex128)
        assert lib.qr_shor_period_finding(c, a, n, L, pd(res)) == 0
        out[f"shor{i}"] = res
    for i, (P, Gq, marked) in enumerate(COUNTING):
        mk = np.ascontiguousarray(marked, dtype=np.uint64)
        res = np.zeros(1 << (P + 2 * Gq), dtype=np.complex128)
        assert lib.qr_counting(P, Gq, len(marked), mk.ctypes.data_as(C.c_void_p), pd(res)) == 0
        out[f"counting_marked{i}"], out[f"counting{i}"] = mk, res
    return out


def main() -> None:
    np.savez_compressed(OUT, **generate())
    print("wrote", OUT, OUT.stat().st_size, "bytes")


if __name__ == "__main__":
    main()
