"""Generate tests/golden/nqubits.npz from QCSim's own dense operator gates (the compiled reference).

Run in a checkout that has the QCSim sources (oracle/Makefile target `ref` builds
oracle/_ref/libqcsref.so from them):

    make -C oracle ref && python tests/golden/make_nqubits.py

Each case is SubAlgo::NQubitsQuantumGate or NQubitsControlledQuantumGate (controlling qubit ctrl >= 0)
of a random complex 2^k x 2^k operator placed at startQubit with startQubit + k = n, the placement whose
extended matrix the reference builds within the operator's bounds: the extended matrix
(getOperatorMatrix, for n <= 6) and the state after Execute on a register holding a random input state.
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import bind as B  # noqa: E402

OUT = Path(__file__).resolve().parent / "nqubits.npz"

# (n, k, ctrl); startQubit = n - k
CASES = [(3, 3, -1), (4, 1, -1), (5, 2, -1), (6, 3, 0), (6, 2, 1), (6, 4, 1), (7, 5, 0), (8, 6, 1)]


def pd(a: np.ndarray):
    return a.view(np.float64).ctypes.data_as(C.POINTER(C.c_double))


def generate(lib=None) -> dict[str, np.ndarray]:
    """every fixture array, produced through ref_driver.cpp's entry points in `lib` (default: the
    compiled reference, B.ref(); B.ref_dropin() runs the same driver over the GPU drop-in register)"""
    lib = lib if lib is not None else B.ref()
    rng = np.random.default_rng(20261204)
    out = {"cases": np.array(CASES, dtype=np.int64)}
    for i, (n, k, ctrl) in enumerate(CASES):
        d, nb = 1 << k, 1 << n
        op = np.ascontiguousarray((rng.standard_normal((d, d)) + 1j * rng.standard_normal((d, d))) / np.sqrt(d))
        psi = np.ascontiguousarray(rng.standard_normal(nb) + 1j * rng.standard_normal(nb))
        psi /= np.linalg.norm(psi)
        ext = np.zeros((nb, nb), dtype=np.complex128)
        reg = B.RefRegister(n, lib=lib)
        reg.set_state(psi)
        st = lib.qr_nqubits_gate(reg.h, n, pd(op), k, n - k, ctrl, pd(ext))
        assert st == 0
        out[f"op{i}"] = op
        out[f"psi{i}"] = psi
        if n <= 6:  # the extended matrices of the larger cases stay out of the fixture (size)
            out[f"ext{i}"] = ext
        out[f"out{i}"] = reg.state()
    return out


def main() -> None:
    np.savez_compressed(OUT, **generate())
    print("wrote", OUT, OUT.stat().st_size, "bytes")


if __name__ == "__main__":
    main()
