"""Generate tests/golden/oracles.npz from QCSim's own gate-built oracles (the compiled reference).

Run in a checkout that has the QCSim sources (oracle/Makefile target `ref` builds oracle/_ref/libqcsref.so from them):

    make -C oracle ref && python tests/golden/make_oracles.py

Each case runs QC::Oracles::OracleWithGatesSimpleFunction (simple = 1) or OracleWithGates (simple = 0) from Oracle.h,
with the function given as a table over the input qubits [start, end], on a random normalised n-qubit state; the
qubit layouts are those of the Deutsch-Jozsa, Bernstein-Vazirani and Simon algorithms with gate-built oracles.  The
fixture holds the inputs and the reference's state after Execute.
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import bind as B  # noqa: E402

OUT = Path(__file__).resolve().parent / "oracles.npz"

# (n, start, end, target, first ancilla, simple, kind of table)
CASES = [
    (3, 0, 0, 1, 2, 1, "bool"),     # one control
    (5, 0, 2, 3, 4, 1, "parity"),   # Bernstein-Vazirani, N = 3
    (7, 0, 3, 4, 5, 1, "bool"),     # Bernstein-Vazirani layout, N = 4, random function
    (5, 0, 2, 3, 4, 1, "balanced"),  # Deutsch-Jozsa, N = 4
    (5, 0, 1, 2, 4, 0, "simon"),    # Simon, N = 2
    (8, 0, 2, 3, 6, 0, "simon"),    # Simon, N = 3
    (11, 0, 3, 4, 8, 0, "simon"),   # Simon, N = 4
]


def table(kind: str, nin: int, nout: int, rng) -> np.ndarray:
    size = 1 << nin
    if kind == "parity":
        s = int(rng.integers(1, size))
        return np.array([bin(x & s).count("1") & 1 for x in range(size)], dtype=np.uint64)
    if kind == "balanced":
        v = np.zeros(size, dtype=np.uint64)
        v[: size // 2] = 1
        return rng.permutation(v)
    if kind == "bool":
        return rng.integers(0, 2, size).astype(np.uint64)
    return rng.integers(0, 1 << nout, size).astype(np.uint64)


def generate(lib=None) -> dict[str, np.ndarray]:
    """every fixture array, produced through ref_driver.cpp's entry points in `lib` (default: the
    compiled reference, B.ref(); B.ref_dropin() runs the same driver over the GPU drop-in register)"""
    lib = lib if lib is not None else B.ref()
    rng = np.random.default_rng(20261206)
    out = {"cases": np.array([c[:6] for c in CASES], dtype=np.int64)}
    for i, (n, start, end, target, anc, simple, kind) in enumerate(CASES):
        nin = end - start + 1
        t = np.ascontiguousarray(table(kind, nin, nin, rng))
        psi = rng.standard_normal(1 << n) + 1j * rng.standard_normal(1 << n)
        psi = np.ascontiguousarray(psi / np.linalg.norm(psi))
        res = psi.copy()
        assert lib.qr_oracle_with_gates(n, start, end, target, anc, simple, t.ctypes.data_as(C.c_void_p),
                                        res.view(np.float64).ctypes.data_as(C.POINTER(C.c_double))) == 0
        out[f"table{i}"], out[f"psi{i}"], out[f"out{i}"] = t, psi, res
    return out


def main() -> None:
    np.savez_compressed(OUT, **generate())
    print("wrote", OUT, OUT.stat().st_size, "bytes")


if __name__ == "__main__":
    main()
