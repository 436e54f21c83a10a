"""ctypes binding of the CPU oracle (libqcs_oracle.so) and of the compiled reference
(oracle/_ref/libqcsref.so) -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this module, as the checker
or the timed CPU baseline.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ORACLE_LIB = HERE / "libqcs_oracle.so"
REF_LIB = HERE / "_ref" / "libqcsref.so"
# QCSim's sources as staged by `make -C oracle stage` (git-ignored, travels with the working tree)
STAGED_SRC = HERE / "_ref" / "src"
# ref_driver.cpp compiled against the GPU drop-in register, and QCSim's test suite on the drop-in
DROPIN_LIB = HERE / "_ref" / "libqcsref_dropin.so"
SUITE_BIN = HERE / "_ref" / "qcsim_tests_dropin"
GPU_LIB = HERE.parent / "qcsim_gb300" / "libqcs_gpu.so"

# qo_gate (oracle/qcs_oracle.h)
QO_GATE = np.dtype([("code", "<i4"), ("q0", "<i4"), ("q1", "<i4"), ("q2", "<i4"), ("p", "<f8", (4,)),
                    ("m", "<f8", (128,))])

_h, _u32, _u64, _d, _sz, _i = C.c_void_p, C.c_uint32, C.c_uint64, C.c_double, C.c_size_t, C.c_int
_pd = C.POINTER(C.c_double)
_pu64 = C.POINTER(C.c_uint64)
_pu32 = C.POINTER(C.c_uint32)

_ORACLE_SIG = {
    "qo_gate_matrix": (_i, [C.c_int32, _pd, _pd, _pd, _pu32, _pu32]),
    "qo_create": (_h, [_u32]), "qo_destroy": (None, [_h]), "qo_set_multithreading": (None, [_h, _i]),
    "qo_set_threads": (None, [_i]), "qo_max_threads": (_i, []),
    "qo_apply": (_i, [_h, C.c_void_p, _sz]), "qo_last_error": (C.c_char_p, [_h]),
    "qo_get_state": (None, [_h, _pd]), "qo_set_state": (None, [_h, _pd]), "qo_nstates": (_u64, [_h]),
    "qo_set_basis": (None, [_h, _u64]), "qo_set_qubit_state": (None, [_h, _u64]), "qo_set_cat": (None, [_h]),
    "qo_set_equal": (None, [_h]), "qo_clear": (None, [_h]), "qo_set_raw": (None, [_h, _u64, _d, _d]),
    "qo_normalize": (None, [_h]), "qo_adjust_phase_normalize": (None, [_h]),
    "qo_measure_all": (_u64, [_h, _d]), "qo_measure": (_u64, [_h, _u32, _u32, _d]),
    "qo_measure_no_collapse": (_u64, [_h, _d]), "qo_measure_no_collapse_sub": (_u64, [_h, _u32, _u32, _d]),
    "qo_sample": (None, [_h, _pd, _sz, _pu64]), "qo_qubit_probability": (_d, [_h, _u32]),
    "qo_fidelity": (_d, [_h, _pd]), "qo_inner": (None, [_h, _pd, _pd, _pd]),
    "qo_qft": (_i, [_h, _u32, _u32, _i, _i]),
    "qo_qaoa_exec": (_i, [_h, _u32, _pu32, _pd, _pd, _u32, _pd, _pd]),
    "qo_ising_energy": (_d, [_u32, _u32, _pu32, _pd, _pd, _u64]),
    "qo_expected_energy": (_d, [_h, _u32, _pu32, _pd, _pd]),
    "qo_rng_create": (_h, [_u64]), "qo_rng_destroy": (None, [_h]), "qo_rng_next": (_u64, [_h]),
    "qo_rng_uniform": (_d, [_h]),
    "qo_random_normal_state": (None, [_u64, _u32, _pd]), "qo_max_abs_diff": (_d, [_pd, _pd, _u64]),
}

_REF_SIG = {
    "qr_create": (_h, [_u32, _u64]), "qr_destroy": (None, [_h]), "qr_seed": (None, [_h, _u64]),
    "qr_set_multithreading": (None, [_h, _i]),
    "qr_gate_matrix": (_i, [C.c_void_p, _pd, _pu32, _pu32]),
    "qr_apply": (_i, [_h, C.c_void_p, _sz]), "qr_last_error": (C.c_char_p, [_h]),
    "qr_get_state": (None, [_h, _pd]), "qr_set_state": (None, [_h, _pd]),
    "qr_measure_all": (_u64, [_h]), "qr_measure": (_u64, [_h, _u32, _u32]), "qr_measure_qubit": (_u64, [_h, _u32]),
    "qr_measure_no_collapse": (_u64, [_h]), "qr_measure_no_collapse_sub": (_u64, [_h, _u32, _u32]),
    "qr_repeated_measure": (_sz, [_h, _sz, _pu64, _pu64]),
    "qr_repeated_measure_sub": (_sz, [_h, _u32, _u32, _sz, _pu64, _pu64]),
    "qr_qubit_probability": (_d, [_h, _u32]), "qr_normalize": (None, [_h]),
    "qr_adjust_phase_normalize": (None, [_h]), "qr_set_basis": (None, [_h, _u64]), "qr_set_equal": (None, [_h]),
    "qr_set_cat": (None, [_h]), "qr_set_raw": (None, [_h, _u64, _d, _d]), "qr_fidelity": (_d, [_h, _pd]),
    "qr_expectation": (None, [_h, C.c_void_p, _sz, _pd, _pd]),
    "qr_record_and_replay": (_i, [_h, C.c_void_p, _sz, _i]),
    "qr_qft": (_i, [_h, _u32, _u32, _u32, _i, _i]),
    "qr_qaoa_exec": (_i, [_h, _u32, _u32, _pu32, _pd, _pd, _u32, _pd, _pd]),
    "qr_ising_energy": (_d, [_u32, _u32, _pu32, _pd, _pd, _u64]),
    "qr_uniforms": (None, [_u64, _sz, _pd]),
    "qr_nqubits_gate": (_i, [_h, _u32, _pd, _u32, _u32, _i, _pd]),
    "qr_pauli_simulation": (_i, [_u32, _pd, _u32, C.c_void_p, _pd, _d, _u32, _pd]),
    "qr_oracle_with_gates": (_i, [_u32, _u32, _u32, _u32, _u32, _i, C.c_void_p, _pd]),
    "qr_grover": (_i, [_u32, _u64, _pd]),
    "qr_draper": (_i, [_u32, _i, _pd, _pd]),
    "qr_phase_estimation": (_i, [_pd, _u32, _u32, _u32, _pd, _pd]),
    "qr_vqe_term": (_i, [_u32, C.c_void_p, _u32, _pd, _pd]),
    "qr_shor_period_finding": (_i, [_u32, _u32, _u32, _u32, _pd]),
    "qr_counting": (_i, [_u32, _u32, _u32, C.c_void_p, _pd]),
}

_oracle = None
_ref = None


def qcsim_source() -> Path | None:
    """the QCSim source directory named by the QCSIM_SRC environment variable, if it exists"""
    s = os.environ.get("QCSIM_SRC")
    return Path(s) if s and Path(s).is_dir() else None


def build_oracle(ref: bool = False, dropin: bool = False) -> None:
    """compile oracle/libqcs_oracle.so; with ref, also QCSim's own register (_ref/libqcsref.so); with
    dropin, also ref_driver.cpp and QCSim's test suite over the GPU drop-in (needs libqcs_gpu.so).  The
    QCSim sources are staged into _ref/src first when QCSIM_SRC names a checkout; the _ref targets are
    built only where a staged copy exists."""
    src = qcsim_source()
    if (ref or dropin) and src is not None:
        subprocess.run(["make", "-s", "-C", str(HERE), "stage", f"QCSIM_SRC={src}"], check=True)
    targets = ["all"]
    if STAGED_SRC.is_dir():
        targets += ["ref"] if ref else []
        targets += ["dropin"] if dropin and GPU_LIB.exists() else []
    jobs = str(min(16, os.cpu_count() or 1))
    subprocess.run(["make", "-s", f"-j{jobs}", "-C", str(HERE), *targets], check=True)


def _bind(path: Path, sig: dict):
    lib = C.CDLL(str(path))
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


def oracle():
    global _oracle
    if _oracle is None:
        if not ORACLE_LIB.exists():
            build_oracle()
        _oracle = _bind(ORACLE_LIB, _ORACLE_SIG)
    return _oracle


def ref_available() -> bool:
    return REF_LIB.exists()


def ref():
    global _ref
    if _ref is None:
        _ref = _bind(REF_LIB, _REF_SIG)
    return _ref


_ref_dropin = None


def dropin_available() -> bool:
    return DROPIN_LIB.exists()


def ref_dropin():
    """ref_driver.cpp's entry points over the GPU drop-in register: QCSim's own gate classes, algorithms
    and sub-algorithms, unmodified, with every QC::QubitRegister backed by libqcs_gpu.so"""
    global _ref_dropin
    if _ref_dropin is None:
        _ref_dropin = _bind(DROPIN_LIB, _REF_SIG)
    return _ref_dropin


def dp(a: np.ndarray):
    return a.ctypes.data_as(_pd)


def records(ops) -> np.ndarray:
    """qo_gate records from (gate, q0, q1, q2) tuples of qcsim_gb300.gates objects: code + parameters,
    plus the matrix for matrix-only gates"""
    arr = np.zeros(len(ops), dtype=QO_GATE)
    for i, op in enumerate(ops):
        gate, qs = op[0], list(op[1:]) + [0, 0]
        arr[i]["code"] = gate.code
        arr[i]["q0"], arr[i]["q1"], arr[i]["q2"] = qs[0], qs[1], qs[2]
        arr[i]["p"][:] = gate.params()
        if gate.code >= 50:
            m = np.ascontiguousarray(gate.getRawOperatorMatrix(), dtype=np.complex128).reshape(-1).view(np.float64)
            arr[i]["m"][: m.size] = m
    return arr


class OracleRegister:
    """the CPU oracle's register"""

    def __init__(self, n: int, multithreading: bool = True):
        self.lib = oracle()
        self.n = n
        self.N = 1 << n
        self.h = self.lib.qo_create(n)
        self.lib.qo_set_multithreading(self.h, int(multithreading))

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.qo_destroy(self.h)
            self.h = None

    def apply(self, ops) -> None:
        recs = records(ops) if not isinstance(ops, np.ndarray) else ops
        if self.lib.qo_apply(self.h, recs.ctypes.data_as(C.c_void_p), len(recs)):
            raise ValueError(self.lib.qo_last_error(self.h).decode())

    def state(self) -> np.ndarray:
        out = np.empty(self.N, dtype=np.complex128)
        self.lib.qo_get_state(self.h, dp(out.view(np.float64)))
        return out

    def set_state(self, v: np.ndarray) -> None:
        v = np.ascontiguousarray(v, dtype=np.complex128)
        self.lib.qo_set_state(self.h, dp(v.view(np.float64)))

    def sample(self, probs: np.ndarray) -> np.ndarray:
        probs = np.ascontiguousarray(probs, dtype=np.float64)
        out = np.empty(len(probs), dtype=np.uint64)
        self.lib.qo_sample(self.h, dp(probs), len(probs), out.ctypes.data_as(_pu64))
        return out


class RefRegister:
    """QCSim's own QubitRegister through ref_driver.cpp, seeded: the compiled reference (ref()), or the
    same driver over the GPU drop-in register (ref_dropin())"""

    def __init__(self, n: int, seed: int = 1, lib=None):
        self.lib = lib if lib is not None else ref()
        self.n = n
        self.N = 1 << n
        self.h = self.lib.qr_create(n, seed)

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.qr_destroy(self.h)
            self.h = None

    def apply(self, ops) -> None:
        recs = records(ops) if not isinstance(ops, np.ndarray) else ops
        if self.lib.qr_apply(self.h, recs.ctypes.data_as(C.c_void_p), len(recs)):
            raise ValueError(self.lib.qr_last_error(self.h).decode())

    def state(self) -> np.ndarray:
        out = np.empty(self.N, dtype=np.complex128)
        self.lib.qr_get_state(self.h, dp(out.view(np.float64)))
        return out

    def set_state(self, v: np.ndarray) -> None:
        v = np.ascontiguousarray(v, dtype=np.complex128)
        self.lib.qr_set_state(self.h, dp(v.view(np.float64)))

    def repeated_measure(self, shots: int, first=None, second=None) -> dict:
        st = np.empty(max(shots, 1), dtype=np.uint64)
        ct = np.empty(max(shots, 1), dtype=np.uint64)
        if first is None:
            k = self.lib.qr_repeated_measure(self.h, shots, st.ctypes.data_as(_pu64), ct.ctypes.data_as(_pu64))
        else:
            k = self.lib.qr_repeated_measure_sub(self.h, first, second, shots, st.ctypes.data_as(_pu64),
                                                 ct.ctypes.data_as(_pu64))
        return {int(a): int(b) for a, b in zip(st[:k], ct[:k])}
