"""ctypes binding of libqcs_gpu.so (include/qcs_gpu.h).

The engine is the CUDA library; this module only loads it and declares the entry points.  There is
no CPU fallback: importing works without the library (so host-side modules stay usable), but the
first call that needs the engine raises EngineUnavailable when libqcs_gpu.so is missing.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = Path(os.environ.get("QCS_GPU_LIB", PKG / "libqcs_gpu.so"))

QCS_OK, QCS_INVALID_ARGUMENT, QCS_OUT_OF_MEMORY, QCS_CUDA_ERROR, QCS_UNSUPPORTED = range(5)
QCS_FP64, QCS_FP32 = 0, 1
QCS_OPT_PASSES = 1
QCS_OPT_FUSION = 2
QCS_OPT_FUSION_MAX_QUBITS = 3
QCS_OPT_TENSOR_CORES = 4

TRAIT_DIAGONAL = 1
TRAIT_ANTIDIAGONAL = 2
TRAIT_SWAP = 4
TRAIT_ISWAP = 8
TRAIT_ISWAPDAG = 16
TRAIT_CONTROLLED = 32
TRAIT_CONTROLQ1 = 64


class EngineUnavailable(RuntimeError):
    """libqcs_gpu.so is not built or cannot be loaded."""


class QcsError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{message} (status {status})")
        self.status = status


class qcs_gate(C.Structure):
    _fields_ = [("k", C.c_uint32), ("q0", C.c_uint32), ("q1", C.c_uint32), ("q2", C.c_uint32),
                ("traits", C.c_uint32), ("reserved", C.c_uint32), ("m", C.c_double * 128)]


GATE_DTYPE = np.dtype([("k", "<u4"), ("q0", "<u4"), ("q1", "<u4"), ("q2", "<u4"), ("traits", "<u4"),
                       ("reserved", "<u4"), ("m", "<f8", (128,))])
assert GATE_DTYPE.itemsize == C.sizeof(qcs_gate)

_h = C.c_void_p
_u32, _u64, _i, _d, _sz = C.c_uint32, C.c_uint64, C.c_int, C.c_double, C.c_size_t
_pd = C.POINTER(C.c_double)
_pu64 = C.POINTER(C.c_uint64)

# name -> (restype, argtypes): every symbol declared in include/qcs_gpu.h
SIGNATURES = {
    "qcs_create": (_i, [_u32, _i, C.POINTER(_h)]),
    "qcs_destroy": (_i, [_h]),
    "qcs_clone": (_i, [_h, C.POINTER(_h)]),
    "qcs_set_stream": (_i, [_h, C.c_void_p]),
    "qcs_synchronize": (_i, [_h]),
    "qcs_last_error": (C.c_char_p, [_h]),
    "qcs_status_string": (C.c_char_p, [_i]),
    "qcs_nqubits": (_u32, [_h]),
    "qcs_nstates": (_u64, [_h]),
    "qcs_precision_of": (_i, [_h]),
    "qcs_device_state": (C.c_void_p, [_h]),
    "qcs_set_basis": (_i, [_h, _u64]),
    "qcs_set_qubit_state": (_i, [_h, _u64]),
    "qcs_set_cat": (_i, [_h]),
    "qcs_set_equal": (_i, [_h]),
    "qcs_clear": (_i, [_h]),
    "qcs_set_amplitude": (_i, [_h, _u64, _d, _d]),
    "qcs_get_amplitude": (_i, [_h, _u64, _pd]),
    "qcs_get_state": (_i, [_h, _pd]),
    "qcs_set_state": (_i, [_h, _pd]),
    "qcs_normalize": (_i, [_h]),
    "qcs_adjust_phase_normalize": (_i, [_h]),
    "qcs_apply_gate": (_i, [_h, _pd, _u32, _u32, _u32, _u32, _u32]),
    "qcs_apply_gates": (_i, [_h, C.c_void_p, _sz]),
    "qcs_apply_operator_matrix": (_i, [_h, _pd]),
    "qcs_apply_operator_on_qubits": (_i, [_h, _pd, _u32, C.POINTER(_u32), _u64]),
    "qcs_apply_diagonal": (_i, [_h, _pd]),
    "qcs_schrodinger_evolve": (_i, [_h, _pd, _pd, _u64]),
    "qcs_qft": (_i, [_h, _u32, _u32, _i, _i]),
    "qcs_one_qubit_transform": (_i, [_h, _pd, _u32, _u32, _u32]),
    "qcs_measure_all": (_i, [_h, _d, _pu64]),
    "qcs_measure": (_i, [_h, _u32, _u32, _d, _pu64]),
    "qcs_measure_no_collapse": (_i, [_h, _d, _pu64]),
    "qcs_sample": (_i, [_h, _pd, _sz, _pu64]),
    "qcs_qubit_probability": (_i, [_h, _u32, _pd]),
    "qcs_probabilities": (_i, [_h, _pd]),
    "qcs_fidelity_host": (_i, [_h, _pd, _pd]),
    "qcs_inner": (_i, [_h, _h, _pd]),
    "qcs_compare": (_i, [_h, _h, _pd, _pd]),
    "qcs_save_state": (_i, [_h]),
    "qcs_restore_state": (_i, [_h]),
    "qcs_restore_state_destructive": (_i, [_h]),
    "qcs_expectation": (_i, [_h, C.c_void_p, _sz, _pd]),
    "qcs_qaoa_batch_create": (_i, [C.c_void_p, _sz, _u32, _i, C.POINTER(_h)]),
    "qcs_qaoa_batch_set_angles": (_i, [_h, _pd, _pd]),
    "qcs_qaoa_batch_set_cluster": (_i, [_h, _i]),
    "qcs_qaoa_batch_set_tile": (_i, [_h, _i, _i]),
    "qcs_qaoa_batch_run": (_i, [_h, _pd]),
    "qcs_qaoa_batch_state": (_i, [_h, _sz, _pd]),
    "qcs_qaoa_batch_amplitudes": (_u64, [_h]),
    "qcs_qaoa_batch_last_error": (C.c_char_p, [_h]),
    "qcs_qaoa_batch_destroy": (_i, [_h]),
    "qcs_apply_matrix": (_i, [_h, C.POINTER(_u32), _u32, _pd]),
    "qcs_mlp_create": (_i, [_i, _u64, C.POINTER(_h)]),
    "qcs_mlp_destroy": (_i, [_h]),
    "qcs_mlp_num_params": (_i, [_h]),
    "qcs_mlp_get_params": (_i, [_h, C.POINTER(C.c_float)]),
    "qcs_mlp_set_params": (_i, [_h, C.POINTER(C.c_float)]),
    "qcs_mlp_predict": (_i, [_h, C.POINTER(C.c_float), _i, C.POINTER(C.c_float)]),
    "qcs_mlp_gradient": (_i, [_h, C.POINTER(C.c_float), C.POINTER(C.c_float), _i, C.POINTER(C.c_float),
                              C.POINTER(C.c_float)]),
    "qcs_mlp_train": (_i, [_h, C.POINTER(C.c_float), C.POINTER(C.c_float), _i, _i, C.c_float, C.POINTER(C.c_float)]),
    "qcs_block_features": (_i, [_u32, C.POINTER(_u32), _u32, _u32, C.POINTER(C.c_float)]),
    "qcs_set_cost_model": (_i, [_h, _h, _pd, _sz]),
    "qcs_fusion_plan": (_i, [_u32, C.c_void_p, _sz, _i, C.POINTER(C.c_uint64), C.POINTER(_u32), _sz, C.POINTER(_sz)]),
    "qcs_fusion_passes": (_i, [_u32, C.c_void_p, _sz, _i, _i, _i, C.POINTER(_u32), _sz, C.POINTER(_sz), C.POINTER(_sz)]),
    "qcs_plan_gate_passes": (_i, [_u32, _i, C.c_void_p, _sz, C.POINTER(_u32), C.POINTER(_u32), _sz, C.POINTER(_sz)]),
    "qcs_set_option": (_i, [_h, _i, _i]),
    "qcs_profile_enable": (_i, [_h, _i]),
    "qcs_profile_read": (_i, [_h, C.c_void_p, _i, C.POINTER(_i)]),
    "qcs_launch_count": (_u64, []),
    "qcs_scratch_bytes": (_i, [_h, C.POINTER(_u64), C.POINTER(_u64)]),
    "qcs_rng_create": (_i, [_u64, C.POINTER(_h)]),
    "qcs_rng_destroy": (_i, [_h]),
    "qcs_rng_uniform": (_i, [_h, _pd, _sz]),
    "qcs_qubit_probability_noalloc": (_i, [_h, _u32, _pd]),
}



class qcs_qaoa_instance(C.Structure):
    _fields_ = [("n", C.c_uint32), ("nedges", C.c_uint32), ("edges", C.POINTER(C.c_uint32)),
                ("J", C.POINTER(C.c_double)), ("h", C.POINTER(C.c_double))]


class qcs_profile_entry(C.Structure):
    _fields_ = [("name", C.c_char * 48), ("launches", C.c_uint64), ("milliseconds", C.c_double), ("bytes", C.c_double),
                ("fp_ops", C.c_double)]


_lib = None


def load() -> C.CDLL:
    """Load libqcs_gpu.so once; raise EngineUnavailable if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise EngineUnavailable(f"{LIB_PATH} is not built; run `python -m qcsim_gb300.build` "
                                "(or __graft_entry__.build()) on a machine with nvcc")
    try:
        lib = C.CDLL(str(LIB_PATH))
    except OSError as e:  # pragma: no cover - depends on the machine
        raise EngineUnavailable(f"cannot load {LIB_PATH}: {e}") from e
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def dptr(a: np.ndarray):
    return a.ctypes.data_as(_pd)


def u64ptr(a: np.ndarray):
    return a.ctypes.data_as(_pu64)


def check(status: int, handle=None) -> None:
    if status == QCS_OK:
        return
    lib = load()
    msg = lib.qcs_last_error(handle).decode() if handle else lib.qcs_status_string(status).decode()
    if status == QCS_INVALID_ARGUMENT:
        raise ValueError(msg)
    if status == QCS_OUT_OF_MEMORY:
        raise MemoryError(msg)
    raise QcsError(status, msg or lib.qcs_status_string(status).decode())
