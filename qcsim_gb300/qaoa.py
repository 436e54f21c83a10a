"""Batched QAOA over the engine (qcs_qaoa_batch_* in include/qcs_gpu.h): many Ising instances of
different sizes, all statevectors resident on the GPU, every layer in one persistent launch replayed
from a CUDA graph.  The circuit per instance is QAOAIsingSubalgorithm::Exec (IsingModel.h:557-567);
<H> is the exact expectation sum_x |psi_x|^2 E(x) (the reference estimates it from 100000 samples,
IsingModel.h:569-578)."""
from __future__ import annotations

import ctypes as C
import json
import time
from pathlib import Path

import numpy as np

from . import _lib as L

CLUSTER_SIZES = (1, 2, 4, 8)  # CTAs per thread-block cluster (portable sizes)
TILE_SHAPES = ((6, 6), (5, 7), (4, 8))  # mixer-pass tiles: (low contiguous qubits, high qubits per pass)


class QaoaBatch:
    def __init__(self, instances: list[dict], p: int, precision: str = "fp64"):
        self._lib = L.load()
        self.instances = instances
        self.p = p
        self._keep = []
        arr = (L.qcs_qaoa_instance * len(instances))()
        for i, inst in enumerate(instances):
            e = np.ascontiguousarray(np.array(inst["edges"], dtype=np.uint32).reshape(-1))
            J = np.ascontiguousarray(inst["J"], dtype=np.float64)
            h = np.ascontiguousarray(inst["h"], dtype=np.float64)
            self._keep += [e, J, h]
            arr[i].n = inst["n"]
            arr[i].nedges = len(inst["edges"])
            arr[i].edges = e.ctypes.data_as(C.POINTER(C.c_uint32))
            arr[i].J = J.ctypes.data_as(C.POINTER(C.c_double))
            arr[i].h = h.ctypes.data_as(C.POINTER(C.c_double))
        self._h = C.c_void_p()
        self.precision = precision
        self.cluster = 0
        self.tile = (6, 6)
        prec = L.QCS_FP64 if precision == "fp64" else L.QCS_FP32
        L.check(self._lib.qcs_qaoa_batch_create(C.cast(arr, C.c_void_p), len(instances), p, prec, C.byref(self._h)))
        self.set_angles(np.array([inst["gammas"] for inst in instances]), np.array([inst["betas"] for inst in instances]))

    def _ck(self, st: int) -> None:
        if st != L.QCS_OK:
            raise L.QcsError(st, self._lib.qcs_qaoa_batch_last_error(self._h).decode())

    def set_angles(self, gammas: np.ndarray, betas: np.ndarray) -> None:
        g = np.ascontiguousarray(gammas, dtype=np.float64)
        b = np.ascontiguousarray(betas, dtype=np.float64)
        self._ck(self._lib.qcs_qaoa_batch_set_angles(self._h, L.dptr(g), L.dptr(b)))

    def set_cluster(self, ctas: int) -> None:
        self._ck(self._lib.qcs_qaoa_batch_set_cluster(self._h, ctas))
        self.cluster = ctas

    def set_tile(self, low: int, high: int) -> None:
        """tile shape of the mixer passes: 2^low contiguous amplitudes times `high` further qubits"""
        self._ck(self._lib.qcs_qaoa_batch_set_tile(self._h, low, high))
        self.tile = (low, high)

    def shape_key(self, precision: str | None = None) -> str:
        """what the schedule depends on: precision, layer count and the instance-size histogram"""
        sizes: dict[int, int] = {}
        for inst in self.instances:
            sizes[inst["n"]] = sizes.get(inst["n"], 0) + 1
        hist = ",".join(f"{n}:{c}" for n, c in sorted(sizes.items()))
        return f"{precision or self.precision}|p{self.p}|{hist}"

    def autotune(self, candidates=CLUSTER_SIZES, shapes=TILE_SHAPES, reps: int = 2, cache: Path | None = None) -> dict:
        """choose the schedule (cluster size: CTAs sharing one instance's tiles) and the mixer-pass tile
        shape by timing one launch of every combination after a warm-up launch; keep the fastest and
        return {"cluster,low,high": seconds}.  With `cache` (a JSON file), a choice recorded for the
        same shape key is reused without timing."""
        key = self.shape_key()
        table = {}
        if cache is not None and Path(cache).exists():
            table = json.loads(Path(cache).read_text())
            if key in table:
                self.set_tile(*table[key]["tile"])
                self.set_cluster(int(table[key]["cluster"]))
                return dict(table[key]["seconds"])
        times = {}
        for low, high in shapes:
            self.set_tile(low, high)
            for cl in candidates:
                self.set_cluster(cl)
                self.run()  # graph capture and warm-up
                best = float("inf")
                for _ in range(reps):
                    t0 = time.perf_counter()
                    self.run()
                    best = min(best, time.perf_counter() - t0)
                times[f"{cl},{low},{high}"] = best
        choice = min(times, key=times.get)
        cl, low, high = (int(x) for x in choice.split(","))
        self.set_tile(low, high)
        self.set_cluster(cl)
        if cache is not None:
            table[key] = {"cluster": cl, "tile": [low, high], "seconds": times}
            Path(cache).write_text(json.dumps(table, indent=1))
        return times

    def run(self) -> np.ndarray:
        out = np.empty(len(self.instances), dtype=np.float64)
        self._ck(self._lib.qcs_qaoa_batch_run(self._h, L.dptr(out)))
        return out

    def state(self, i: int) -> np.ndarray:
        out = np.empty(1 << self.instances[i]["n"], dtype=np.complex128)
        self._ck(self._lib.qcs_qaoa_batch_state(self._h, i, out.view(np.float64).ctypes.data_as(C.POINTER(C.c_double))))
        return out

    @property
    def amplitudes(self) -> int:
        return int(self._lib.qcs_qaoa_batch_amplitudes(self._h))

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.qcs_qaoa_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
