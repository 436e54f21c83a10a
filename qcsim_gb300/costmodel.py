"""Learned fusion: an MLP cost model for the FP32 fused path.

The engine records the device time of fused-block applications (one block per shared-memory pass,
minus the time of a pass that moves the same amplitudes), trains a 3-layer MLP (F -> 64 -> 64 -> 1,
ReLU, FP32) on log-times with its own CUDA kernels (forward, backward, Adam), and uses the model to
pick the fusion partition of a gate list (fusion mode 2).  The greedy fuser with blocks of at most
5 qubits is the fallback.

MlpRef is the CPU restatement of the same network used to check the GPU gradients.
"""
from __future__ import annotations

import ctypes as C
import math
from pathlib import Path

import numpy as np

from . import _lib as L

H = 64
F = 13
MODEL_DIR = Path(__file__).resolve().parent / "models"

_pf = C.POINTER(C.c_float)


def fptr(a: np.ndarray):
    return a.ctypes.data_as(_pf)


def features(n: int, qubits, ngates: int) -> np.ndarray:
    """the engine's feature vector of a block (qubits ascending)"""
    lib = L.load()
    q = np.ascontiguousarray(sorted(qubits), dtype=np.uint32)
    out = np.zeros(F, dtype=np.float32)
    L.check(lib.qcs_block_features(n, q.ctypes.data_as(C.POINTER(C.c_uint32)), len(q), ngates, fptr(out)))
    return out


def fusion_plan(n: int, recs: np.ndarray, max_qubits: int) -> list[tuple[int, int]]:
    """(qubit mask, gate count) of each block of the greedy fuser's partition"""
    lib = L.load()
    recs = np.ascontiguousarray(recs, dtype=L.GATE_DTYPE)
    cap = len(recs) + 1
    masks = np.zeros(cap, dtype=np.uint64)
    ng = np.zeros(cap, dtype=np.uint32)
    nb = C.c_size_t()
    L.check(lib.qcs_fusion_plan(n, recs.ctypes.data_as(C.c_void_p), len(recs), max_qubits,
                                masks.ctypes.data_as(C.POINTER(C.c_uint64)), ng.ctypes.data_as(C.POINTER(C.c_uint32)),
                                cap, C.byref(nb)))
    return [(int(masks[i]), int(ng[i])) for i in range(nb.value)]


def fusion_passes(n: int, recs: np.ndarray, max_qubits: int, tile_qubits: int, tensor_cores: bool) -> list[int]:
    """the shared-memory pass of each block of fusion_plan's partition (host only)"""
    lib = L.load()
    recs = np.ascontiguousarray(recs, dtype=L.GATE_DTYPE)
    cap = len(recs) + 1
    pob = np.zeros(cap, dtype=np.uint32)
    nb, npass = C.c_size_t(), C.c_size_t()
    L.check(lib.qcs_fusion_passes(n, recs.ctypes.data_as(C.c_void_p), len(recs), max_qubits, tile_qubits, int(tensor_cores),
                                  pob.ctypes.data_as(C.POINTER(C.c_uint32)), cap, C.byref(nb), C.byref(npass)))
    out = [int(x) for x in pob[:nb.value]]
    assert not out or max(out) + 1 == npass.value
    return out


def gate_passes(n: int, recs: np.ndarray, precision: str = "fp64") -> list[tuple[int, int]]:
    """(operations, TileFactor operations) of each shared-memory pass qcs_apply_gates plans for an unfused
    gate list (host only)"""
    lib = L.load()
    recs = np.ascontiguousarray(recs, dtype=L.GATE_DTYPE)
    cap = len(recs) + 1
    nops = np.zeros(cap, dtype=np.uint32)
    nfac = np.zeros(cap, dtype=np.uint32)
    npass = C.c_size_t()
    L.check(lib.qcs_plan_gate_passes(n, L.QCS_FP64 if precision == "fp64" else L.QCS_FP32, recs.ctypes.data_as(C.c_void_p),
                                     len(recs), nops.ctypes.data_as(C.POINTER(C.c_uint32)),
                                     nfac.ctypes.data_as(C.POINTER(C.c_uint32)), cap, C.byref(npass)))
    return [(int(nops[i]), int(nfac[i])) for i in range(min(cap, npass.value))]


class Mlp:
    """the engine's MLP (qcs_mlp_*)"""

    def __init__(self, inputs: int = F, seed: int = 1):
        self._lib = L.load()
        self.F = inputs
        self._h = C.c_void_p()
        L.check(self._lib.qcs_mlp_create(inputs, seed, C.byref(self._h)))
        self.nparams = int(self._lib.qcs_mlp_num_params(self._h))

    @property
    def handle(self):
        return self._h

    def params(self) -> np.ndarray:
        p = np.empty(self.nparams, dtype=np.float32)
        L.check(self._lib.qcs_mlp_get_params(self._h, fptr(p)))
        return p

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == self.nparams
        L.check(self._lib.qcs_mlp_set_params(self._h, fptr(p)))

    def predict(self, x: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.empty(len(x), dtype=np.float32)
        L.check(self._lib.qcs_mlp_predict(self._h, fptr(x), len(x), fptr(y)))
        return y

    def gradient(self, x: np.ndarray, t: np.ndarray):
        x = np.ascontiguousarray(x, dtype=np.float32)
        t = np.ascontiguousarray(t, dtype=np.float32)
        g = np.empty(self.nparams, dtype=np.float32)
        loss = C.c_float()
        L.check(self._lib.qcs_mlp_gradient(self._h, fptr(x), fptr(t), len(x), fptr(g), C.byref(loss)))
        return g, float(loss.value)

    def train(self, x: np.ndarray, t: np.ndarray, steps: int, lr: float) -> float:
        x = np.ascontiguousarray(x, dtype=np.float32)
        t = np.ascontiguousarray(t, dtype=np.float32)
        loss = C.c_float()
        L.check(self._lib.qcs_mlp_train(self._h, fptr(x), fptr(t), len(x), steps, lr, C.byref(loss)))
        return float(loss.value)

    def close(self):
        if getattr(self, "_h", None):
            self._lib.qcs_mlp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class MlpRef:
    """CPU restatement (float64) of the engine's MLP: same layout and loss"""

    def __init__(self, params: np.ndarray, inputs: int = F):
        p = np.asarray(params, dtype=np.float64)
        self.F = inputs
        o = 0
        self.W1 = p[o:o + H * inputs].reshape(H, inputs); o += H * inputs
        self.b1 = p[o:o + H]; o += H
        self.W2 = p[o:o + H * H].reshape(H, H); o += H * H
        self.b2 = p[o:o + H]; o += H
        self.W3 = p[o:o + H]; o += H
        self.b3 = p[o]

    def forward(self, x):
        self.x = np.asarray(x, dtype=np.float64)
        self.z1 = self.x @ self.W1.T + self.b1
        self.h1 = np.maximum(self.z1, 0)
        self.z2 = self.h1 @ self.W2.T + self.b2
        self.h2 = np.maximum(self.z2, 0)
        return self.h2 @ self.W3 + self.b3

    def loss_and_grad(self, x, t):
        y = self.forward(x)
        B = len(y)
        dy = 2 * (y - t) / B
        gW3 = dy @ self.h2
        gb3 = dy.sum()
        dh2 = np.outer(dy, self.W3) * (self.z2 > 0)
        gW2 = dh2.T @ self.h1
        gb2 = dh2.sum(0)
        dh1 = (dh2 @ self.W2) * (self.z1 > 0)
        gW1 = dh1.T @ self.x
        gb1 = dh1.sum(0)
        g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3, [gb3]])
        return float(np.mean((y - t) ** 2)), g


def random_unitary(k: int, rng: np.random.Generator) -> np.ndarray:
    a = rng.standard_normal((1 << k, 1 << k)) + 1j * rng.standard_normal((1 << k, 1 << k))
    q, r = np.linalg.qr(a)
    return q * (np.diag(r) / np.abs(np.diag(r)))


def apply_matrix(reg, qubits, m) -> None:
    lib = L.load()
    q = np.ascontiguousarray(qubits, dtype=np.uint32)
    mm = np.ascontiguousarray(m, dtype=np.complex128)
    reg._ck(lib.qcs_apply_matrix(reg.handle, q.ctypes.data_as(C.POINTER(C.c_uint32)), len(q),
                                 mm.view(np.float64).ctypes.data_as(C.POINTER(C.c_double))))


def sample_blocks(circuits: int, seed: int, nmin: int = 24, nmax: int = 32, depth: int = 3) -> list[tuple[int, tuple, int]]:
    """blocks of the fuser's partitions of `circuits` seeded random circuits (n in [nmin, nmax], 10% of
    one-qubit slots replaced by controlled rotations, largest block 1..5): (n, qubits, gate count)"""
    from . import circuits as Cc, gates as G
    out = []
    rng = np.random.default_rng(seed)
    for i in range(circuits):
        n = int(rng.integers(nmin, nmax + 1))
        ops = Cc.layered_circuit(n, depth, seed=seed * 1000003 + i, p3=0.02, controlled_frac=0.1)
        mq = int(rng.integers(1, 6))
        for mask, ng in fusion_plan(n, G.records(ops), mq):
            out.append((n, tuple(q for q in range(n) if (mask >> q) & 1), ng))
    return out


def _pass_ms(prof: dict) -> float:
    """average device time of the shared-memory passes in a profile (CUDA-core and tensor-core passes)"""
    launches = sum(v[0] for k, v in prof.items() if k.startswith("tile_pass"))
    return sum(v[1] for k, v in prof.items() if k.startswith("tile_pass")) / launches


def time_blocks(samples, reps: int = 3, seed: int = 0, log=print) -> tuple[np.ndarray, np.ndarray, dict, dict]:
    """device time of each sampled block applied alone in a pass, minus the time of a CUDA-core pass over
    the same register that carries only a one-qubit identity (the memory cost every pass pays).  Blocks
    of 4 and 5 qubits run in tensor-core passes, smaller ones in CUDA-core passes; a block's target is
    thus its whole cost beyond streaming the register once.  Returns features, log(ms) targets and the
    per-size times of the identity passes of both kinds (the tensor-core one carries a 4-qubit
    identity block)."""
    import torch
    from .register import QubitRegister
    rng = np.random.default_rng(seed)
    by_n: dict[int, list] = {}
    for s in samples:
        by_n.setdefault(s[0], []).append(s)
    X, T, pass_ms, pass_ms_tc = [], [], {}, {}

    def pass_time(reg, qubits, m) -> float:
        apply_matrix(reg, qubits, m)  # warm
        reg.read_profile()
        for _ in range(reps):
            apply_matrix(reg, qubits, m)
        return _pass_ms(reg.read_profile())

    for n in sorted(by_n):
        reg = QubitRegister(n, seed=1, precision="fp32")
        reg.profile(True)
        base = pass_time(reg, [0], np.eye(2, dtype=np.complex128))
        base_tc = pass_time(reg, [0, 1, 2, 3], np.eye(16, dtype=np.complex128))
        pass_ms[n], pass_ms_tc[n] = base, base_tc
        for (nn, qubits, ng) in by_n[n]:
            u = random_unitary(len(qubits), rng)
            ms = pass_time(reg, list(qubits), u)
            X.append(features(n, qubits, ng))
            T.append(math.log(max(ms - base, 0.02 * base)))
        reg.profile(False)
        reg.close()
        torch.cuda.synchronize()
        log(f"n={n}: {len(by_n[n])} blocks timed, pass {base:.3f} ms, tensor-core pass {base_tc:.3f} ms")
    return np.array(X, dtype=np.float32), np.array(T, dtype=np.float32), pass_ms, pass_ms_tc


def partition_features(n: int, recs: np.ndarray, max_qubits: int) -> tuple[np.ndarray, int]:
    """the greedy partition with blocks of at most max_qubits, as the engine scores it in fusion mode 2:
    the features of its blocks (in tensor-core passes, which run when a block has 4 or more qubits, a
    smaller block counts as the 4-qubit block it is widened to, with the lowest qubits it lacks) and the
    number of shared-memory passes it packs into"""
    plan = fusion_plan(n, recs, max_qubits)
    tc = n >= 12 and any(bin(m).count("1") >= 4 for m, _ in plan)
    X = []
    for mask, ng in plan:
        q = [b for b in range(n) if (mask >> b) & 1]
        b = 0
        while tc and len(q) < 4:
            if b not in q:
                q.append(b)
            b += 1
        X.append(features(n, sorted(q), ng))
    pob = fusion_passes(n, recs, max_qubits, 12 if tc else 13, tc)
    return np.array(X, dtype=np.float32).reshape(-1, F), (max(pob) + 1 if pob else 0)


def calibration_runs(count: int, seed: int, log=print) -> list:
    """device time of whole fused gate lists: `count` seeded layered circuits (24-32 qubits, depth 6-16,
    10% controlled rotations), each run with the greedy partitions of largest block 1..5.  Returns
    (block features, passes, n, milliseconds) per run."""
    import torch
    from . import circuits as Cc, gates as G
    from .register import QubitRegister
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        n = int(rng.integers(24, 33))
        depth = int(rng.integers(6, 17))
        recs = G.records(Cc.layered_circuit(n, depth, seed=seed * 7919 + i, p3=0.02, controlled_frac=0.1))
        for mq in range(1, 6):
            X, npass = partition_features(n, recs, mq)
            reg = QubitRegister(n, seed=1, precision="fp32")
            reg.set_fusion(1, mq)
            reg.profile(True)
            reg.apply_records(recs)  # first touch and planning structures
            reg.read_profile()
            reg.apply_records(recs)
            prof = reg.read_profile()
            reg.close()
            torch.cuda.synchronize()
            ms = sum(v[1] for k, v in prof.items() if k.startswith("tile_pass"))
            out.append((X, npass, n, ms))
        log(f"calibration circuit {i}: {n} qubits, depth {depth}: " + ", ".join(f"{r[3]:.2f}" for r in out[-5:]) + " ms")
    return out


def calibrate(mlp: Mlp, pass_ms: dict, runs: list, rounds: int = 4, steps: int = 1500, lr: float = 1e-3,
              per_run: int = 96, seed: int = 0) -> dict:
    """fit the block costs to whole-list timings: a list's time beyond its passes' streaming cost,
    t - passes x pass_ms[n], is shared among its blocks in proportion to the model's current predictions,
    and the model is trained on those shares; repeated `rounds` times.  Block costs measured one block
    per pass miss how blocks that share a pass add up; this step fits the sum the partition choice
    compares.  Returns the mean absolute log error of the predicted list times before and after."""
    rng = np.random.default_rng(seed)

    def list_error() -> float:
        err = []
        for X, npass, n, ms in runs:
            pred = float(np.exp(mlp.predict(X)).sum()) + npass * pass_ms[n] if len(X) else npass * pass_ms[n]
            err.append(abs(math.log(pred / ms)))
        return float(np.mean(err))

    before = list_error()
    for _ in range(rounds):
        xs, ts = [], []
        for X, npass, n, ms in runs:
            if not len(X):
                continue
            p = np.exp(mlp.predict(X)).astype(np.float64)
            resid = max(ms - npass * pass_ms[n], 0.05 * ms)
            share = p * (resid / p.sum())
            idx = rng.permutation(len(X))[:per_run]
            xs.append(X[idx])
            ts.append(np.log(share[idx]).astype(np.float32))
        mlp.train(np.concatenate(xs), np.concatenate(ts), steps=steps, lr=lr)
    return {"list_log_error_before": before, "list_log_error_after": list_error()}


def save(mlp: Mlp, pass_ms: dict, path: Path | None = None, meta: dict | None = None, pass_ms_tc: dict | None = None) -> Path:
    """the parameters and a 128-entry table: [n] = one CUDA-core pass over n qubits, [64 + n] = one
    tensor-core pass (0 where not measured)"""
    path = path or (MODEL_DIR / "fusion_cost_mlp.npz")
    path.parent.mkdir(exist_ok=True)
    table = np.zeros(128)
    for n, v in pass_ms.items():
        table[int(n)] = v
    for n, v in (pass_ms_tc or {}).items():
        table[64 + int(n)] = v
    np.savez(path, params=mlp.params(), pass_ms=table, **{k: np.asarray(v) for k, v in (meta or {}).items()})
    return path


def load(path: Path | None = None) -> tuple[Mlp, np.ndarray]:
    path = path or (MODEL_DIR / "fusion_cost_mlp.npz")
    d = np.load(path)
    m = Mlp(F)
    m.set_params(d["params"])
    table = np.zeros(128)
    table[: d["pass_ms"].size] = d["pass_ms"]
    return m, table


def attach(reg, mlp: Mlp, pass_ms: np.ndarray) -> None:
    """fusion mode 2 on this register: the partition with the lowest predicted time"""
    lib = L.load()
    t = np.ascontiguousarray(pass_ms, dtype=np.float64)
    reg._cost_model = (mlp, t)  # keep alive with the register
    reg._ck(lib.qcs_set_cost_model(reg.handle, mlp.handle, L.dptr(t), len(t)))
    reg.set_fusion(2, 5)  # candidate partitions with blocks of up to 5 qubits


def train_from_timings(X: np.ndarray, T: np.ndarray, steps: int = 3000, lr: float = 3e-3, seed: int = 1,
                       holdout: float = 0.15):
    """fit the MLP on (features, log ms); returns the model and held-out error figures"""
    rng = np.random.default_rng(seed)
    idx = rng.permutation(len(X))
    nh = max(1, int(holdout * len(X)))
    te, tr = idx[:nh], idx[nh:]
    mlp = Mlp(F, seed=seed)
    loss = mlp.train(X[tr], T[tr], steps=steps, lr=lr)
    pred = mlp.predict(X[te])
    rel = np.abs(np.exp(pred) - np.exp(T[te])) / np.exp(T[te])
    return mlp, {"train_mse_log": loss, "holdout_mape": float(np.mean(rel)), "holdout_median_ape": float(np.median(rel)),
                 "train": int(len(tr)), "holdout": int(nh)}


def _main() -> None:
    import argparse
    import json
    import time
    ap = argparse.ArgumentParser(description="record fused-block timings on the GPU and train the fusion cost model")
    ap.add_argument("--circuits", type=int, default=20000)
    ap.add_argument("--timed", type=int, default=2400, help="distinct blocks timed on the GPU")
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--out", default=str(MODEL_DIR / "fusion_cost_mlp.npz"))
    ap.add_argument("--calibrate", type=int, default=60, help="circuits timed whole for the calibration step (0: none)")
    args = ap.parse_args()
    t0 = time.time()
    samples = sample_blocks(args.circuits, args.seed)
    distinct = {}
    for n, q, ng in samples:
        key = (n, q)
        distinct[key] = max(distinct.get(key, 0), ng)
    rng = np.random.default_rng(args.seed)
    keys = list(distinct)
    rng.shuffle(keys)
    # stratify by block width so wide blocks are represented
    by_w: dict[int, list] = {}
    for k in keys:
        by_w.setdefault(len(k[1]), []).append(k)
    per = max(1, args.timed // max(1, len(by_w)))
    chosen = []
    for w in sorted(by_w):
        chosen += by_w[w][:per]
    chosen = [(n, q, distinct[(n, q)]) for (n, q) in chosen]
    t1 = time.time()
    X, T, pass_ms, pass_ms_tc = time_blocks(chosen)
    t2 = time.time()
    mlp, metrics = train_from_timings(X, T)
    if args.calibrate:
        runs = calibration_runs(args.calibrate, args.seed)
        metrics.update(calibrate(mlp, pass_ms, runs))
        metrics["calibration_runs"] = len(runs)
    t3 = time.time()
    metrics.update({"circuits": args.circuits, "blocks_sampled": len(samples), "distinct_blocks": len(distinct),
                    "blocks_timed": len(chosen), "seconds_sampling": t1 - t0, "seconds_timing": t2 - t1,
                    "seconds_training": t3 - t2, "pass_ms": {str(k): v for k, v in pass_ms.items()},
                    "pass_ms_tc": {str(k): v for k, v in pass_ms_tc.items()}})
    path = save(mlp, pass_ms, Path(args.out), meta={"X": X, "T": T}, pass_ms_tc=pass_ms_tc)
    print(json.dumps({"model": str(path), **metrics}))


if __name__ == "__main__":
    _main()
