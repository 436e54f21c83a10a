"""Benchmark of the statevector hot path: the 30-qubit complex<double> layered random circuit
(depth 60, Toffoli/CCZ at 5% of positions, seed 1) on one GB300.

A step applies one layer of the circuit (its 1-qubit gates, CNOT matching and inserted 3-qubit gates,
about 47 gates) to the 30-qubit register resident in HBM; steps walk through the circuit's 60 layers.
`value` is gates/s over the K timed steps (whole job: the sum over ranks' gates / the slowest rank's
time).  `e2e` repeats the steps through the C ABI from host gate records with a device->host read of a
qubit probability after every step.  The state (16 GiB) is larger than L2, so no flush is needed.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

The line also carries: the roofline of the dominant kernel (algorithmic bytes of the gates its launches
applied over their CUDA-event time; DRAM traffic per launch from the committed ncu summary), the same
kernel's FP64-compute ceiling (`fp64_roofline`: FP64 instructions of its gate arithmetic per second
against cuBLAS DGEMM measured in the same run), the same layers with one kernel per gate (`per_gate`),
QFT-30 (`qft`), the first four layers on fused FP32 registers against FP64 (`fused_fp32`: greedy blocks
of at most 4 qubits on the tensor cores and the learned partition), the 20-qubit depth-40 circuit timed whole on the GPU and
on the CPU reference (`c0`), SM clocks sampled during the timed region, and the CPU reference on a bounded
sample (`cpu_baseline`: QCSim's own QubitRegister compiled on the host where its sources were staged,
else the oracle's restatement; OpenMP on all host threads).  `parity_at_size` checks the engine against
that CPU reference at the full size: the baseline's gate sample, the QFT of a random normal state, and
1024 seeded shots from it.  Unless --quick, the line also carries the other configurations:
`c2_precision` (33 qubits, depth 80: fused FP32 with blocks of at most 3, 4 and 5 qubits against plain FP64), `c3_qaoa` (512 QAOA instances, p = 4,
one launch, FP64 and FP32) and `c4_learned` (an unseen 32-qubit circuit of depth 100 with 10% controlled
rotations: the learned partition against the greedy fuser with largest blocks of 3, 4 and 5 qubits and
unfused FP64).

--impl reference times the same CPU reference on the same workload, a bounded number of gates per step.
The configurations also run alone: --config precision, qaoa (sharded over ranks under torchrun), learned,
and schrodinger (QCSim's split-operator SchrodingerSimulation: Trotter steps/s, with --qubits and --steps).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "30q circuit gates/s & HBM frac; fused FP32 vs plain FP64 time @1-F≤1e-6"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--qubits", type=int, default=30)
    ap.add_argument("--depth", type=int, default=60)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-gates", type=int, default=60, help="gates in the CPU baseline sample (a third per reference-arm step)")
    ap.add_argument("--model", default=None, help="learned config: cost-model file")
    ap.add_argument("--config", default="layered", choices=["layered", "precision", "qaoa", "learned", "schrodinger"],
                    help="layered: the 30-qubit FP64 circuit (headline); precision: fused FP32 vs plain FP64")
    ap.add_argument("--max-block", type=int, default=None, help="precision config: largest fused block (default: 3, 4 and 5)")
    ap.add_argument("--no-fused", action="store_true", help="skip the fused-FP32 comparison in the layered line")
    ap.add_argument("--quick", action="store_true",
                    help="leave the precision (33 qubits), QAOA-batch and learned-fusion configurations out of the line")
    args = ap.parse_args()
    args.max_block_given = args.max_block is not None
    return args


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def algorithmic_bytes(gate, n: int, amp_bytes: int = 16) -> float:
    """2 * s * 2^n * f(g), f = fraction of rows of the gate matrix that differ from the identity row"""
    m = gate.getRawOperatorMatrix()
    d = m.shape[0]
    changed = sum(1 for r in range(d) if not np.array_equal(m[r], np.eye(d)[r]))
    return 2.0 * amp_bytes * (2 ** n) * changed / d


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms while running"""

    FIELDS = "clocks.sm,clocks.max.sm,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown," \
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown," \
             "clocks_event_reasons.sw_power_cap"

    def __init__(self, index: int = 0):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_init(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
        return rank, world, local, dist
    return rank, world, local, None


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, v: float) -> float:
    from qcsim_gb300 import replicas
    return replicas.max_over_ranks(dist, v, device="cuda")


def layers_of(ops, n):
    """split the layered circuit into its layers (a layer ends with its last CNOT and any 3-qubit gate
    inserted after it)"""
    layers, cur, seen_cx = [], [], 0
    per_layer_cx = n // 2
    for op in ops:
        cur.append(op)
        if type(op[0]).__name__ == "CNOTGate":
            seen_cx += 1
        if seen_cx == per_layer_cx:
            layers.append(cur)
            cur, seen_cx = [], 0
    if cur:
        layers[-1].extend(cur)
    return layers


def reference_cpu():
    """the CPU implementation timed beside the engine: QCSim's own QubitRegister compiled on this host
    (oracle/_ref/libqcsref.so, kind "reference"), built where QCSim's sources were staged, else the
    oracle's restatement of its loops (kind "port").  Both run OpenMP on every host thread.  Returns
    (kind, register factory, thread count)."""
    from oracle import bind
    bind.build_oracle(ref=True)
    lib = bind.oracle()
    threads = lib.qo_max_threads()
    if bind.ref_available():
        return "reference", (lambda n, seed=1: bind.RefRegister(n, seed)), threads
    return "port", (lambda n, seed=1: bind.OracleRegister(n)), threads


def host_bytes_available() -> int:
    try:
        for ln in open("/proc/meminfo"):
            if ln.startswith("MemAvailable"):
                return int(ln.split()[1]) * 1024
    except OSError:
        pass
    return 0


def cpu_baseline(args, ops, rank):
    """the CPU reference on a bounded sample of the workload: the first `cpu_gates` gates at the full
    size (fewer qubits only if the host cannot hold the reference's two state vectors).  Returns the
    baseline object, and the register and gate sample for the parity check at this size."""
    kind, make, threads = reference_cpu()
    n = args.qubits
    need = 2 * 16 * (2 ** n)
    avail = host_bytes_available()
    while n > 20 and need > 0.6 * avail:
        n -= 1
        need //= 2
    reg = make(n, args.seed)
    sample = [op for op in ops if max(op[1:1 + op[0].getQubitsNumber()]) < n][: args.cpu_gates]
    reg.apply(sample[:1])  # warm-up (first touch)
    t0 = time.perf_counter()
    reg.apply(sample[1:])
    dt = time.perf_counter() - t0
    gps = (len(sample) - 1) / dt
    scaled = gps * (2 ** n) / (2 ** args.qubits)
    base = {"value": scaled, "unit": "gates/s", "cores": threads, "kind": kind,
            "sample": f"gates 2-{len(sample)} of the circuit on a {n}-qubit register, {dt:.2f} s"
                      + ("" if n == args.qubits else f", scaled by 2^{n - args.qubits} to {args.qubits} qubits")}
    return base, reg, sample, n


def max_abs_diff(a: np.ndarray, b: np.ndarray) -> float:
    from oracle import bind
    a = np.ascontiguousarray(a, dtype=np.complex128)
    b = np.ascontiguousarray(b, dtype=np.complex128)
    return float(bind.oracle().qo_max_abs_diff(bind.dp(a.view(np.float64)), bind.dp(b.view(np.float64)), a.size))


def shot_identity(a: dict, b: dict, shots: int) -> float:
    """the fraction of shots on which two histograms of the same seeded uniforms agree"""
    return sum(min(c, b.get(k, 0)) for k, c in a.items()) / shots if shots else 1.0


def shots_near_boundary(state: np.ndarray, probs: np.ndarray, eps: float, chunk: int = 1 << 24) -> int:
    """how many of the uniforms lie within eps of an entry of the state's cumulative probability table
    (where the two engines' rounding can choose neighbouring states); the table is built chunk by chunk"""
    p = np.sort(probs)
    near = np.zeros(p.size, dtype=bool)
    total = 0.0
    for lo in range(0, state.size, chunk):
        seg = state[lo:lo + chunk]
        cdf = np.cumsum(seg.real * seg.real + seg.imag * seg.imag) + total
        a, b = np.searchsorted(p, [cdf[0] - eps, cdf[-1] + eps])
        for i in range(a, b):
            j = min(np.searchsorted(cdf, p[i]), cdf.size - 1)
            if abs(cdf[j] - p[i]) < eps or (j > 0 and abs(cdf[j - 1] - p[i]) < eps):
                near[i] = True
        total = float(cdf[-1])
    return int(near.sum())


def parity_at_size(n: int, seed: int, ref_reg, sample, kind: str, shots: int = 1024) -> dict:
    """the engine against the CPU reference at the bench's own size, on the same inputs:
    (1) the circuit sample the CPU baseline applied, on a fresh FP64 engine register: max |da|;
    (2) the QFT of all n qubits on a random normal state (QuantumFourierTransform.h:35-60, with the
    swaps): max |da|, then `shots` seeded RepeatedMeasure shots on each (QubitRegister.h:227-271): the
    fraction of identical shots, and the shots whose cumulative probability lies within 1e-12 of a table
    boundary of the other engine's (where rounding can pick the neighbouring state)."""
    import torch
    import qcsim_gb300 as Q
    from qcsim_gb300 import _lib as L, gates as G
    from oracle import bind
    out = {"qubits": n, "reference_kind": kind, "tolerance": 1e-12}
    t0 = time.perf_counter()
    reg = Q.QubitRegister(n, seed=seed)
    reg.apply_records(G.records(sample))
    torch.cuda.synchronize()
    ref_state = ref_reg.state()
    out["circuit"] = {"gates": len(sample), "max_abs_amplitude_difference": max_abs_diff(reg.getRegisterStorage(), ref_state)}
    del ref_state
    # QFT on a random normal state: the reference register is reused (its RNG still unused), the engine's
    # register reseeded with the same seed, so both draw the same uniforms for the shots
    v = np.empty(1 << n, dtype=np.complex128)
    bind.oracle().qo_random_normal_state(seed, n, bind.dp(v.view(np.float64)))
    ref_reg.set_state(v)
    tq = time.perf_counter()
    if kind == "reference":
        ref_reg.lib.qr_qft(ref_reg.h, n, 0, n - 1, 0, 1)
    else:
        ref_reg.lib.qo_qft(ref_reg.h, 0, n - 1, 0, 1)
    ref_qft_s = time.perf_counter() - tq
    reg.setRegisterStorageFastNoNormalize(v)
    del v
    L.check(reg._lib.qcs_qft(reg.handle, 0, n - 1, 0, 1), reg.handle)
    got = reg.getRegisterStorage()
    ref_state = ref_reg.state()
    qft = {"max_abs_amplitude_difference": max_abs_diff(got, ref_state), "reference_seconds": ref_qft_s}
    # shots: the engine's RepeatedMeasure and the reference's, each from a generator seeded with `seed`
    reg.seed(seed)
    g_hist = reg.RepeatedMeasure(shots)
    if kind == "reference":
        ref_reg.lib.qr_seed(ref_reg.h, seed)
        r_hist = ref_reg.repeated_measure(shots)
    else:
        from qcsim_gb300.rng import Mt19937_64
        gen = Mt19937_64(seed)
        probs = np.array([1.0 - gen.uniform() for _ in range(shots)])
        keys, cnt = np.unique(ref_reg.sample(probs), return_counts=True)
        r_hist = {int(k): int(c) for k, c in zip(keys, cnt)}
    from qcsim_gb300.rng import Mt19937_64
    gen = Mt19937_64(seed)
    near = shots_near_boundary(ref_state, np.array([1.0 - gen.uniform() for _ in range(shots)]), 1e-12)
    del ref_state, got
    qft.update({"shots": shots, "shot_identity_rate": shot_identity(g_hist, r_hist, shots), "shots_near_boundary": near})
    out["qft"] = qft
    out["seconds"] = time.perf_counter() - t0
    reg.close()
    return out


def small_config_both(seed: int) -> dict:
    """the 20-qubit layered circuit of depth 40 (the CPU-sized configuration) end to end on the GPU
    (one ApplyGates call, state resident) and on the CPU reference (QCSim's register where its sources
    are staged, else the oracle's restatement) with every host thread"""
    import torch
    import qcsim_gb300 as Q
    from qcsim_gb300 import circuits, gates as G
    ops = circuits.layered_circuit(20, 40, seed=seed)
    recs = G.records(ops)
    reg = Q.QubitRegister(20, seed=seed)
    reg.apply_records(recs)  # warm-up
    reg.setToBasisState(0)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    reg.apply_records(recs)
    torch.cuda.synchronize()
    gpu_s = time.perf_counter() - t0
    gpu_state = reg.getRegisterStorage()
    reg.close()
    kind, make, threads = reference_cpu()
    ref = make(20, seed)
    t0 = time.perf_counter()
    ref.apply(ops)
    cpu_s = time.perf_counter() - t0
    err = max_abs_diff(gpu_state, ref.state())
    return {"workload": f"layered random circuit, 20 qubits, depth 40, seed {seed} ({len(ops)} gates)",
            "gpu_seconds": gpu_s, "cpu_seconds": cpu_s, "cpu_kind": kind, "cpu_cores": threads, "gpu_gates_per_s": len(ops) / gpu_s,
            "cpu_gates_per_s": len(ops) / cpu_s, "max_abs_amplitude_difference": err}


def run_reference(args):
    """the reference arm: QCSim's own register compiled on this host (or the oracle's restatement where
    QCSim's sources are not staged) applies the same circuit, a bounded window of gates per step"""
    rank, world, local, dist = dist_init(args)
    if rank != 0:
        return
    from qcsim_gb300 import circuits
    kind, make, threads = reference_cpu()
    n = args.qubits
    ops = circuits.layered_circuit(n, args.depth, seed=args.seed, p3=0.05)
    reg = make(n, args.seed)
    g = max(1, args.cpu_gates // 3)
    pos = 0
    for _ in range(args.warmup):
        reg.apply(ops[pos:pos + g])
        pos += g
    t0 = time.perf_counter()
    done = 0
    for _ in range(args.steps):
        chunk = ops[pos % len(ops):pos % len(ops) + g]
        reg.apply(chunk)
        done += len(chunk)
        pos += g
    dt = time.perf_counter() - t0
    v = done / dt
    what = "QCSim's QubitRegister compiled on this host" if kind == "reference" else "the oracle's restatement of QCSim's loops"
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "gates/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"layered random circuit, {n} qubits, depth {args.depth}, Toffoli/CCZ at 5%, "
                                   f"seed {args.seed}; {g} gates per step", "qubits": n},
            "cpu_baseline": {"value": v, "unit": "gates/s", "cores": threads, "kind": kind,
                             "sample": f"{what}; {g} gates per step, {args.steps} timed steps on the full {n}-qubit register"},
            "e2e": {"value": v, "unit": "gates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_gb300(args):
    rank, world, local, dist = dist_init(args)
    import torch
    torch.cuda.set_device(local)
    import qcsim_gb300 as Q
    from qcsim_gb300 import _lib as L, circuits, gates as G

    lib = L.load()
    n = args.qubits
    ops = circuits.layered_circuit(n, args.depth, seed=args.seed, p3=0.05)
    layers = layers_of(ops, n)
    recs = [G.records(lay) for lay in layers]
    bytes_layer = [sum(algorithmic_bytes(op[0], n) for op in lay) for lay in layers]

    stream = torch.cuda.Stream()
    reg = Q.QubitRegister(n, seed=args.seed)
    lib.qcs_set_stream(reg.handle, stream.cuda_stream)

    def step(i):
        reg.apply_records(recs[i % len(recs)])

    # warm-up
    for i in range(args.warmup):
        step(i)
    torch.cuda.synchronize()

    # timed region (device time, events on the engine's stream; the engine also brackets each of its
    # launches with events so the dominant kernel's average duration comes from this same region)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reg.profile(True)
    reg.read_profile()
    launches0 = lib.qcs_launch_count()
    with ClockSampler(local) as clk:
        barrier(dist)
        torch.cuda.synchronize()
        e0.record(stream)
        gates = 0
        alg_bytes = 0.0
        for i in range(args.warmup, args.warmup + args.steps):
            step(i)
            gates += len(layers[i % len(layers)])
            alg_bytes += bytes_layer[i % len(layers)]
        e1.record(stream)
        torch.cuda.synchronize()
        barrier(dist)
    launches = lib.qcs_launch_count() - launches0
    prof_ops = reg.read_profile(fp_ops=True)
    prof = {k: v[:3] for k, v in prof_ops.items()}
    reg.profile(False)
    ms = e0.elapsed_time(e1)
    ms_max = max_over_ranks(dist, ms)
    value = gates * world / (ms_max / 1e3)
    peak, peak_kind = peaks()
    hbm_frac = alg_bytes / (ms / 1e3) / (peak * 1e9)
    roofline = roofline_of(prof, peak, peak_kind, n, alg_bytes)
    fp64_roof = fp64_roofline_of(prof_ops, roofline["kernel"], dgemm_tflops())

    # end to end through the C ABI: host gate records in, a qubit probability out, every step
    barrier(dist)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    h2d = 0
    for i in range(args.warmup, args.warmup + args.steps):
        r = recs[i % len(recs)]
        reg.apply_records(r)
        h2d += r.nbytes
        reg.GetQubitProbability(i % n)
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(dist, time.perf_counter() - t0)
    e2e = {"value": gates * world / e2e_s, "unit": "gates/s", "h2d_bytes_per_step": h2d / args.steps,
           "d2h_bytes_per_step": 8}

    # the same layers with one kernel per gate (the plain per-gate path), profiled the same way
    extra = {}
    if rank == 0:
        reg.set_passes(False)
        reg.profile(True)
        reg.read_profile()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        pg_gates, pg_bytes = 0, 0.0
        for i in range(min(args.steps, 6)):
            step(i)
            pg_gates += len(layers[i % len(layers)])
            pg_bytes += bytes_layer[i % len(layers)]
        b.record(stream)
        b.synchronize()
        pg_ms = a.elapsed_time(b)
        pg_prof = reg.read_profile()
        reg.profile(False)
        reg.set_passes(True)
        extra["per_gate"] = {"gates_per_s": pg_gates / (pg_ms / 1e3), "hbm_frac_per_gate": pg_bytes / (pg_ms / 1e3) / (peak * 1e9),
                             "kernels": {k: {"launches": v[0], "ms": v[1], "GB/s": v[2] / (v[1] / 1e3) / 1e9 if v[1] else None}
                                         for k, v in pg_prof.items()}}

    # QFT over all qubits, device-timed, one call (its time does not depend on the amplitudes, so the
    # circuit's output state serves as the input; QFT parity on random normal inputs is in the tests)
    if rank == 0:
        torch.cuda.synchronize()
        qops = circuits.qft_circuit(0, n - 1)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        lib.qcs_qft(reg.handle, 0, n - 1, 0, 1)
        b.record(stream)
        b.synchronize()
        qft_ms = a.elapsed_time(b)
        qb = sum(algorithmic_bytes(op[0], n) for op in qops)
        extra["qft"] = {"qubits": n, "seconds": qft_ms / 1e3, "gates": len(qops), "gates_per_s": len(qops) / (qft_ms / 1e3),
                        "hbm_frac_per_gate": qb / (qft_ms / 1e3) / (peak * 1e9)}

    # the metric's second half on the same circuit: its first four layers on a fresh FP64 register and on
    # fused FP32 registers (greedy blocks of at most 4 qubits; the learned partition), device time and fidelity
    if rank == 0 and not args.no_fused:
        fops = [op for lay in layers[:4] for op in lay]
        extra["fused_fp32"] = {"workload": f"layers 0-3 of the circuit above ({len(fops)} gates); greedy blocks of at most "
                                           "4 qubits on the tensor cores (the engine's default at this size), and the partition "
                                           "of the shipped learned cost model",
                               **fused_vs_fp64(n, fops, 4, args.seed, learned=True)}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        reg.close()  # the parity and configuration legs below need the device memory
        cpu, ref_reg, sample, n_ref = cpu_baseline(args, ops, rank)
        extra["parity_at_size"] = parity_at_size(n_ref, args.seed, ref_reg, sample, cpu["kind"])
        del ref_reg
        extra["c0"] = small_config_both(args.seed)
    if rank == 0 and world == 1 and not args.quick:
        reg.close()
        extra["c2_precision"] = precision_config(33, 80, args.seed, (3, 4, 5))
        extra["c3_qaoa"] = qaoa_config(args.seed, args.steps, dist=None)
        extra["c4_learned"] = learned_config(32, 100, args.seed, None)

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "gates/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": {"workload": f"layered random circuit, {n} qubits complex<double> (16 GiB), depth "
                                       f"{args.depth}, Toffoli/CCZ at 5% of positions, seed {args.seed}; one layer "
                                       "per step", "qubits": n, "gates_timed": gates, "parallelism": f"replicas{world}",
                           "l2": "state (16 GiB) larger than L2"},
                "hbm_frac_per_gate": hbm_frac, "roofline": roofline, "fp64_roofline": fp64_roof, "cpu_baseline": cpu, "e2e": e2e,
                "clocks": clk.summary(), "gpu_launches": int(launches), **extra}
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


def roofline_of(prof: dict, peak: float, peak_kind: str, n: int, gate_bytes: float) -> dict:
    """the kernel family with the largest share of device time, as an HBM roofline point.

    achieved = algorithmic bytes per launch / average launch duration, where the algorithmic bytes are
    the per-gate figure 2 x 16 B x 2^n x f(g) summed over the gates the launches applied (f = fraction of
    rows of the gate matrix that differ from the identity).  When the family ran every launch of the
    timed region (the shared-memory pass does on the layered circuit), those are all the gates timed.
    pass_bytes_per_launch is what one launch must move at least (every amplitude it touches read and
    written once); traffic is the DRAM bytes ncu measured for one launch of the family."""
    total = sum(v[1] for v in prof.values()) or 1.0
    all_launches = sum(v[0] for v in prof.values())
    dom = max(prof, key=lambda k: prof[k][1])
    launches, ms, pass_bytes = prof[dom]
    alg_per_launch = gate_bytes / launches if launches == all_launches else pass_bytes / launches
    avg_s = ms / launches / 1e3
    achieved = alg_per_launch / avg_s / 1e9
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": read_traffic(dom, n), "kernel": dom, "peak_source": peak_kind,
            "algorithmic_bytes_per_launch": alg_per_launch, "avg_launch_ms": ms / launches,
            "pass_bytes_per_launch": pass_bytes / launches, "pass_GBps": pass_bytes / launches / avg_s / 1e9,
            "share_of_device_time": ms / total, "launches": launches}


def dgemm_tflops(size: int = 4096) -> float:
    """the GPU's FP64 rate: cuBLAS DGEMM (torch.matmul on float64, size^3, best of 3 after a warm-up
    call), in TFLOP/s"""
    import torch
    a = torch.randn(size, size, dtype=torch.float64, device="cuda")
    b = torch.randn_like(a)
    c = torch.matmul(a, b)
    best = float("inf")
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b, out=c)
        e1.record()
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1))
    del a, b, c
    return 2.0 * size ** 3 / (best / 1e3) / 1e12


def fp64_roofline_of(prof_ops: dict, kernel: str, dgemm: float) -> dict:
    """the FP64-compute ceiling of a kernel family: floating-point instructions its launches issued (the
    engine counts them per pass from the gate forms: an FMA, multiply or add on an amplitude component is
    one) per second of its device time, against the DGEMM rate in instructions (one FMA = one
    instruction = two flops)"""
    launches, ms, _, ops = prof_ops[kernel]
    achieved = ops / (ms / 1e3) / 1e12
    peak = dgemm / 2.0
    return {"bound": "fp64", "kernel": kernel, "achieved": achieved, "peak": peak, "unit": "T FP64 instr/s",
            "frac": achieved / peak, "fp_ops_per_launch": ops / launches,
            "peak_source": "cuBLAS DGEMM 4096^3 measured in this run, one instruction per FMA", "dgemm_tflops": dgemm}


def read_traffic(kernel_family: str, n: int):
    """DRAM bytes per launch from the committed ncu summaries (profiles/*.md, a line
    'traffic <family> <bytes> qubits <m>'), scaled by 2^(n - m): a launch of these families sweeps the
    whole register, so its traffic grows in proportion to the amplitude count.  None if not captured."""
    for p in sorted((ROOT / "profiles").glob("*.md")):
        for ln in p.read_text().splitlines():
            parts = ln.strip().strip("|").split()
            if len(parts) >= 5 and parts[0] == "traffic" and parts[1] == kernel_family and parts[3] == "qubits":
                try:
                    return float(parts[2]) * 2.0 ** (n - int(parts[4]))
                except ValueError:
                    pass
    return None


def fused_vs_fp64(n: int, ops: list, max_block: int, seed: int = 1, learned: bool = False) -> dict:
    """the same gate list on a plain FP64 register and on a fused FP32 register (greedy blocks of at most
    max_block qubits; 4- and 5-qubit blocks on the tensor cores): device time of each (the call includes
    the host-side planning) and the fidelity / max amplitude error of the FP32 result"""
    import ctypes as C
    import torch
    import qcsim_gb300 as Q
    from qcsim_gb300 import _lib as L, gates as G
    lib = L.load()
    recs = G.records(ops)
    stream = torch.cuda.Stream()
    out, regs = {}, {}
    runs = ("fp64", "fp32", "learned") if learned else ("fp64", "fp32")
    for prec in runs:
        reg = Q.QubitRegister(n, seed=seed, precision="fp64" if prec == "fp64" else "fp32")
        lib.qcs_set_stream(reg.handle, stream.cuda_stream)
        if prec == "fp32":
            reg.set_fusion(1, max_block)
        elif prec == "learned":
            from qcsim_gb300 import costmodel
            mlp, pass_ms = costmodel.load()  # the GPU-trained model shipped with the package
            costmodel.attach(reg, mlp, pass_ms)
        reg.profile(True)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        reg.apply_records(recs)
        b.record(stream)
        b.synchronize()
        prof = reg.read_profile()
        reg.profile(False)
        out[prec] = {"seconds": a.elapsed_time(b) / 1e3, "kernels": {k: {"launches": v[0], "ms": v[1]} for k, v in prof.items()}}
        regs[prec] = reg
    f, d = C.c_double(), C.c_double()
    L.check(lib.qcs_compare(regs["fp64"].handle, regs["fp32"].handle, C.byref(f), C.byref(d)), regs["fp64"].handle)
    res = {"gates": len(ops), "max_block_qubits": max_block, "fp64_seconds": out["fp64"]["seconds"],
           "fp32_fused_seconds": out["fp32"]["seconds"], "speedup": out["fp64"]["seconds"] / out["fp32"]["seconds"],
           "one_minus_fidelity": 1.0 - f.value, "max_abs_amplitude_error": d.value,
           "fp64_kernels": out["fp64"]["kernels"], "fp32_kernels": out["fp32"]["kernels"]}
    if learned:
        L.check(lib.qcs_compare(regs["fp64"].handle, regs["learned"].handle, C.byref(f), C.byref(d)), regs["fp64"].handle)
        res["learned"] = {"seconds": out["learned"]["seconds"], "speedup": out["fp64"]["seconds"] / out["learned"]["seconds"],
                          "one_minus_fidelity": 1.0 - f.value, "max_abs_amplitude_error": d.value,
                          "kernels": out["learned"]["kernels"]}
    for r in regs.values():
        r.close()
    return res


def precision_config(n: int, depth: int, seed: int, blocks=(3, 4, 5)) -> dict:
    """the precision configuration: the layered circuit on a plain FP64 register (16 * 2^n bytes) and on a
    fused FP32 register (8 * 2^n bytes) with greedy blocks of at most 3 qubits (CUDA cores) and of at most
    4 and 5 qubits (every block as a 3xTF32 product on the tensor cores): device time of each, the
    speed-up of the faster FP32 run, and every FP32 result's fidelity and max amplitude error against the
    FP64 one"""
    import ctypes as C
    import torch
    import qcsim_gb300 as Q
    from qcsim_gb300 import _lib as L, circuits, gates as G
    lib = L.load()
    ops = circuits.layered_circuit(n, depth, seed=seed)
    recs = G.records(ops)
    stream = torch.cuda.Stream()

    def timed(reg):
        lib.qcs_set_stream(reg.handle, stream.cuda_stream)
        reg.profile(True)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        reg.apply_records(recs)
        b.record(stream)
        b.synchronize()
        prof = reg.read_profile()
        reg.profile(False)
        return a.elapsed_time(b) / 1e3, {k: {"launches": v[0], "ms": v[1]} for k, v in prof.items()}

    r64 = Q.QubitRegister(n, seed=seed)
    t64, k64 = timed(r64)
    out = {"workload": f"layered random circuit, {n} qubits, depth {depth}, seed {seed}; FP64 {16 << n >> 30} GiB, "
                       f"FP32 {8 << n >> 30} GiB", "gates": len(ops), "fp64_seconds": t64, "fp64_kernels": k64, "fp32_fused": {}}
    for mb in blocks:
        r32 = Q.QubitRegister(n, seed=seed, precision="fp32")
        r32.set_fusion(1, mb)
        t32, k32 = timed(r32)
        f, d = C.c_double(), C.c_double()
        L.check(lib.qcs_compare(r64.handle, r32.handle, C.byref(f), C.byref(d)), r64.handle)
        out["fp32_fused"][f"max_block_{mb}"] = {"seconds": t32, "speedup": t64 / t32, "one_minus_fidelity": 1.0 - f.value,
                                                 "max_abs_amplitude_error": d.value, "kernels": k32}
        r32.close()
    r64.close()
    best = min(out["fp32_fused"], key=lambda k: out["fp32_fused"][k]["seconds"])
    out.update({"best": best, "fp32_fused_seconds": out["fp32_fused"][best]["seconds"], "speedup": t64 / out["fp32_fused"][best]["seconds"],
                "one_minus_fidelity": out["fp32_fused"][best]["one_minus_fidelity"],
                "max_abs_amplitude_error": out["fp32_fused"][best]["max_abs_amplitude_error"]})
    return out


def run_precision(args):
    """fused FP32 (greedy blocks of at most --max-block qubits, and of at most 3 and 5 unless given)
    against plain FP64 on the same layered circuit"""
    blocks = (args.max_block,) if args.max_block_given else (3, 4, 5)
    res = precision_config(args.qubits, args.depth, args.seed, blocks)
    line = {"metric": "fused FP32 vs plain FP64 time @1-F<=1e-6", "config": {
                "workload": res.pop("workload"), "gates": res.pop("gates"), "max_block_qubits": list(blocks)},
            **res, "data": "synthetic"}
    print(json.dumps(line))


def qaoa_config(seed: int, steps: int, dist=None, rank: int = 0, world: int = 1) -> dict | None:
    """512 random 3-regular Ising instances (n even in 12..24), p = 4: <H> for every instance in one
    persistent launch replayed from a CUDA graph, FP64 and FP32, after the autotuner picks the schedule;
    instances/s and amplitude-layer updates/s; energies against the CPU oracle's exact <H> on a sample of
    instances.  Under torchrun the instances are dealt to ranks by cost and the energies gathered at the
    end; rank 0 returns the result, the others None."""
    import ctypes as C
    from qcsim_gb300 import circuits, qaoa, replicas
    from oracle import bind as B
    insts = circuits.qaoa_instances(512, seed=seed, nmin=12, nmax=24, p=4)
    mine = replicas.shard_by_cost(replicas.qaoa_costs(insts), world)[rank]
    out = {}
    for prec in ("fp64", "fp32"):
        batch = qaoa.QaoaBatch([insts[i] for i in mine], 4, prec)
        tuned = batch.autotune()  # the schedule shape (cluster size, mixer tile), chosen by timing
        batch.run()
        times = []
        for _ in range(max(3, steps // 5)):
            barrier(dist)
            t0 = time.perf_counter()
            e = batch.run()
            times.append(max_over_ranks(dist, time.perf_counter() - t0))
        amps = sum(1 << insts[i]["n"] for i in range(len(insts)))
        energies = replicas.gather_values(dist, mine, e, len(insts), device="cuda")
        out[prec] = {"cluster": batch.cluster, "tile": list(batch.tile), "autotune_seconds": tuned,
                     "seconds_per_launch": statistics.median(times),
                     "instances_per_s": len(insts) / statistics.median(times),
                     "amplitude_layers_per_s": amps * 4 / statistics.median(times), "energies": energies}
        batch.close()
    if rank != 0:
        return None
    # exact <H> of a sample of instances from the CPU oracle's statevector
    lib = B.oracle()
    errs = {"fp64": 0.0, "fp32": 0.0}
    checked = []
    for i in range(0, 512, 37):
        inst = insts[i]
        if inst["n"] > 20:
            continue
        e = np.array(inst["edges"], dtype=np.uint32).reshape(-1)
        J, h = np.array(inst["J"]), np.array(inst["h"])
        g, b = np.array(inst["gammas"]), np.array(inst["betas"])
        reg = B.OracleRegister(inst["n"])
        pu = e.ctypes.data_as(C.POINTER(C.c_uint32))
        lib.qo_qaoa_exec(reg.h, len(inst["edges"]), pu, B.dp(J), B.dp(h), 4, B.dp(g), B.dp(b))
        ref = lib.qo_expected_energy(reg.h, len(inst["edges"]), pu, B.dp(J), B.dp(h))
        for prec in errs:
            errs[prec] = max(errs[prec], abs(out[prec]["energies"][i] - ref))
        checked.append(i)
    return {"workload": f"512 random 3-regular Ising graphs, n even in 12..24, J = +-1, h ~ N(0, 0.5^2), p = 4, seed {seed}",
            "amplitudes": int(sum(1 << x["n"] for x in insts)),
            "fp64": {k: v for k, v in out["fp64"].items() if k != "energies"},
            "fp32": {k: v for k, v in out["fp32"].items() if k != "energies"},
            "max_abs_energy_error_vs_oracle": errs,
            "oracle_checked": f"{len(checked)} instances (every 37th with n <= 20: {[insts[i]['n'] for i in checked]} qubits)"}


def run_qaoa(args):
    """the QAOA batch alone (sharded over ranks under torchrun)"""
    rank, world, local, dist = dist_init(args)
    res = qaoa_config(args.seed, args.steps, dist, rank, world)
    if res is not None:
        line = {"metric": "QAOA batch: <H> for 512 instances per launch", "config": {
                    "workload": res.pop("workload"), "amplitudes": res.pop("amplitudes")},
                **res, "n_gpus": world, "scaling": "strong", "data": "synthetic"}
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


def learned_config(n: int, depth: int, seed: int, model: str | None) -> dict:
    """learned fusion on an unseen circuit (n qubits, depth, 10% of one-qubit slots controlled
    rotations): device time and fidelity of the FP32 path with the MLP's partition, with the greedy
    fuser (largest block 3, 4 and 5), and of the unfused plain FP64 path.  Each FP32 time includes the
    partition search and planning of its first (and only) call."""
    import ctypes as C
    import torch
    import qcsim_gb300 as Q
    from qcsim_gb300 import _lib as L, circuits, costmodel, gates as G
    lib = L.load()
    ops = circuits.layered_circuit(n, depth, seed=9001 + seed, controlled_frac=0.1)
    recs = G.records(ops)
    stream = torch.cuda.Stream()
    mlp, pass_ms = costmodel.load(Path(model) if model else None)

    def timed(reg):
        lib.qcs_set_stream(reg.handle, stream.cuda_stream)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        reg.apply_records(recs)
        b.record(stream)
        b.synchronize()
        return a.elapsed_time(b) / 1e3

    r64 = Q.QubitRegister(n, seed=1)
    t64 = timed(r64)
    res = {"fp64_unfused_seconds": t64}
    for name, setup in (("greedy5", lambda r: r.set_fusion(1, 5)), ("greedy4", lambda r: r.set_fusion(1, 4)),
                        ("greedy3", lambda r: r.set_fusion(1, 3)), ("learned", lambda r: costmodel.attach(r, mlp, pass_ms))):
        r32 = Q.QubitRegister(n, seed=1, precision="fp32")
        setup(r32)
        t = timed(r32)
        f, d = C.c_double(), C.c_double()
        L.check(lib.qcs_compare(r64.handle, r32.handle, C.byref(f), C.byref(d)), r64.handle)
        res[name] = {"seconds": t, "speedup_vs_fp64": t64 / t, "one_minus_fidelity": 1 - f.value,
                     "max_abs_amplitude_error": d.value}
        r32.close()
    r64.close()
    best = min(("greedy3", "greedy4", "greedy5"), key=lambda k: res[k]["seconds"])
    return {"workload": f"layered random circuit, {n} qubits, depth {depth}, 10% controlled rotations, seed "
                        f"{9001 + seed} (not seen in training)", "gates": len(ops), **res,
            "learned_gain_vs_best_greedy": res[best]["seconds"] / res["learned"]["seconds"], "best_greedy": best}


def run_learned(args):
    res = learned_config(args.qubits, args.depth, args.seed, args.model)
    line = {"metric": "learned fusion: MLP partition vs greedy vs unfused FP64", "config": {
                "workload": res.pop("workload"), "gates": res.pop("gates")}, **res, "data": "synthetic"}
    print(json.dumps(line))


def run_schrodinger(args):
    """QCSim's SchrodingerSimulation::Execute at full size: a Gaussian packet (2^n grid points) meeting a
    square barrier, Trotter steps through qcs_schrodinger_evolve.  Reported: device time per step (the
    potential and kinetic diagonals ride inside the IQFT / QFT shared-memory passes), the wall time of
    the whole Execute (host operator set-up, uploads and steps), the passes' roofline, and the CPU oracle
    (its QFT on all host threads) on one step of the same register"""
    import torch
    from qcsim_gb300 import _lib as L, circuits
    from qcsim_gb300.schrodinger import SchrodingerSimulation
    from oracle import bind as B, schrodinger as OS
    lib = L.load()
    n, steps = args.qubits, args.steps
    nb = 1 << n
    dt, dx = 0.002, 0.05
    sim = SchrodingerSimulation(n, dt, dx, steps)
    stream = torch.cuda.Stream()
    lib.qcs_set_stream(sim.reg.handle, stream.cuda_stream)
    sim.setGaussian(nb // 4, nb / 64.0, 20.0)
    sim.setConstantPotentialInTheMiddle(50.0, nb // 64)
    psi0 = sim.getRegisterStorage().copy()
    sim.setNrSteps(args.warmup)
    sim.Execute()  # warm-up (planning structures, allocations)
    sim.reg.setRegisterStorageFastNoNormalize(psi0)
    sim.setNrSteps(steps)
    torch.cuda.synchronize()
    sim.reg.profile(True)
    sim.reg.read_profile()
    t0 = time.perf_counter()
    sim.Execute()
    wall = time.perf_counter() - t0
    prof = sim.reg.read_profile(fp_ops=True)
    sim.reg.profile(False)
    launches, pass_ms, pass_bytes, _ = prof["tile_pass"]
    step_s = pass_ms / 1e3 / steps
    peak, peak_kind = peaks()
    s = 16
    qb = sum(algorithmic_bytes(op[0], n) for op in circuits.qft_circuit(0, n - 1))
    alg_step = 2 * qb + 2 * 3 * s * nb  # the two transforms' gates, and two diagonal sweeps (state in and out, table in)
    norm = float(np.linalg.norm(sim.getRegisterStorage()))
    # CPU: the oracle's steps (its QFT on all host threads) on the same start state, one step
    pot, kin = sim.Init()
    B.build_oracle()
    c0 = time.perf_counter()
    OS.evolve_with(psi0 / np.linalg.norm(psi0), n, pot, kin, 1)
    cpu_s = time.perf_counter() - c0
    line = {"metric": "Schrodinger split-operator Trotter steps/s", "value": 1.0 / step_s, "unit": "steps/s",
            "higher_is_better": True, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"SchrodingerSimulation, {n} qubits ({nb} grid points), dt {dt}, dx {dx}, Gaussian packet at "
                                   f"{nb // 4} on a barrier of height 50 and half-width {nb // 64}; {steps} timed steps",
                       "qubits": n, "steps": steps, "warmup_steps": args.warmup},
            "ms_per_step": step_s * 1e3, "passes_per_step": launches / steps,
            "execute_wall_seconds": wall, "norm_after": norm,
            "roofline": {"bound": "hbm", "achieved": alg_step / step_s / 1e9, "peak": peak, "unit": "GB/s",
                         "frac": alg_step / step_s / 1e9 / peak, "peak_source": peak_kind,
                         "algorithmic_bytes_per_step": alg_step,
                         "pass_GBps": pass_bytes / (pass_ms / 1e3) / 1e9},
            "cpu_baseline": {"value": 1.0 / cpu_s, "unit": "steps/s", "cores": B.oracle().qo_max_threads(), "kind": "port",
                             "sample": f"one step of the same {n}-qubit register, {cpu_s:.2f} s"}}
    print(json.dumps(line))


def main():
    args = parse()
    if args.config == "schrodinger":
        run_schrodinger(args)
        return
    if args.config == "precision":
        run_precision(args)
        return
    if args.config == "learned":
        run_learned(args)
        return
    if args.config == "qaoa":
        run_qaoa(args)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
