"""The benchmark's output contract on CPU: the reference arm (the CPU reference on the bench workload)
prints one JSON line with the required keys, and the roofline helpers compute algorithmic bandwidth,
physical pass bandwidth and scaled DRAM traffic as documented."""
import json
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))


def test_reference_arm_prints_one_contract_line():
    from oracle import bind
    bind.build_oracle()
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--qubits", "14", "--steps", "2",
                        "--warmup", "1", "--cpu-gates", "30"], capture_output=True, text=True, cwd=ROOT, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
                "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e", "impl"):
        assert key in d, key
    assert d["impl"] == "reference" and d["unit"] == "gates/s" and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    # QCSim's own register where its sources are staged (oracle/_ref), else the oracle's restatement
    want = "reference" if bind.STAGED_SRC.is_dir() else "port"
    assert d["cpu_baseline"]["kind"] == want and d["cpu_baseline"]["cores"] >= 1


def test_roofline_helpers():
    import bench
    # two launches of a pass family that carried every launch: algorithmic bytes = the gates' bytes
    prof = {"tile_pass": (2, 10.0, 2 * 34359738368.0)}
    r = bench.roofline_of(prof, 6791.0, "measured", 30, 10 * 34359738368.0)
    assert r["launches"] == 2 and r["avg_launch_ms"] == pytest.approx(5.0)
    assert r["algorithmic_bytes_per_launch"] == pytest.approx(5 * 34359738368.0)
    assert r["achieved"] == pytest.approx(5 * 34359738368.0 / 5e-3 / 1e9)
    assert r["pass_GBps"] == pytest.approx(34359738368.0 / 5e-3 / 1e9)
    assert r["frac"] == pytest.approx(r["achieved"] / 6791.0)
    # the committed 26-qubit ncu capture scales with the amplitude count
    t26, t30 = bench.read_traffic("tile_pass", 26), bench.read_traffic("tile_pass", 30)
    assert t26 is not None and t30 == pytest.approx(16 * t26)
    assert bench.read_traffic("no_such_kernel", 30) is None
    # a family that did not carry every launch keeps its own byte count
    prof = {"tile_pass": (2, 10.0, 4.0e9), "ctrl1q_swap": (1, 1.0, 1.0e9)}
    r = bench.roofline_of(prof, 6791.0, "measured", 30, 123.0)
    assert r["algorithmic_bytes_per_launch"] == pytest.approx(2.0e9)


def test_fp64_roofline_helper():
    import bench
    prof = {"tile_pass": (4, 100.0, 4 * 34359738368.0, 4 * 2.0e10)}
    r = bench.fp64_roofline_of(prof, "tile_pass", 1.2)
    assert r["bound"] == "fp64" and r["fp_ops_per_launch"] == pytest.approx(2.0e10)
    assert r["achieved"] == pytest.approx(8.0e10 / 0.1 / 1e12)
    assert r["peak"] == pytest.approx(0.6) and r["frac"] == pytest.approx(r["achieved"] / 0.6)


def test_parity_helpers():
    """the parity leg's helpers: the identity rate of two shot histograms of the same uniforms, the count
    of uniforms within eps of a cumulative-table entry (chunked as on a 30-qubit state), the layer split
    of the layered circuit, and the oracle's max amplitude difference"""
    import numpy as np
    import bench
    from qcsim_gb300 import circuits
    assert bench.shot_identity({1: 3, 2: 1}, {1: 3, 2: 1}, 4) == 1.0
    assert bench.shot_identity({1: 3, 2: 1}, {1: 2, 3: 2}, 4) == 0.5
    assert bench.shot_identity({}, {}, 0) == 1.0
    state = np.sqrt(np.array([0.25, 0.25, 0.5], dtype=np.complex128))  # cumulative table 0.25, 0.5, 1.0
    probs = np.array([0.1, 0.25 + 1e-14, 0.5 - 1e-13, 0.75, 1.0 - 1e-15])
    for chunk in (1, 2, 1 << 24):
        assert bench.shots_near_boundary(state, probs, 1e-12, chunk=chunk) == 3
    ops = circuits.layered_circuit(12, 5, seed=2, p3=0.05)
    layers = bench.layers_of(ops, 12)
    assert len(layers) == 5 and sum(map(len, layers)) == len(ops)
    assert all(sum(type(o[0]).__name__ == "CNOTGate" for o in layer) == 6 for layer in layers)
    from oracle import bind
    bind.build_oracle()
    a = np.array([1 + 2j, 3 - 1j, 0.5j])
    assert bench.max_abs_diff(a, a + np.array([0, 1e-9, 0])) == pytest.approx(1e-9)
