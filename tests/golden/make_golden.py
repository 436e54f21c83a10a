"""Generate tests/golden/golden.npz from QCSim's own QubitRegister (the compiled reference).

Run in a checkout that has the QCSim sources (oracle/Makefile target `ref` builds
oracle/_ref/libqcsref.so from them):

    make -C oracle ref && python tests/golden/make_golden.py

The fixtures pin the CPU oracle (tests/test_oracle_golden.py) and, through it, the GPU engine.
Everything below is produced by the reference's code paths: its gate classes, ApplyGate dispatch,
measurement scans, QFT sub-algorithm and QAOA circuit builder.
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import bind as B  # noqa: E402
from qcsim_gb300 import circuits, gates as G  # noqa: E402

OUT = Path(__file__).resolve().parent / "golden.npz"

PARAMS = (0.7, 0.3, -1.1, 0.25)
C0_PROBE = 256  # amplitudes recorded from each 20-qubit state


def uniforms(seed: int, n: int, lib=None) -> np.ndarray:
    u = np.zeros(n)
    (lib if lib is not None else B.ref()).qr_uniforms(seed, n, B.dp(u))
    return u


def random_ops(rng: np.random.Generator, n: int, count: int, codes) -> list:
    ops = []
    for _ in range(count):
        code = int(rng.choice(codes))
        g = G.make(code, *rng.uniform(0, 2 * np.pi, 4))
        qs = [int(x) for x in rng.choice(n, size=3, replace=False)]
        ops.append((g, *qs))
    return ops


def generate(lib=None) -> dict[str, np.ndarray]:
    """every fixture array, produced through ref_driver.cpp's entry points in `lib` (default: the
    compiled reference, B.ref(); B.ref_dropin() runs the same driver over the GPU drop-in register)"""
    r = lib if lib is not None else B.ref()
    out: dict[str, np.ndarray] = {}

    # 1. gate matrices and traits of every reference gate class
    codes = sorted(G.BY_CODE)
    mats = np.zeros((len(codes), 128))
    ks = np.zeros(len(codes), dtype=np.uint32)
    trs = np.zeros(len(codes), dtype=np.uint32)
    for i, code in enumerate(codes):
        rec = B.records([(G.make(code, *PARAMS), 0, 1, 2)])
        k, t = C.c_uint32(), C.c_uint32()
        r.qr_gate_matrix(rec.ctypes.data_as(C.c_void_p), B.dp(mats[i]), C.byref(k), C.byref(t))
        ks[i], trs[i] = k.value, t.value
    out["gate_codes"] = np.array(codes, dtype=np.int32)
    out["gate_params"] = np.array(PARAMS)
    out["gate_mats"], out["gate_k"], out["gate_traits"] = mats, ks, trs

    # 2. random circuits over every gate class (and matrix-only gates), n = 3..10
    rng = np.random.default_rng(20240611)
    circ_recs, circ_n, circ_states = [], [], []
    for t in range(24):
        n = 3 + t % 8
        ops = random_ops(rng, n, 40, codes)
        if t % 3 == 0:  # matrix-only (AppliedGate) gates dispatch to the dense paths
            for k in (1, 2, 3):
                a = rng.standard_normal((1 << k, 1 << k)) + 1j * rng.standard_normal((1 << k, 1 << k))
                q, _ = np.linalg.qr(a)
                qs = [int(x) for x in rng.choice(n, size=3, replace=False)]
                ops.append((G.AppliedGate(q, *qs), *qs))
        recs = B.records(ops)
        reg = B.RefRegister(n, lib=r)
        reg.apply(recs)
        circ_recs.append(recs)
        circ_n.append(n)
        circ_states.append(reg.state())
    out["circ_n"] = np.array(circ_n)
    out["circ_len"] = np.array([len(x) for x in circ_recs])
    out["circ_recs"] = np.concatenate(circ_recs)
    out["circ_states"] = np.concatenate(circ_states)

    # 3. layered circuit, 12 qubits, depth 10, Toffoli/CCZ at 5% of positions: full state, qubit
    #    probabilities, RepeatedMeasure(1024) with rng seed 7, then MeasureAll
    ops = circuits.layered_circuit(12, 10, seed=4, p3=0.05)
    reg = B.RefRegister(12, seed=7, lib=r)
    reg.apply(ops)
    out["l12_recs"] = B.records(ops)
    out["l12_state"] = reg.state()
    out["l12_qprob"] = np.array([r.qr_qubit_probability(reg.h, q) for q in range(12)])
    h = reg.repeated_measure(1024)
    out["l12_hist"] = np.array(sorted(h.items()), dtype=np.uint64)
    out["l12_measure_all"] = np.array([r.qr_measure_all(reg.h)], dtype=np.uint64)

    # 4. the 20-qubit layered workload, depth 40, seeds 1..3: probe amplitudes, qubit probabilities,
    #    1024 shots with rng seed s (full states are regenerated by the oracle)
    probe = np.random.default_rng(99).choice(1 << 20, size=C0_PROBE, replace=False).astype(np.uint64)
    out["c0_probe_idx"] = np.sort(probe)
    c0_amp, c0_qp, c0_hist, c0_norm = [], [], [], []
    for s in (1, 2, 3):
        ops = circuits.layered_circuit(20, 40, seed=s)
        reg = B.RefRegister(20, seed=s, lib=r)
        reg.apply(ops)
        st = reg.state()
        c0_amp.append(st[out["c0_probe_idx"]])
        c0_qp.append([r.qr_qubit_probability(reg.h, q) for q in range(20)])
        hh = reg.repeated_measure(1024)
        c0_hist.append(np.array(sorted(hh.items()), dtype=np.uint64))
        c0_norm.append(float(np.sum(np.abs(st) ** 2)))
    out["c0_amp"] = np.array(c0_amp)
    out["c0_qprob"] = np.array(c0_qp)
    out["c0_hist_len"] = np.array([len(x) for x in c0_hist])
    out["c0_hist"] = np.concatenate(c0_hist)
    out["c0_norm"] = np.array(c0_norm)

    # 5. measurement known answers on 1/2|00> - i/2|01> + 1/sqrt(2)|11> (MeasurementsTests.cpp:34-43):
    #    MeasureQubit(0), MeasureQubit(1), Measure(0, 1), MeasureAll, MeasureNoCollapse for 16 seeds each
    kat = np.zeros(4, dtype=np.complex128)
    kat[0], kat[1], kat[3] = 0.5, -0.5j, 1 / np.sqrt(2)
    out["kat_state"] = kat
    rows = []
    states_after = []
    for s in range(16):
        for op in range(5):
            reg = B.RefRegister(2, seed=1000 + s, lib=r)
            reg.set_state(kat)
            r.qr_normalize(reg.h)
            if op == 0:
                v = r.qr_measure_qubit(reg.h, 0)
            elif op == 1:
                v = r.qr_measure_qubit(reg.h, 1)
            elif op == 2:
                v = r.qr_measure(reg.h, 0, 1)
            elif op == 3:
                v = r.qr_measure_all(reg.h)
            else:
                v = r.qr_measure_no_collapse(reg.h)
            rows.append((s, op, v))
            states_after.append(reg.state())
    out["kat_rows"] = np.array(rows, dtype=np.uint64)
    out["kat_after"] = np.array(states_after)

    # 6. sub-register measurements on a 10-qubit random state (Measure(first, second) with collapse,
    #    RepeatedMeasure(first, second, 500))
    v = rng.standard_normal(1 << 10) + 1j * rng.standard_normal(1 << 10)
    v /= np.linalg.norm(v)
    out["sub_state"] = v
    sub_rows, sub_after, sub_hist = [], [], []
    for (a, b) in ((0, 0), (3, 5), (2, 9), (9, 9), (0, 9)):
        reg = B.RefRegister(10, seed=31 + a * 10 + b, lib=r)
        reg.set_state(v)
        val = r.qr_measure(reg.h, a, b)
        sub_rows.append((a, b, val))
        sub_after.append(reg.state())
        reg2 = B.RefRegister(10, seed=77 + a * 10 + b, lib=r)
        reg2.set_state(v)
        hh = reg2.repeated_measure(500, a, b)
        sub_hist.append(np.array([(a, b, k, c) for k, c in sorted(hh.items())], dtype=np.uint64))
    out["sub_rows"] = np.array(sub_rows, dtype=np.uint64)
    out["sub_after"] = np.array(sub_after)
    out["sub_hist"] = np.concatenate(sub_hist)

    # 7. edge cases of the scans: a state with total probability 0.81 (scans fall off the end:
    #    MeasureAll -> last state, MeasureNoCollapse -> 0, RepeatedMeasure -> table size)
    w = v * 0.9
    out["edge_state"] = w
    edge = []
    for s in range(12):
        reg = B.RefRegister(10, seed=500 + s, lib=r)
        reg.set_state(w)
        a1 = r.qr_measure_no_collapse(reg.h)
        hh = reg.repeated_measure(64)
        reg.set_state(w)
        a0 = r.qr_measure_all(reg.h)
        edge.append([s, a0, a1] + [k for k in sorted(hh) for _ in range(hh[k])])
    out["edge_rows"] = np.array(edge, dtype=np.uint64)

    # 8. QFT / IQFT (the reference sub-algorithm) on basis states and on a random state
    qft_in, qft_out, qft_cfg = [], [], []
    for (n, s0, e0, inv, sw, basis) in ((6, 0, 5, 0, 1, 1), (6, 0, 5, 1, 1, 1), (8, 0, 7, 0, 1, -1),
                                         (8, 2, 6, 0, 1, -1), (8, 1, 7, 1, 0, -1), (9, 0, 8, 0, 0, 5)):
        if basis >= 0:
            st = np.zeros(1 << n, dtype=np.complex128)
            st[basis] = 1
        else:
            st = rng.standard_normal(1 << n) + 1j * rng.standard_normal(1 << n)
            st /= np.linalg.norm(st)
        reg = B.RefRegister(n, lib=r)
        reg.set_state(st)
        r.qr_qft(reg.h, n, s0, e0, inv, sw)
        qft_in.append(np.pad(st, (0, 512 - st.size)))
        qft_out.append(np.pad(reg.state(), (0, 512 - st.size)))
        qft_cfg.append((n, s0, e0, inv, sw))
    out["qft_in"], out["qft_out"], out["qft_cfg"] = np.array(qft_in), np.array(qft_out), np.array(qft_cfg)

    # 9. QAOA circuits (QAOAIsingSubalgorithm::Exec) and Ising energies on small instances
    insts = circuits.qaoa_instances(4, seed=8, nmin=6, nmax=10, p=2)
    qa_states, qa_meta, qa_energy = [], [], []
    for inst in insts:
        n = inst["n"]
        e = np.array(inst["edges"], dtype=np.uint32).reshape(-1)
        J, hv = np.array(inst["J"]), np.array(inst["h"])
        gm, bt = np.array(inst["gammas"]), np.array(inst["betas"])
        reg = B.RefRegister(n, lib=r)
        r.qr_qaoa_exec(reg.h, n, len(inst["edges"]), e.ctypes.data_as(C.POINTER(C.c_uint32)), B.dp(J), B.dp(hv),
                       len(gm), B.dp(gm), B.dp(bt))
        qa_states.append(np.pad(reg.state(), (0, 1024 - (1 << n))))
        qa_energy.append([r.qr_ising_energy(n, len(inst["edges"]), e.ctypes.data_as(C.POINTER(C.c_uint32)), B.dp(J),
                                            B.dp(hv), x) for x in range(1 << n)] + [0.0] * (1024 - (1 << n)))
        qa_meta.append(n)
    out["qaoa_n"] = np.array(qa_meta)
    out["qaoa_states"] = np.array(qa_states)
    out["qaoa_energy"] = np.array(qa_energy)
    out["qaoa_seed"] = np.array([8, 6, 10, 2])

    # 10. ExpectationValue of matrix-only gates, and Compute / Uncompute replay
    ops = random_ops(rng, 6, 30, codes)
    exp_ops = random_ops(rng, 6, 5, [c for c in codes if c < 40])
    exp_gates = [(G.AppliedGate(g.getRawOperatorMatrix(), a, b, c), a, b, c) for (g, a, b, c) in exp_ops]
    reg = B.RefRegister(6, lib=r)
    reg.apply(ops)
    re, im = C.c_double(), C.c_double()
    recs = B.records(exp_gates)
    r.qr_expectation(reg.h, recs.ctypes.data_as(C.c_void_p), len(recs), C.byref(re), C.byref(im))
    out["exp_recs"], out["exp_pre"] = B.records(ops), recs
    out["exp_value"] = np.array([re.value, im.value])
    out["exp_state_after"] = reg.state()
    replay = []
    for mode in (1, 2):
        reg = B.RefRegister(6, lib=r)
        rr = B.records(ops)
        r.qr_record_and_replay(reg.h, rr.ctypes.data_as(C.c_void_p), len(rr), mode)
        replay.append(reg.state())
    out["replay_states"] = np.array(replay)

    # 11. the reference's random stream: uniforms of std::mt19937_64(seed) for three seeds
    out["rng_uniforms"] = np.array([uniforms(s, 64, r) for s in (1, 7, 123456789)])

    return out


def main() -> None:
    if not B.ref_available():
        raise SystemExit("oracle/_ref/libqcsref.so missing: run `make -C oracle ref` in a QCSim checkout")
    np.savez_compressed(OUT, **generate())
    print(f"wrote {OUT} ({OUT.stat().st_size / 1024:.0f} KiB)")


if __name__ == "__main__":
    main()
