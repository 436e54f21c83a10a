"""Host-side checks that need no GPU: the gate library mirrors the reference's classes, the seeded
generators are deterministic, and libqcs_gpu.so loads and exports every entry point of
include/qcs_gpu.h (no compute calls)."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from qcsim_gb300 import _lib as L
from qcsim_gb300 import circuits, gates as G
from qcsim_gb300.rng import Mt19937_64
from oracle import bind

ROOT = Path(__file__).resolve().parents[1]


def test_gate_library_matches_reference(golden):
    p = tuple(golden["gate_params"])
    for code, m, k, t in zip(golden["gate_codes"], golden["gate_mats"], golden["gate_k"], golden["gate_traits"]):
        g = G.make(int(code), *p)
        d = 1 << int(k)
        assert g.getQubitsNumber() == k
        assert g.traits() == t, (code, g.traits(), t)
        got = np.ascontiguousarray(g.getRawOperatorMatrix()).reshape(-1).view(np.float64)
        assert np.array_equal(got, m[: 2 * d * d]), code


def test_gate_records_layout():
    rec = G.to_record(G.ControlledPhaseShiftGate(0.3), 4, 2)
    assert rec["k"] == 2 and rec["q0"] == 4 and rec["q1"] == 2
    assert rec["traits"] == L.TRAIT_CONTROLLED | L.TRAIT_DIAGONAL
    assert rec["m"][30] == np.cos(0.3) and rec["m"][31] == np.sin(0.3)
    assert L.GATE_DTYPE.itemsize == 6 * 4 + 128 * 8


def test_rng_matches_reference(golden):
    for row, seed in zip(golden["rng_uniforms"], (1, 7, 123456789)):
        m = Mt19937_64(seed)
        assert np.array_equal(np.array([m.uniform() for _ in range(row.size)]), row)


def test_layered_generator_shape():
    ops = circuits.layered_circuit(20, 40, seed=1)
    assert len(ops) == 40 * (20 + 10)
    ops2 = circuits.layered_circuit(20, 40, seed=1)
    assert all(type(a[0]) is type(b[0]) and a[1:] == b[1:] for a, b in zip(ops, ops2))
    ops3 = circuits.layered_circuit(30, 60, seed=1, p3=0.05)
    n3 = sum(1 for o in ops3 if o[0].getQubitsNumber() == 3)
    assert 60 <= n3 <= 230  # about 5% of 2700 positions
    for o in ops3:
        assert len(set(o[1:1 + o[0].getQubitsNumber()])) == o[0].getQubitsNumber()


def test_qaoa_instances():
    insts = circuits.qaoa_instances(16, seed=3)
    for inst in insts:
        n = inst["n"]
        assert n % 2 == 0 and 12 <= n <= 24
        deg = np.zeros(n, dtype=int)
        for i, j in inst["edges"]:
            assert i < j
            deg[i] += 1
            deg[j] += 1
        assert np.all(deg == 3)
        assert len(set(inst["edges"])) == len(inst["edges"])


def _declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:[A-Za-z_][\w\s\*]*?)\b(qcs_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return names


def test_c_abi_exports_every_declared_symbol():
    lib_path = L.LIB_PATH
    if not lib_path.exists():
        pytest.skip("libqcs_gpu.so not built")
    lib = C.CDLL(str(lib_path))
    declared = _declared_symbols()
    assert len(declared) >= 40
    missing = [n for n in sorted(declared) if not hasattr(lib, n)]
    assert not missing, missing
    # the Python binding declares exactly the header's entry points
    assert declared == set(L.SIGNATURES), declared ^ set(L.SIGNATURES)


def test_plain_c_caller(tmp_path):
    """include/qcs_gpu.h is plain C: tests/c_abi_consumer.c, compiled with gcc as C11 and linked with
    libqcs_gpu.so, calls the entry points that need no GPU (status strings, the reference's random stream,
    qcs_create's argument check, the gate-pass and fusion planning) and gets what the Python binding gets"""
    import shutil
    import subprocess
    from qcsim_gb300 import costmodel
    from qcsim_gb300.register import Rng
    if not L.LIB_PATH.exists():
        pytest.skip("libqcs_gpu.so not built")
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("gcc not found")
    exe = tmp_path / "c_abi_consumer"
    subprocess.run([gcc, "-std=c11", "-Wall", "-Wextra", "-Werror", f"-I{ROOT / 'include'}", str(ROOT / "tests" / "c_abi_consumer.c"),
                    f"-L{L.LIB_PATH.parent}", "-lqcs_gpu", f"-Wl,-rpath,{L.LIB_PATH.parent}", "-lm", "-o", str(exe)],
                   check=True, capture_output=True, text=True)
    out = dict(line.split(" ", 1) for line in subprocess.run([str(exe)], check=True, capture_output=True, text=True,
                                                              timeout=60).stdout.splitlines())
    assert out["status"] == "invalid argument"
    assert [float(x) for x in out["uniform"].split()] == Rng(7).uniform(3).tolist()
    assert int(out["create_zero_qubits"]) == L.QCS_INVALID_ARGUMENT
    # one pass: the 12 H gates as tile operations, the 4 RZ gates outside the tile as tile factors
    assert out["plan"].split() == ["0", "1", "16", "4"]
    ops = [(G.HadamardGate(), q) for q in range(12)] + [(G.RzGate(0.3 + 0.1 * q), q) for q in range(12, 16)]
    status, nblocks, folded = (int(x) for x in out["fusion"].split())
    assert status == 0 and folded == 16 and nblocks == len(costmodel.fusion_plan(16, G.records(ops), 4))


def test_status_strings_without_gpu():
    if not L.LIB_PATH.exists():
        pytest.skip("libqcs_gpu.so not built")
    lib = L.load()
    assert lib.qcs_status_string(L.QCS_INVALID_ARGUMENT) == b"invalid argument"
    # creation fails cleanly (no device here, or an invalid size)
    h = C.c_void_p()
    assert lib.qcs_create(0, L.QCS_FP64, C.byref(h)) == L.QCS_INVALID_ARGUMENT


def test_engine_rng_matches_reference(golden):
    if not L.LIB_PATH.exists():
        pytest.skip("libqcs_gpu.so not built")
    from qcsim_gb300.register import Rng
    for row, seed in zip(golden["rng_uniforms"], (1, 7, 123456789)):
        assert np.array_equal(Rng(seed).uniform(row.size), row)


def test_fusion_plan_covers_every_gate():
    """the greedy fuser (host code of the engine) keeps every gate, in blocks no wider than asked
    unless a single gate is wider"""
    if not L.LIB_PATH.exists():
        pytest.skip("libqcs_gpu.so not built")
    from qcsim_gb300 import costmodel
    for n, mq in ((20, 5), (24, 3), (30, 2), (12, 1)):
        ops = circuits.layered_circuit(n, 6, seed=n, p3=0.05, controlled_frac=0.1)
        plan = costmodel.fusion_plan(n, G.records(ops), mq)
        assert sum(ng for _, ng in plan) == len(ops)
        for mask, ng in plan:
            width = bin(mask).count("1")
            assert width <= max(mq, 3) and ng >= 1
    # wider blocks never mean more blocks
    ops = circuits.layered_circuit(26, 8, seed=3)
    counts = [len(costmodel.fusion_plan(26, G.records(ops), mq)) for mq in (2, 3, 4, 5)]
    assert counts == sorted(counts, reverse=True)


def _restated_gate_passes(layer, kmax: int, low_run: int, window: int = 64) -> int:
    """the gate-pass planner's packing rule, restated: each pass takes, in order and looking at most
    `window` gates ahead, every gate whose tile position (its target, unless the gate is diagonal) fits a
    tile of `kmax` qubits that always holds qubits 0..low_run-1, and which shares no qubit with an earlier
    gate left waiting"""
    masks = []
    for op in layer:
        g, k = op[0], op[0].getQubitsNumber()
        touch = 0
        for q in op[1:1 + k]:
            touch |= 1 << q
        masks.append((touch, 0 if g.traits() & L.TRAIT_DIAGONAL else 1 << op[1]))
    placed, first, passes = [False] * len(masks), 0, 0
    while True:
        while first < len(masks) and placed[first]:
            first += 1
        if first == len(masks):
            return passes
        tmask, waiting, scanned, taken = (1 << low_run) - 1, 0, 0, 0
        for i in range(first, len(masks)):
            if scanned >= window:
                break
            if placed[i]:
                continue
            scanned += 1
            touch, need = masks[i]
            if (touch & waiting) == 0 and (bin(tmask | need).count("1") <= kmax or taken == 0):
                placed[i], taken, tmask = True, taken + 1, tmask | need
            else:
                waiting |= touch
        passes += 1


def test_gate_pass_planning():
    """the pass planner of unfused gate lists (host code, qcs_plan_gate_passes): per layer of the 30-qubit
    layered circuit it forms exactly the passes of the restated packing rule (FP64: 12-qubit tiles, FP32:
    13, both holding the 16- or 32-amplitude low run); the diagonal gates outside a pass's tile merge into
    TileFactor operations only when two or more of them are phases or diagonals"""
    if not L.LIB_PATH.exists():
        pytest.skip("libqcs_gpu.so not built")
    import bench
    from qcsim_gb300 import costmodel
    layers = bench.layers_of(circuits.layered_circuit(30, 60, seed=1, p3=0.05), 30)
    for precision, kmax, low_run in (("fp64", 12, 4), ("fp32", 13, 5)):
        got = [len(costmodel.gate_passes(30, G.records(layer), precision)) for layer in layers]
        assert got == [_restated_gate_passes(layer, kmax, low_run) for layer in layers], precision
    r = np.random.default_rng(5)
    ops = [(G.HadamardGate(), q) for q in range(12)]
    for q in range(12, 18):
        ops.append((G.RzGate(float(r.uniform(0, 2 * np.pi))), q))
        ops.append((G.PhaseShiftGate(float(r.uniform(0, 2 * np.pi))), q))
    ops += [(G.ControlledPhaseShiftGate(0.7), 15, 13), (G.ControlledZGate(), 16, 12)]
    # FP64 tile = qubits 0-11: all 14 diagonal gates merge (the CZ's sign too); FP32 tile = 0-12: the phases
    # on qubit 12 stay tile operations and the CZ, with its control in the tile, stays its own operation
    assert costmodel.gate_passes(18, G.records(ops), "fp64") == [(26, 14)]
    assert costmodel.gate_passes(18, G.records(ops), "fp32") == [(26, 11)]
    assert costmodel.gate_passes(18, G.records(ops[:13]), "fp64") == [(13, 0)]  # a single non-tile phase
    assert costmodel.gate_passes(12, G.records(ops[:12]), "fp64") == []  # one kernel per gate below 14 qubits


def test_tensor_core_tile_swizzle():
    """the tensor-core pass's shared-memory swizzle (tc_swizzle in tile.cuh, read from the source): the
    low-four-bit vectors of the 12 tile bits' offsets are distinct and nonzero and avoid 0011, 1100 and
    1111, so any 7 of them span GF(2)^4; hence for every block on 4 or 5 tile bits, four of the other bits
    have independent vectors, and the 16 lanes of a half-warp that differ in those four row bits read 16
    different 8-byte bank pairs"""
    import itertools
    src = (ROOT / "qcsim_gb300" / "csrc" / "tile.cuh").read_text()
    table = int(re.search(r"\(0x([0-9A-Fa-f]+)ULL >> \(4 \* \(b - 4\)\)\)", src).group(1), 16)
    vec = [(1 << b) & 15 if b < 4 else (1 << b) & 15 ^ ((table >> (4 * (b - 4))) & 15) for b in range(12)]
    assert len(set(vec)) == 12 and 0 not in vec and not {0b0011, 0b1100, 0b1111} & set(vec)

    def rank(vs):
        span = {0}
        for v in vs:
            span |= {x ^ v for x in span}
        return len(span).bit_length() - 1

    assert all(rank(c) == 4 for c in itertools.combinations(vec, 7))
    for k in (4, 5):
        for block in itertools.combinations(range(12), k):
            others = [vec[b] for b in range(12) if b not in block]
            # the first four independent ones, as the host's row order picks them
            chosen = []
            for v in others:
                if len(chosen) < 4 and rank(chosen + [v]) > len(chosen):
                    chosen.append(v)
            lanes = set()
            for m in range(16):
                x = 0
                for r in range(4):
                    if (m >> r) & 1:
                        x ^= chosen[r]
                lanes.add(x)
            assert len(lanes) == 16, block


def test_pass_packing_respects_order_and_tiles():
    """the pass planner of the fused path (host code): every block lands in exactly one pass, a block
    never runs before an earlier block it shares a qubit with, every pass fits its tile, and look-ahead
    packing needs no more passes than packing strictly in order"""
    if not L.LIB_PATH.exists():
        pytest.skip("libqcs_gpu.so not built")
    from qcsim_gb300 import costmodel
    for n, mq, k, tc in ((26, 5, 12, True), (30, 3, 13, False), (24, 4, 12, True), (20, 2, 13, False)):
        ops = circuits.layered_circuit(n, 8, seed=n + mq, p3=0.05, controlled_frac=0.1)
        recs = G.records(ops)
        plan = costmodel.fusion_plan(n, recs, mq)
        passes = costmodel.fusion_passes(n, recs, mq, k, tc)
        assert len(passes) == len(plan)
        low = (1 << min(n, max(4, k - 8))) - 1  # the low run every tile holds (tile.cuh low_run_qubits)
        union: dict[int, int] = {}
        for (mask, _), p in zip(plan, passes):
            union[p] = union.get(p, low) | mask
        assert sorted(union) == list(range(len(union)))
        assert all(bin(m).count("1") <= k for m in union.values())
        for i in range(len(plan)):
            for j in range(i + 1, len(plan)):
                if plan[i][0] & plan[j][0]:
                    assert passes[i] <= passes[j], (i, j)
        # strictly in order: a new pass whenever the next block does not fit
        in_order, cur = 1, low
        for mask, _ in plan:
            if bin(cur | mask).count("1") > k:
                in_order, cur = in_order + 1, low | mask
            else:
                cur |= mask
        assert len(union) <= in_order


def test_block_features_layout():
    if not L.LIB_PATH.exists():
        pytest.skip("libqcs_gpu.so not built")
    from qcsim_gb300 import costmodel
    f = costmodel.features(30, (0, 5, 29), 7)
    assert f.shape == (costmodel.F,)
    assert f[0] == pytest.approx(3 / 5) and f[1] == pytest.approx(7 / 32) and f[2] == pytest.approx(30 / 32)
    assert f[5] == pytest.approx(1 / 5) and f[6] == pytest.approx(1 / 5) and f[10] == 1


def test_committed_cost_model_is_sane():
    """the GPU-trained cost model shipped with the package: its parameters load, the CPU restatement of
    the network predicts finite block times, a 5-qubit block of six gates costs less per gate than a
    one-gate 1-qubit block, the same block costs more on 30 than on 26 qubits, and the per-size pass
    times (CUDA-core and tensor-core) double with each qubit"""
    from qcsim_gb300 import costmodel as cm
    d = np.load(cm.MODEL_DIR / "fusion_cost_mlp.npz")
    ref = cm.MlpRef(d["params"].astype(np.float64))
    x = np.stack([cm.features(30, [3], 1), cm.features(30, [2, 7, 11, 20, 29], 6),
                  cm.features(26, [2, 7, 11, 20, 25], 6)]).astype(np.float64)
    y = np.exp(ref.forward(x).reshape(-1))
    assert np.all(np.isfinite(y)) and y[1] / 6 < y[0] and y[1] > y[2]
    pm = d["pass_ms"]
    assert all(1.6 < pm[n + 1] / pm[n] < 2.4 for n in range(24, 32))
    assert all(1.6 < pm[64 + n + 1] / pm[64 + n] < 2.4 for n in range(24, 32))


def test_records_match_to_record():
    """the whole-list conversion gives, byte for byte, the records to_record makes one gate at a time: reused
    and distinct gate objects, parametrised gates, matrix-only gates of 1-3 qubits, short (gate, q0) tuples"""
    from qcsim_gb300 import circuits
    from qcsim_gb300 import gates as G
    rng = np.random.default_rng(4)
    h, ccx = G.HadamardGate(), G.ToffoliGate()
    ops = circuits.layered_circuit(12, 4, seed=9, controlled_frac=0.2)
    ops += [(h, 3), (ccx, 5, 1, 2), (h, 0), (ccx, 2, 0, 1), (G.RzGate(0.7), 4)]
    for k in (1, 2, 3):
        d = 1 << k
        m = rng.standard_normal((d, d)) + 1j * rng.standard_normal((d, d))
        ops.append((G.AppliedGate(m, 0, 1, 2), *range(k)))
    ops = [ops[i] for i in rng.permutation(len(ops))]
    want = np.zeros(len(ops), dtype=L.GATE_DTYPE)
    for i, op in enumerate(ops):
        qs = list(op[1:]) + [0, 0]
        G.to_record(op[0], qs[0], qs[1], qs[2], out=want[i])
    assert G.records(ops).tobytes() == want.tobytes()
    assert G.records([]).size == 0


@pytest.mark.skipif(not bind.DROPIN_LIB.exists(), reason="needs QCSim's sources staged and make -C oracle dropin")
def test_reference_driver_builds_on_the_dropin():
    """ref_driver.cpp compiled against the drop-in register loads (no GPU call) and exports the same entry
    points as the compiled reference, and QCSim's test-suite program over the drop-in is built"""
    lib = C.CDLL(str(bind.DROPIN_LIB))
    missing = [name for name in bind._REF_SIG if not hasattr(lib, name)]
    assert not missing, missing
    assert bind.SUITE_BIN.exists()
