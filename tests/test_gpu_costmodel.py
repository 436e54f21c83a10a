"""Learned fusion: the engine's MLP kernels against the CPU restatement (gradients), training, and the
learned partition choice on the FP32 path."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cm():
    from qcsim_gb300 import _lib, costmodel
    _lib.load()
    return costmodel


def test_gradient_matches_cpu(cm):
    rng = np.random.default_rng(0)
    mlp = cm.Mlp(cm.F, seed=3)
    x = rng.uniform(0, 1, (300, cm.F)).astype(np.float32)
    t = rng.standard_normal(300).astype(np.float32)
    g, loss = mlp.gradient(x, t)
    ref = cm.MlpRef(mlp.params())
    rloss, rg = ref.loss_and_grad(x.astype(np.float64), t.astype(np.float64))
    assert abs(loss - rloss) <= 1e-4 * max(1.0, abs(rloss))
    assert np.abs(g - rg).max() <= 1e-4 * max(1.0, np.abs(rg).max())
    # and a finite-difference check of the CPU gradient on a few parameters
    p = mlp.params().astype(np.float64)
    for i in rng.choice(p.size, 8, replace=False):
        e = np.zeros_like(p)
        e[i] = 1e-4
        lp = cm.MlpRef(p + e).loss_and_grad(x, t)[0]
        lm = cm.MlpRef(p - e).loss_and_grad(x, t)[0]
        assert abs((lp - lm) / 2e-4 - rg[i]) <= 1e-3 * max(1.0, abs(rg[i]))


def test_predict_matches_cpu(cm):
    rng = np.random.default_rng(1)
    mlp = cm.Mlp(cm.F, seed=5)
    x = rng.uniform(0, 1, (1000, cm.F)).astype(np.float32)
    y = mlp.predict(x)
    ref = cm.MlpRef(mlp.params()).forward(x.astype(np.float64))
    assert np.abs(y - ref).max() <= 1e-4 * max(1.0, np.abs(ref).max())


def test_training_fits_a_smooth_target(cm):
    rng = np.random.default_rng(2)
    x = rng.uniform(0, 1, (2048, cm.F)).astype(np.float32)
    t = (np.sin(3 * x[:, 0]) + x[:, 1] * x[:, 2] - 0.5 * x[:, 3]).astype(np.float32)
    mlp = cm.Mlp(cm.F, seed=7)
    before = float(np.mean((mlp.predict(x) - t) ** 2))
    after = mlp.train(x, t, steps=1500, lr=3e-3)
    assert after < 0.05 * before and after < 1e-2


def test_learned_partition_runs_and_matches(cm):
    """fusion mode 2 with an (untrained) model still computes the same state: any partition is exact"""
    from qcsim_gb300 import QubitRegister, circuits
    from test_gpu_parity import oracle_state
    n = 16
    ops = circuits.layered_circuit(n, 6, seed=31, controlled_frac=0.1)
    mlp = cm.Mlp(cm.F, seed=9)
    reg = QubitRegister(n, seed=1, precision="fp32")
    cm.attach(reg, mlp, np.full(64, 1.0))
    reg.ApplyGates(ops)
    got = reg.getRegisterStorage()
    want = oracle_state(n, ops)
    assert np.abs(got - want).max() < 2e-6


def test_apply_matrix_any_order(cm):
    """qcs_apply_matrix: matrix bit j is qubits[j], in any order"""
    from qcsim_gb300 import QubitRegister, gates as G
    from test_gpu_parity import oracle_state, rand_state
    rng = np.random.default_rng(4)
    n = 15
    init = rand_state(n, 3)
    for prec, k in (("fp64", 3), ("fp32", 5), ("fp64", 4)):
        qs = [int(x) for x in rng.choice(n, size=k, replace=False)]
        u = cm.random_unitary(k, rng)
        reg = QubitRegister(n, seed=1, precision=prec)
        reg.setRegisterStorageFastNoNormalize(init)
        cm.apply_matrix(reg, qs, u)
        # the same operator as a product of matrix-only gates is not available for k > 3; compare with
        # a dense CPU application
        want = init.reshape([2] * n)
        axes = [n - 1 - q for q in reversed(qs)]  # tensor axes of the qubits, matrix bit k-1 first
        t = np.moveaxis(want, axes, list(range(k))).reshape(1 << k, -1)
        t = (u @ t).reshape([2] * k + [2] * (n - k))
        want = np.moveaxis(t, list(range(k)), axes).reshape(-1)
        tol = 1e-12 if prec == "fp64" else 2e-6
        assert np.abs(reg.getRegisterStorage() - want).max() <= tol, (prec, k, qs)
    _ = (G, oracle_state)


LEARNED_MARGIN = 0.98  # the learned partition's time must be at most this fraction of greedy <=3's
BEST_SLACK = 1.15      # ... and at most this multiple of the fastest greedy partition's


def test_trained_model_beats_the_fixed_fuser(cm):
    """the committed, GPU-trained cost model against the method without it, on an unseen 26-qubit circuit
    of depth 12 with 10% controlled rotations: the learned partition must take at most LEARNED_MARGIN of
    the time of greedy blocks of at most 3 qubits on the CUDA cores, and at most BEST_SLACK of the fastest
    greedy partition (largest block 3, 4 or 5, found here by timing all three, which the model does not
    do); every FP32 result stays within 1-F <= 1e-6 of the FP64 path."""
    import ctypes as C
    import torch
    from qcsim_gb300 import QubitRegister, _lib as L, circuits, gates as G
    lib = L.load()
    n = 26
    ops = circuits.layered_circuit(n, 12, seed=4242, controlled_frac=0.1)
    recs = G.records(ops)
    mlp, pass_ms = cm.load()
    ref = QubitRegister(n, seed=1)
    ref.apply_records(recs)

    def run(setup):
        reg = QubitRegister(n, seed=1, precision="fp32")
        setup(reg)
        reg.apply_records(recs)  # planning and first-touch warm-up
        best = 1e9
        for _ in range(3):
            reg.setToBasisState(0)
            torch.cuda.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            reg.apply_records(recs)
            b.record()
            b.synchronize()
            best = min(best, a.elapsed_time(b))
        f, d = C.c_double(), C.c_double()
        L.check(lib.qcs_compare(ref.handle, reg.handle, C.byref(f), C.byref(d)), ref.handle)
        reg.close()
        return best, 1.0 - f.value

    t_greedy5, inf_greedy5 = run(lambda r: r.set_fusion(1, 5))
    t_greedy4, inf_greedy4 = run(lambda r: r.set_fusion(1, 4))
    t_greedy3, inf_greedy3 = run(lambda r: r.set_fusion(1, 3))
    t_learned, inf_learned = run(lambda r: cm.attach(r, mlp, pass_ms))
    assert max(inf_greedy5, inf_greedy4, inf_greedy3, inf_learned) <= 1e-6
    t_best = min(t_greedy3, t_greedy4, t_greedy5)
    print(f"learned {t_learned:.2f} ms, greedy<=3 {t_greedy3:.2f} ms, greedy<=4 {t_greedy4:.2f} ms, greedy<=5 {t_greedy5:.2f} ms")
    assert t_learned <= LEARNED_MARGIN * t_greedy3, (t_learned, t_greedy3, t_greedy5)
    assert t_learned <= BEST_SLACK * t_best, (t_learned, t_greedy3, t_greedy5)
