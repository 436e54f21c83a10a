"""QCSim's own C++ code, unmodified, running on the GPU drop-in register.

Two programs are built from QCSim's sources with qcsim_gb300/cpp ahead of them on the include path
(oracle/Makefile target `dropin`), so every QC::QubitRegister they create is the GPU-backed drop-in that
forwards to libqcs_gpu.so through the C ABI:

- oracle/_ref/qcsim_tests_dropin: QCSim's statevector test functions (Tests.cpp, GatesTests.cpp,
  MeasurementsTests.cpp, AdderTests.cpp, ... , VQETests.cpp) in the order of its tests(0) chain
  (Tests.cpp:761-785), each with the reference's own pass condition.
- oracle/_ref/libqcsref_dropin.so: ref_driver.cpp (the driver that produced the golden fixtures from
  QCSim's own register) over the drop-in.  Re-running each fixture generator through it must give the
  committed fixtures: 1e-12 on amplitudes, probabilities and energies; identical measurement outcomes
  and histograms (the drop-in keeps the reference's mt19937_64 stream on the host).

Both need QCSim's sources staged into oracle/_ref/src (make -C oracle stage); without them the tests
skip and say so.
"""
import importlib
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / "tests" / "golden"
TOL = 1e-12

SUITE = ["basicTests", "quantumAdderTests", "DeutschJozsaTests", "SimonTests", "BernsteinVaziraniTests", "GroverTests",
         "PhaseEstimationTests", "ShorTests", "TeleportationTests", "SuperdenseCodingTests", "QuantumCryptograpyTests",
         "ParadoxesTests", "GamesTests", "distributedTests", "CountingTests", "QMLTests", "IsingTests", "VQETests"]


@pytest.fixture(scope="module")
def bind():
    from qcsim_gb300 import _lib
    try:
        _lib.load()
    except _lib.EngineUnavailable as e:
        pytest.fail(f"engine not built: {e}")
    from oracle import bind as B
    if not B.STAGED_SRC.is_dir():
        pytest.skip("QCSim's sources are not staged (make -C oracle stage QCSIM_SRC=...)")
    if not (B.DROPIN_LIB.exists() and B.SUITE_BIN.exists()):
        B.build_oracle(dropin=True)
    return B


def test_qcsim_statevector_suite_on_dropin(bind):
    """every function of QCSim's statevector test chain passes with the GPU register"""
    r = subprocess.run([str(bind.SUITE_BIN)], capture_output=True, text=True, timeout=1500)
    results = {}
    for ln in r.stdout.splitlines():
        if ln.startswith("@@ "):
            _, name, ok, secs = ln.split()
            results[name] = (ok == "1", float(secs))
    failed = [k for k, (ok, _) in results.items() if not ok]
    assert not failed and r.returncode == 0, (failed, r.returncode, r.stdout[-3000:], r.stderr[-2000:])
    assert list(results) == SUITE, list(results)
    print({k: round(v[1], 2) for k, v in results.items()})


def _same(name: str, a: np.ndarray, b: np.ndarray) -> None:
    """integers exactly; floating point to TOL; records field by field.  Inputs the generators draw
    through LAPACK (the random unitaries of np.linalg.qr) differ in the last bits between hosts, so
    the gate records that carry them are compared like every other floating-point value."""
    assert a.shape == b.shape, name
    if a.dtype.names:
        for f in a.dtype.names:
            _same(f"{name}.{f}", a[f], b[f])
    elif a.dtype.kind in "iu":
        assert np.array_equal(a, b), name
    elif a.size:
        err = float(np.abs(a - b).max())
        assert err <= TOL, (name, err)


def _compare(out: dict, want) -> None:
    assert set(out) <= set(want.files), set(out) - set(want.files)
    for k, a in out.items():
        _same(k, np.asarray(a), want[k])


@pytest.mark.parametrize("generator,fixture", [("make_golden", "golden"), ("make_algorithms", "algorithms"),
                                               ("make_oracles", "oracles"), ("make_pauli", "pauli"),
                                               ("make_nqubits", "nqubits")])
def test_reference_driver_on_dropin_reproduces_fixtures(bind, generator, fixture):
    """the fixture generators re-run through ref_driver.cpp over the drop-in reproduce what QCSim's own
    register produced: gate matrices and traits, random circuits, measurements and their collapse, the
    QFT, QAOA circuits, ExpectationValue and Compute/Uncompute replay (golden); Grover, the Draper adders,
    phase estimation, VQE's ansatz, Shor's period finding and quantum counting (algorithms); the
    gate-built oracles (oracles); the Pauli-string Hamiltonian simulation (pauli); the N-qubit operator
    gates (nqubits)"""
    if str(GOLDEN) not in sys.path:
        sys.path.insert(0, str(GOLDEN))
    gen = importlib.import_module(generator)
    kwargs = {"max_shor_qubits": 8} if generator == "make_algorithms" else {}
    out = gen.generate(bind.ref_dropin(), **kwargs)
    _compare(out, np.load(GOLDEN / f"{fixture}.npz"))
