"""Seeded synthetic workloads: layered random circuits, the QFT gate list, random 3-regular QAOA
instances.  Circuits are lists of (gate, q0, q1, q2) tuples, i.e. ApplyGate's arguments.

Layered random circuit (seed s, n qubits, depth d): a Mt19937_64(s) stream drives everything.  Each
layer draws, for q = 0..n-1, a gate type in {H, RX, RY, RZ} and an angle uniform in [0, 2*pi) (drawn
for every slot, unused by H); then a Fisher-Yates shuffle p of 0..n-1 and CNOTs with target p[2i+1]
and control p[2i].  With p3 > 0, after every gate a uniform draw below p3 inserts a Toffoli or CCZ
(one more draw picks which) on three distinct uniformly drawn qubits (the first is the target).
"""
from __future__ import annotations

import math

import numpy as np

from . import gates as G
from .rng import Mt19937_64

TWO_PI = 2.0 * math.pi


def layered_circuit(n: int, depth: int, seed: int, p3: float = 0.0, controlled_frac: float = 0.0) -> list:
    g = Mt19937_64(seed)
    ops: list = []

    def maybe_3q():
        if p3 > 0.0 and n >= 3 and g.uniform() < p3:
            cls = G.ToffoliGate if g.uniform() < 0.5 else G.CCZGate
            qs: list[int] = []
            while len(qs) < 3:
                q = g.randint(n)
                if q not in qs:
                    qs.append(q)
            ops.append((cls(), qs[0], qs[1], qs[2]))

    for _ in range(depth):
        for q in range(n):
            kind = g.randint(4)
            theta = g.uniform() * TWO_PI
            if controlled_frac > 0.0 and n >= 2 and g.uniform() < controlled_frac:
                # a controlled rotation with a random control in place of the 1-qubit slot
                c = g.randint(n - 1)
                c = c + 1 if c >= q else c
                cls = (G.ControlledRxGate, G.ControlledRyGate, G.ControlledRzGate, G.ControlledPhaseShiftGate)[kind]
                ops.append((cls(theta), q, c, 0))
            elif kind == 0:
                ops.append((G.HadamardGate(), q, 0, 0))
            else:
                cls = (None, G.RxGate, G.RyGate, G.RzGate)[kind]
                ops.append((cls(theta), q, 0, 0))
            maybe_3q()
        perm = list(range(n))
        for i in range(n - 1, 0, -1):
            j = g.randint(i + 1)
            perm[i], perm[j] = perm[j], perm[i]
        for i in range(n // 2):
            ops.append((G.CNOTGate(), perm[2 * i + 1], perm[2 * i], 0))
            maybe_3q()
    return ops


def qft_circuit(start: int, end: int, inverse: bool = False, do_swap: bool = True) -> list:
    """QuantumFourierTransform::QFT / IQFT as a gate list (QuantumFourierTransform.h:35-87,
    QubitsSwapper.h:23-34)"""
    ops: list = []
    swaps = []
    a, b = start, end
    while a < b:
        swaps.append((G.SwapGate(), a, b, 0))
        a, b = a + 1, b - 1
    if not inverse:
        ops.append((G.HadamardGate(), end, 0, 0))
        for cur in range(end, start, -1):
            phase = math.pi / 2
            for c in range(cur - 1, start - 1, -1):
                ops.append((G.ControlledPhaseShiftGate(phase), cur, c, 0))
                phase *= 0.5
            ops.append((G.HadamardGate(), cur - 1, 0, 0))
        if do_swap:
            ops.extend(swaps)
    else:
        if do_swap:
            ops.extend(swaps)
        for cur in range(start + 1, end + 1):
            ops.append((G.HadamardGate(), cur - 1, 0, 0))
            phase = -math.pi / 2
            for c in range(cur - 1, start - 1, -1):
                ops.append((G.ControlledPhaseShiftGate(phase), cur, c, 0))
                phase *= 0.5
        ops.append((G.HadamardGate(), end, 0, 0))
    return ops


def random_normal_state(n: int, seed: int) -> np.ndarray:
    """a_x = (g1 + i g2) / norm with g iid N(0, 1) (numpy PCG64 stream of the seed)"""
    rng = np.random.default_rng(seed)
    v = rng.standard_normal(2 << n).view(np.complex128)
    return v / np.linalg.norm(v)


def random_3regular(n: int, g: Mt19937_64) -> list[tuple[int, int]]:
    """random 3-regular simple graph by the configuration model with rejection; edges (i, j), i < j"""
    if n % 2 or n < 4:
        raise ValueError("a 3-regular graph needs an even n >= 4")
    while True:
        stubs = [v for v in range(n) for _ in range(3)]
        for i in range(len(stubs) - 1, 0, -1):
            j = g.randint(i + 1)
            stubs[i], stubs[j] = stubs[j], stubs[i]
        edges = set()
        ok = True
        for k in range(0, len(stubs), 2):
            a, b = stubs[k], stubs[k + 1]
            if a == b:
                ok = False
                break
            e = (min(a, b), max(a, b))
            if e in edges:
                ok = False
                break
            edges.add(e)
        if ok:
            return sorted(edges)


def gaussian(g: Mt19937_64) -> float:
    """N(0, 1) by Box-Muller from two uniform draws"""
    u1 = 1.0 - g.uniform()
    u2 = g.uniform()
    return math.sqrt(-2.0 * math.log(u1)) * math.cos(TWO_PI * u2)


def qaoa_instances(count: int, seed: int, nmin: int = 12, nmax: int = 24, p: int = 4, h_sigma: float = 0.5) -> list:
    """random 3-regular Ising instances: n even in [nmin, nmax], J_ij = +-1, h_i ~ N(0, h_sigma^2),
    gamma_l, beta_l uniform in [0, pi)"""
    g = Mt19937_64(seed)
    evens = list(range(nmin + (nmin % 2), nmax + 1, 2))
    out = []
    for _ in range(count):
        n = evens[g.randint(len(evens))]
        edges = random_3regular(n, g)
        J = [1.0 if g.uniform() < 0.5 else -1.0 for _ in edges]
        h = [h_sigma * gaussian(g) for _ in range(n)]
        gammas = [g.uniform() * math.pi for _ in range(p)]
        betas = [g.uniform() * math.pi for _ in range(p)]
        out.append({"n": n, "edges": edges, "J": J, "h": h, "gammas": gammas, "betas": betas})
    return out


def qaoa_circuit(inst: dict) -> list:
    """QAOAIsingSubalgorithm::Exec (IsingModel.h:557-567) after the reset: H on all qubits, then per
    layer CNOT(i<-j) RZ(2 gamma J_ij)(i) CNOT(i<-j) for each edge, RZ(gamma h_i) for h_i != 0, and
    RX(2 beta) on all qubits (IsingModel.h:491-554)"""
    n = inst["n"]
    ops: list = [(G.HadamardGate(), q, 0, 0) for q in range(n)]
    for gamma, beta in zip(inst["gammas"], inst["betas"]):
        for (i, j), J in zip(inst["edges"], inst["J"]):
            ops.append((G.CNOTGate(), i, j, 0))
            ops.append((G.RzGate(2 * gamma * J), i, 0, 0))
            ops.append((G.CNOTGate(), i, j, 0))
        for q in range(n):
            if inst["h"][q] != 0.0:
                ops.append((G.RzGate(gamma * inst["h"][q]), q, 0, 0))
        for q in range(n):
            ops.append((G.RxGate(2 * beta), q, 0, 0))
    return ops


def ising_energies(inst: dict) -> np.ndarray:
    """E(x) = -(sum h_i s_i + sum J_ij s_i s_j), s = +1 for bit 0 and -1 for bit 1 (IsingModel.h:106-119,
    203-206), for every basis state x"""
    n = inst["n"]
    x = np.arange(1 << n, dtype=np.uint64)
    spins = [1.0 - 2.0 * ((x >> np.uint64(q)) & np.uint64(1)).astype(np.float64) for q in range(n)]
    e = np.zeros(1 << n)
    for q in range(n):
        e += inst["h"][q] * spins[q]
    for (i, j), J in zip(inst["edges"], inst["J"]):
        e += J * spins[i] * spins[j]
    return -e
