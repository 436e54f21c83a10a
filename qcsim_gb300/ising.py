"""QCSim's Ising model and its QAOA sub-algorithm over one engine register: Models::IsingModel
(IsingModel.h:29-217) and Models::QAOAIsingSubalgorithm (IsingModel.h:219-665).

Execute is the reference's optimiser.  Each step estimates the gradient in every gamma_l and beta_l by
central differences of the sampled energy (100000 shots by default), takes an AdamW step, re-runs the
circuit and stops when two successive energies differ by at most deltaE.  The circuit of Exec (H on every
qubit, then per layer CNOT-RZ-CNOT on every interaction, RZ(gamma h_i) on every site with h_i != 0, RX(2 beta)
on every qubit, and optionally the CNOT ring plus RY(2 beta)) goes to the engine as one gate list per run.
Sampled energies come from the register's RepeatedMeasure, so a seeded register reproduces a run.  For many
instances at fixed angles, qcsim_gb300.qaoa.QaoaBatch runs the same circuit batched with exact <H>.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from . import gates as G


@dataclass
class Interaction:
    """IsingModel::Interaction (IsingModel.h:32-36)"""
    i: int = 0
    j: int = 0
    J: float = 1.0


def _interaction(x) -> Interaction:
    return x if isinstance(x, Interaction) else Interaction(int(x[0]), int(x[1]), float(x[2]))


class IsingModel:
    """Models::IsingModel (IsingModel.h:29-217): spins s_i (False = +1, True = -1), fields h_i and couplings
    J_ij on i < j; E = -(sum_i h_i s_i + sum_{i<j} J_ij s_i s_j).  Bit i of a basis state is spin i."""

    def __init__(self):
        self.Clear()

    def Clear(self) -> None:
        self.spins: list[bool] = []
        self.h: list[float] = []
        self.neighbours: dict[int, set[int]] = {}
        self.interactions: dict[tuple[int, int], float] = {}

    def AddInteraction(self, i: int, j: int, J: float) -> None:
        if i == j:
            return
        if i > j:
            i, j = j, i
        if j >= len(self.spins):
            return
        self.neighbours.setdefault(i, set()).add(j)
        self.interactions[(i, j)] = float(J)

    def Set(self, *args) -> None:
        """Set(spins, interactions=[], hvals=[]) or Set(interactions=[], hvals=[]) (IsingModel.h:56-76);
        interactions are Interaction objects or (i, j, J) tuples"""
        if args and len(args[0]) and isinstance(args[0][0], (bool, np.bool_)):
            spins, ints, hvals = list(args[0]), (args[1] if len(args) > 1 else []), (args[2] if len(args) > 2 else [])
            self.Clear()
            self.spins = [bool(s) for s in spins]
            self.h = [float(v) for v in hvals][: len(self.spins)]
            self.h += [0.0] * (len(self.spins) - len(self.h))
        else:
            ints, hvals = (args[0] if args else []), (args[1] if len(args) > 1 else [])
            self.Clear()
            self.h = [float(v) for v in hvals]
            self.spins = [False] * len(self.h)
        for x in ints:
            x = _interaction(x)
            self.AddInteraction(x.i, x.j, x.J)

    def SetH(self, i: int, hval: float) -> None:
        if i < len(self.spins):
            self.h[i] = float(hval)

    def GetH(self, i: int | None = None):
        if i is None:
            return self.h
        return self.h[i] if i < len(self.h) else 0.0

    def SetSpin(self, i: int, s: bool) -> None:
        if i < len(self.spins):
            self.spins[i] = bool(s)

    def GetSpin(self, i: int) -> bool:
        return self.spins[i] if i < len(self.spins) else False

    def GetSpins(self) -> list[bool]:
        return self.spins

    def GetNeighbours(self) -> dict[int, set[int]]:
        return self.neighbours

    def GetInteractions(self) -> dict[tuple[int, int], float]:
        return self.interactions

    def SetState(self, state: int) -> None:
        for pos in range(len(self.spins)):
            self.spins[pos] = bool(state & 1)
            state >>= 1

    def Energy(self, state: int | None = None) -> float:
        """IsingModel.h:106-127 (sets the spins to state first when given)"""
        if state is not None:
            self.SetState(state)
        e = 0.0
        for i, s in enumerate(self.spins):
            si = -1 if s else 1
            e += self.GetH(i) * si
            for j in sorted(self.neighbours.get(i, ())):
                e += self.interactions[(i, j)] * si * (-1 if self.spins[j] else 1)
        return -e

    def Energies(self) -> np.ndarray:
        """E(x) for every basis state x, with the per-state sums in the order of Energy"""
        n = len(self.spins)
        x = np.arange(1 << n, dtype=np.int64)
        s = [1 - 2 * ((x >> i) & 1) for i in range(n)]
        e = np.zeros(1 << n)
        for i in range(n):
            e += self.GetH(i) * s[i]
            for j in sorted(self.neighbours.get(i, ())):
                e += self.interactions[(i, j)] * s[i] * s[j]
        return -e

    def GetMinEnergyState(self) -> int:
        """the first state of lowest energy (IsingModel.h:136-154)"""
        return int(np.argmin(self.Energies()))

    def GetMinEnergyStates(self) -> set[int]:
        """every state within 1e-9 of the lowest energy, scanned as IsingModel.h:156-179 does"""
        res: set[int] = set()
        minE = float(np.finfo(np.float64).max)
        for state, e in enumerate(self.Energies().tolist()):
            if minE > e and abs(minE - e) > 1e-9:
                minE = e
                res = {state}
            elif abs(minE - e) <= 1e-9:
                res.add(state)
        return res


class QAOAIsingSubalgorithm:
    """Models::QAOAIsingSubalgorithm (IsingModel.h:219-665) with the reference's defaults: p = 1, gamma and beta
    starting at 1, deltaE 5e-4, finite-difference step 1e-3, AdamW step 5e-4 (beta1 0.8, beta2 0.95, lambda
    1e-3), 100000 shots per energy.  Interactions are applied in ascending (i, j) order (the reference walks
    an unordered map; the ZZ terms commute)."""

    def __init__(self):
        self.model = IsingModel()
        self.h = G.HadamardGate()
        self.cnot = G.CNOTGate()
        self.deltaE = 0.0005
        self.gammaStart = [1.0]
        self.betaStart = [1.0]
        self.sGamma: list[float] = []
        self.mGamma: list[float] = []
        self.sBeta: list[float] = []
        self.mBeta: list[float] = []
        self.beta1 = 0.8
        self.beta2 = 0.95
        self.lambda_ = 0.001
        self.stepNr = 0
        self.epsilon = 0.001
        self.stepSize = 0.0005
        self.nrMeasurements = 100000
        self.betterMixing = False
        self.history: list[float] = []  # the energy after every optimiser step (the reference prints it)

    # ---- the model (IsingModel.h:275-364) ----
    def Clear(self) -> None:
        self.model.Clear()

    def AddInteraction(self, i: int, j: int, J: float) -> None:
        self.model.AddInteraction(i, j, J)

    def Set(self, *args) -> None:
        self.model.Set(*args)

    def SetH(self, i: int, hval: float) -> None:
        self.model.SetH(i, hval)

    def GetH(self, i: int | None = None):
        return self.model.GetH(i)

    def SetSpin(self, i: int, s: bool) -> None:
        self.model.SetSpin(i, s)

    def GetSpin(self, i: int) -> bool:
        return self.model.GetSpin(i)

    def Energy(self, state: int | None = None) -> float:
        return self.model.Energy(state)

    def SetState(self, state: int) -> None:
        self.model.SetState(state)

    def GetMinEnergyState(self) -> int:
        return self.model.GetMinEnergyState()

    def GetMinEnergyStates(self) -> set[int]:
        return self.model.GetMinEnergyStates()

    def GetSpins(self) -> list[bool]:
        return self.model.GetSpins()

    def GetNeighbours(self):
        return self.model.GetNeighbours()

    def GetInteractions(self):
        return self.model.GetInteractions()

    # ---- optimiser settings (IsingModel.h:366-483) ----
    def GetDeltaE(self) -> float:
        return self.deltaE

    def SetDeltaE(self, dE: float) -> None:
        self.deltaE = dE

    def GetGammaStart(self) -> list[float]:
        return self.gammaStart

    def SetGammaStart(self, gamma: float, index: int = 0) -> None:
        if index < len(self.gammaStart):
            self.gammaStart[index] = float(gamma)

    def GetBetaStart(self) -> list[float]:
        return self.betaStart

    def SetBetaStart(self, beta: float, index: int = 0) -> None:
        if index < len(self.betaStart):
            self.betaStart[index] = float(beta)

    def GetP(self) -> int:
        return len(self.gammaStart)

    def SetP(self, p: int) -> None:
        if p < 1:
            return
        self.gammaStart = (self.gammaStart + [1.0] * p)[:p]
        self.betaStart = (self.betaStart + [1.0] * p)[:p]

    def GetEpsilon(self) -> float:
        return self.epsilon

    def SetEpsilon(self, eps: float) -> None:
        self.epsilon = eps

    def GetStepSize(self) -> float:
        return self.stepSize

    def SetStepSize(self, step: float) -> None:
        self.stepSize = step

    def SetBeta1(self, b1: float) -> None:
        self.beta1 = b1

    def GetBeta1(self) -> float:
        return self.beta1

    def SetBeta2(self, b2: float) -> None:
        self.beta2 = b2

    def GetBeta2(self) -> float:
        return self.beta2

    def SetLambda(self, lam: float) -> None:
        self.lambda_ = lam

    def GetLambda(self) -> float:
        return self.lambda_

    def GetNrMeasurements(self) -> int:
        return self.nrMeasurements

    def SetNrMeasurements(self, nr) -> None:
        self.nrMeasurements = int(nr)

    def SetMixing(self, better: bool) -> None:
        self.betterMixing = bool(better)

    def GetMixing(self) -> bool:
        return self.betterMixing

    # ---- the circuit (IsingModel.h:485-567) ----
    def circuit(self, nrQubits: int, gamma, beta) -> list[tuple]:
        """the gates of Exec after the reset to |0>, as (gate, q0, q1, q2) tuples"""
        ops: list[tuple] = [(self.h, q) for q in range(nrQubits)]
        for g, b in zip(gamma, beta):
            for q1 in sorted(self.model.neighbours):
                for q2 in sorted(self.model.neighbours[q1]):
                    J = self.model.interactions.get((q1, q2))
                    rz = G.RzGate(2 * g * J if J is not None else 2 * g)
                    ops += [(self.cnot, q1, q2), (rz, q1), (self.cnot, q1, q2)]
            for q in range(nrQubits):
                hval = self.model.GetH(q)
                if hval != 0.0:
                    ops.append((G.RzGate(g * hval), q))
            rx = G.RxGate(2 * b)
            ops += [(rx, q) for q in range(nrQubits)]
            if self.betterMixing:
                last = nrQubits - 1
                ops += [(self.cnot, q + 1, q) for q in range(last)]
                ops.append((self.cnot, 0, last))
                ry = G.RyGate(2 * b)
                ops += [(ry, q) for q in range(nrQubits)]
        return ops

    def Exec(self, reg, gamma, beta) -> None:
        reg.setToBasisState(0)
        reg.ApplyGates(self.circuit(reg.getNrQubits(), gamma, beta))

    def EnergyExpectationValue(self, reg, nrShots: int = 100000) -> float:
        """sum over the measured states (ascending, as the reference's std::map) of E(x) count / nrShots
        (IsingModel.h:569-578)"""
        res = reg.RepeatedMeasure(nrShots)
        energy = 0.0
        for state in sorted(res):
            energy += self.Energy(state) * float(res[state]) / nrShots
        return energy

    def GradientDescentStep(self, reg, gamma: list[float], beta: list[float], eps: float = 0.0002,
                            alpha: float = 0.0001, nrShots: int = 100000):
        """central differences of the sampled energy in every gamma_l and beta_l and one AdamW step, with the
        reference's in-place bias correction of the moments (IsingModel.h:580-636)"""
        twoEps = 2.0 * eps
        newGamma, newBeta = [0.0] * len(gamma), [0.0] * len(beta)
        self.stepNr += 1
        div1 = 1.0 / (1.0 - math.pow(self.beta1, self.stepNr))
        div2 = 1.0 / (1.0 - math.pow(self.beta2, self.stepNr))
        for i in range(len(gamma)):
            gv, bv = gamma[i], beta[i]
            gamma[i] = gv - eps
            self.Exec(reg, gamma, beta)
            E1 = self.EnergyExpectationValue(reg, nrShots)
            gamma[i] = gv + eps
            self.Exec(reg, gamma, beta)
            E2 = self.EnergyExpectationValue(reg, nrShots)
            gamma[i] = gv
            beta[i] = bv - eps
            self.Exec(reg, gamma, beta)
            E3 = self.EnergyExpectationValue(reg, nrShots)
            beta[i] = bv + eps
            self.Exec(reg, gamma, beta)
            E4 = self.EnergyExpectationValue(reg, nrShots)
            beta[i] = bv

            grad = (E2 - E1) / twoEps
            self.mGamma[i] = (self.beta1 * self.mGamma[i] - (1.0 - self.beta1) * grad) * div1
            self.sGamma[i] = (self.beta2 * self.sGamma[i] + (1.0 - self.beta2) * grad * grad) * div2
            newGamma[i] = gv + alpha * (self.mGamma[i] / math.sqrt(self.sGamma[i] + 1e-8) - self.lambda_ * gv)

            grad = (E4 - E3) / twoEps
            self.mBeta[i] = (self.beta1 * self.mBeta[i] - (1.0 - self.beta1) * grad) * div1
            self.sBeta[i] = (self.beta2 * self.sBeta[i] + (1.0 - self.beta2) * grad * grad) * div2
            newBeta[i] = bv + alpha * (self.mBeta[i] / math.sqrt(self.sBeta[i] + 1e-8) - self.lambda_ * bv)
        return newGamma, newBeta

    def Execute(self, reg) -> int:
        """optimise the angles, then return the measured state of lowest E(x) count / shots at the best angles
        (IsingModel.h:220-273)"""
        Eold = float(np.finfo(np.float64).max)
        Emin = Eold
        E = 0.0
        gamma, beta = list(self.gammaStart), list(self.betaStart)
        opt = (list(gamma), list(beta))
        p = len(self.gammaStart)
        self.sGamma, self.mGamma = [0.0] * p, [0.0] * p
        self.sBeta, self.mBeta = [0.0] * p, [0.0] * p
        self.stepNr = 0
        self.history = []
        i = 0
        while abs(E - Eold) > self.deltaE and i < 100000:
            Eold = E
            gamma, beta = self.GradientDescentStep(reg, gamma, beta, self.epsilon, self.stepSize, self.nrMeasurements)
            self.Exec(reg, gamma, beta)
            E = self.EnergyExpectationValue(reg, self.nrMeasurements)
            self.history.append(E)
            if E < Emin:
                Emin = E
                opt = (list(gamma), list(beta))
            i += 1
        self.Exec(reg, *opt)
        res = reg.RepeatedMeasure(self.nrMeasurements)
        Emin = float(np.finfo(np.float64).max)
        state = 0
        for s in sorted(res):
            e = self.Energy(s) * float(res[s]) / self.nrMeasurements
            if e < Emin:
                Emin, state = e, s
        self.sGamma, self.mGamma, self.sBeta, self.mBeta = [], [], [], []
        return state
