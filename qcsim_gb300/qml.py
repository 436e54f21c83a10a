"""QCSim's q-means clustering over the engine: MachineLearning::QMeansClustering2D (QMeansClustering2D.h:11-276).

Each 2D point is encoded on a qubit by a U(theta, phi) gate (theta = pi/2 (x + y), phi = pi/2 (x + 1 - y) on the
normalised coordinates), and the overlap of a point with a centroid is estimated by a swap test on three qubits
(H, Fredkin controlled by qubit 0, H; the probability of measuring qubit 0 as 0 grows with the overlap).  Every
point joins the centroid of largest measured overlap, the centroids move to their clusters' means, and the
steps repeat until no point changes cluster.  The swap test is one gate list per estimate and its statistics
come from the register's RepeatedMeasure; the starting centroids are drawn with a seeded numpy generator (a
clock-seeded std::mt19937_64 in the reference).
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from . import gates as G
from .algorithms import QuantumAlgorithm


@dataclass
class DataPoint:
    x: float = 0.0
    y: float = 0.0


@dataclass
class ClusterDataPoint(DataPoint):
    cluster: int = 0


class QMeansClustering2D(QuantumAlgorithm):
    """MachineLearning::QMeansClustering2D (QMeansClustering2D.h:11-276)"""

    def __init__(self, addseed: int = 0, choice_seed: int | None = None, **kw):
        super().__init__(3, addseed, **kw)
        self._rng = np.random.default_rng(choice_seed)
        self.m_data: list[ClusterDataPoint] = []
        self.centroids: list[ClusterDataPoint] = []
        self.xmin = self.xmax = self.ymin = self.ymax = 0.0
        self.xspan = self.yspan = 1.0
        self.ugate1, self.ugate2 = G.UGate(), G.UGate()
        self.hadamard, self.cswap = G.HadamardGate(), G.FredkinGate()

    def Execute(self) -> int:
        self.ExecuteWithoutMeasurement()
        return self.Measure(0)

    def ExecuteWithMultipleMeasurements(self, nrMeasurements: int = 1000) -> dict:
        self.ExecuteWithoutMeasurement()
        return self.RepeatedMeasure(0, 0, nrMeasurements)

    def setData(self, data) -> None:
        """copy the points and the bounding box; both spans become the larger one (QMeansClustering2D.h:52-79)"""
        self.m_data = [ClusterDataPoint(float(p.x), float(p.y), 0) for p in data]
        xs = [p.x for p in self.m_data]
        ys = [p.y for p in self.m_data]
        self.xmin, self.xmax = min(xs, default=float("inf")), max(xs, default=float("-inf"))
        self.ymin, self.ymax = min(ys, default=float("inf")), max(ys, default=float("-inf"))
        self.xspan = self.yspan = max(self.xmax - self.xmin, self.ymax - self.ymin)

    def getData(self) -> list[ClusterDataPoint]:
        return self.m_data

    def getCentroids(self) -> list[ClusterDataPoint]:
        return self.centroids

    def Cluster(self, k: int, nrMeasurements: int = 1000, maxSteps: int = 100000) -> bool:
        self.getStartCentroids(k)
        return self.Update(nrMeasurements, maxSteps)

    def SetDataPoint1(self, p) -> None:
        self._set_bloch(self.ugate1, p)

    def SetDataPoint2(self, p) -> None:
        self._set_bloch(self.ugate2, p)

    def _set_bloch(self, ugate, p) -> None:
        x = (p.x - self.xmin) / self.xspan
        y = (p.y - self.ymin) / self.yspan
        ugate.SetParams(0.5 * math.pi * (x + y), 0.5 * math.pi * (x + 1.0 - y))

    def ExecuteWithoutMeasurement(self) -> None:
        self.setToBasisState(0)
        self.ApplyGates([(self.ugate1, 1), (self.ugate2, 2), (self.hadamard, 0), (self.cswap, 2, 1, 0),
                         (self.hadamard, 0)])

    def getStartCentroids(self, k: int) -> list[ClusterDataPoint]:
        """k distinct data points (no two closer than 0.1 of the span) as the first centroids; the chosen points
        are swapped to the front while drawing and the swaps are undone afterwards (QMeansClustering2D.h:108-150).
        The reference computes the distance limit once per process (a function-local static); here it is
        computed from the current data on every call."""
        eps = 0.01 * self.xspan * self.xspan
        self.centroids = [ClusterDataPoint() for _ in range(k)]
        stack: list[int] = []
        for c in range(k):
            while True:
                index = int(self._rng.integers(c, len(self.m_data)))
                cand = self.m_data[index]
                self.centroids[c] = ClusterDataPoint(cand.x, cand.y, c)
                if all((cand.x - o.x) ** 2 + (cand.y - o.y) ** 2 >= eps for o in self.centroids[:c]):
                    break
            stack.append(index)
            self.m_data[c], self.m_data[index] = self.m_data[index], self.m_data[c]
        while stack:
            top = stack[-1]
            self.m_data[top], self.m_data[len(stack) - 1] = self.m_data[len(stack) - 1], self.m_data[top]
            stack.pop()
        return self.centroids

    def UpdateCentroids(self) -> None:
        sizes = [0] * len(self.centroids)
        for c in self.centroids:
            c.x = c.y = 0.0
        for p in self.m_data:
            self.centroids[p.cluster].x += p.x
            self.centroids[p.cluster].y += p.y
            sizes[p.cluster] += 1
        for c, n in zip(self.centroids, sizes):
            if n:
                c.x /= n
                c.y /= n

    def UpdateClusters(self, nrMeasurements: int) -> bool:
        """every point to the centroid with the most 0 outcomes of the swap test; True when none moved
        (QMeansClustering2D.h:172-205)"""
        terminate = True
        for p in self.m_data:
            overlap, cluster = 0, 0
            self.SetDataPoint1(p)
            for c, centroid in enumerate(self.centroids):
                self.SetDataPoint2(centroid)
                res = self.ExecuteWithMultipleMeasurements(nrMeasurements)
                if res.get(0, 0) > overlap:
                    overlap, cluster = res.get(0, 0), c
            if p.cluster != cluster:
                terminate = False
                p.cluster = cluster
        return terminate

    def Update(self, nrMeasurements: int, maxSteps: int) -> bool:
        terminate = False
        i = 0
        while i < maxSteps and not terminate:
            terminate = self.UpdateStep(nrMeasurements)
            i += 1
        return terminate

    def UpdateStep(self, nrMeasurements: int) -> bool:
        terminate = self.UpdateClusters(nrMeasurements)
        if not terminate:
            self.UpdateCentroids()
        return terminate
