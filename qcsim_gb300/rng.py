"""std::mt19937_64 and std::uniform_real_distribution<double>(0, 1) in pure Python.

Used to generate seeded circuits on the host without the engine (the draws match the C++ standard
library's, so a C++ caller with the same seed builds the same circuit).
"""
from __future__ import annotations

import math

_MASK = (1 << 64) - 1


class Mt19937_64:
    def __init__(self, seed: int):
        self.mt = [0] * 312
        self.mt[0] = seed & _MASK
        for i in range(1, 312):
            prev = self.mt[i - 1]
            self.mt[i] = (6364136223846793005 * (prev ^ (prev >> 62)) + i) & _MASK
        self.idx = 312

    def _twist(self) -> None:
        mt = self.mt
        for i in range(312):
            y = (mt[i] & 0xFFFFFFFF80000000) | (mt[(i + 1) % 312] & 0x7FFFFFFF)
            v = mt[(i + 156) % 312] ^ (y >> 1)
            if y & 1:
                v ^= 0xB5026F5AA96619E9
            mt[i] = v
        self.idx = 0

    def next(self) -> int:
        if self.idx >= 312:
            self._twist()
        z = self.mt[self.idx]
        self.idx += 1
        z ^= (z >> 29) & 0x5555555555555555
        z ^= (z << 17) & 0x71D67FFFEDA60000
        z ^= (z << 37) & 0xFFF7EEE000000000
        z ^= z >> 43
        return z & _MASK

    def uniform(self) -> float:
        """generate_canonical<double, 53>: one 64-bit draw / 2^64, kept below 1"""
        r = float(self.next()) / 18446744073709551616.0
        return r if r < 1.0 else math.nextafter(1.0, 0.0)

    def randint(self, n: int) -> int:
        """an integer in [0, n) from one uniform draw"""
        return min(int(self.uniform() * n), n - 1)
