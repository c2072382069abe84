"""Seeded walker sets of the benchmark workloads.

The uneven batch draws each walker's |U| and beta from a 64-bit Mersenne
Twister, MT19937-64 (Matsumoto and Nishimura; Nishimura, ACM TOMACS 10 (2000)
348), the engine std::mt19937_64 of the C++ standard library.  It is restated
here from its published recurrence so that the walker set is the same on every
machine and in every language that seeds std::mt19937_64 with the same value.
"""
from __future__ import annotations

from typing import List

_MASK64 = (1 << 64) - 1


class MT19937_64:
    """The MT19937-64 engine (w = 64, n = 312, m = 156, r = 31), seeded like
    std::mt19937_64(seed).  The C++ standard's check: the 10000th output of the
    default-seeded engine (seed 5489) is 9981545732273789042."""

    N, M = 312, 156
    A = 0xB5026F5AA96619E9
    UPPER, LOWER = 0xFFFFFFFF80000000, 0x7FFFFFFF

    def __init__(self, seed: int = 5489):
        mt = [seed & _MASK64]
        for i in range(1, self.N):
            prev = mt[-1]
            mt.append((6364136223846793005 * (prev ^ (prev >> 62)) + i) & _MASK64)
        self.mt = mt
        self.idx = self.N

    def _twist(self):
        mt = self.mt
        for i in range(self.N):
            x = (mt[i] & self.UPPER) | (mt[(i + 1) % self.N] & self.LOWER)
            xa = x >> 1
            if x & 1:
                xa ^= self.A
            mt[i] = mt[(i + self.M) % self.N] ^ xa
        self.idx = 0

    def __call__(self) -> int:
        if self.idx >= self.N:
            self._twist()
        y = self.mt[self.idx]
        self.idx += 1
        y ^= (y >> 29) & 0x5555555555555555
        y ^= (y << 17) & 0x71D67FFFEDA60000
        y ^= (y << 37) & 0xFFF7EEE000000000
        y ^= y >> 43
        return y & _MASK64

    def canonical(self) -> float:
        """A double in [0, 1) formed as std::generate_canonical<double, 53> forms it
        from one 64-bit output: the output rounded to double, over 2^64."""
        u = float(self()) / 18446744073709551616.0
        return u if u < 1.0 else 0.99999999999999989  # nextafter(1, 0)


UNEVEN_SIDES = (6, 8, 10, 12)
UNEVEN_BETAS = (4.0, 6.0, 8.0)


def uneven_batch(dq, per_size: int = 64, seed: int = 7, dtau: float = 0.05, pace: int = 10,
                 sides=UNEVEN_SIDES, seed0: int = 7000) -> List:
    """Walkers of the uneven batch: per_size repulsive walkers for each lattice side in
    `sides` (N = 36 ... 144), t = 1, mu = 0, dtau = 0.05, stabilization every 10 slices,
    dense exp(-dtau K).  For walker w (side-major order) two consecutive canonical draws
    u, u' of std::mt19937_64(seed) give |U|_w = 2 + 4u and beta_w = (4, 6, 8)[floor(3u')],
    so Lt_w = beta_w / dtau = 80, 120 or 160.  Walker w's Metropolis seed is seed0 + w."""
    eng = MT19937_64(seed)
    out = []
    for L in sides:
        for _ in range(per_size):
            u = 2.0 + 4.0 * eng.canonical()
            beta = UNEVEN_BETAS[min(2, int(3.0 * eng.canonical()))]
            out.append(dq.WalkerDesc(model=0, L=L, U=u, mu=0.0, beta=beta, Lt=int(round(beta / dtau)), pace=pace,
                                     seed=seed0 + len(out)))
    return out
