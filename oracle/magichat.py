"""MagicHat restated (test infrastructure only).

pngf-opt/magichat.hpp:32-111 draws hat entries without replacement with a
std::mt19937 seeded by rng_seed and std::uniform_int_distribution<> over
[0, num_left-1] followed by a swap-remove. Its results depend on the C++
standard library; the reference's are those of GCC's libstdc++, which maps a
32-bit engine output to [0, range) with Lemire's multiply-and-reject method
(D. Lemire, "Fast Random Integer Generation in an Interval", ACM TOMACS 29(1),
2019). Both the engine (the standard MT19937 recurrence and seeding) and that
published method are restated here from their definitions.
"""
from __future__ import annotations


class MT19937:
    """std::mt19937 (32-bit Mersenne Twister, standard parameters)."""

    N, M = 624, 397

    def __init__(self, seed: int):
        self.seed(seed)

    def seed(self, seed: int):
        mt = [0] * self.N
        mt[0] = seed & 0xFFFFFFFF
        for i in range(1, self.N):
            mt[i] = (1812433253 * (mt[i - 1] ^ (mt[i - 1] >> 30)) + i) & 0xFFFFFFFF
        self.mt = mt
        self.idx = self.N

    def _twist(self):
        mt = self.mt
        for i in range(self.N):
            y = (mt[i] & 0x80000000) | (mt[(i + 1) % self.N] & 0x7FFFFFFF)
            v = mt[(i + self.M) % self.N] ^ (y >> 1)
            if y & 1:
                v ^= 0x9908B0DF
            mt[i] = v
        self.idx = 0

    def __call__(self) -> int:
        if self.idx >= self.N:
            self._twist()
        y = self.mt[self.idx]
        self.idx += 1
        y ^= y >> 11
        y ^= (y << 7) & 0x9D2C5680
        y ^= (y << 15) & 0xEFC60000
        y ^= y >> 18
        return y & 0xFFFFFFFF

    def copy(self):
        c = MT19937.__new__(MT19937)
        c.mt = list(self.mt)
        c.idx = self.idx
        return c


def uniform_below(gen: MT19937, s: int) -> int:
    """Integer in [0, s) from 32-bit draws, Lemire's method."""
    m = gen() * s
    low = m & 0xFFFFFFFF
    if low < s:
        t = ((1 << 32) - s) % s
        while low < t:
            m = gen() * s
            low = m & 0xFFFFFFFF
    return m >> 32


class MagicHat:
    def __init__(self, seed: int, run_index: int, num_entries: int):
        if seed == 0:
            raise ValueError("seed 0 asks for a random seed; the oracle needs a fixed one")
        self.rng_seed = seed
        self.gen = MT19937(seed & 0xFFFFFFFF)
        self.total = num_entries
        self.num_left = num_entries
        self.entry = list(range(num_entries))

    def rand_binary(self) -> int:
        return self.gen() & 1

    def draw(self) -> int:
        if self.num_left <= 0:
            return -1
        idx = uniform_below(self.gen, self.num_left)
        val = self.entry[idx]
        self.entry[idx] = self.entry[self.num_left - 1]
        self.num_left -= 1
        return val

    def reset(self):
        self.entry = list(range(self.total))
        self.num_left = self.total
        return self.num_left
