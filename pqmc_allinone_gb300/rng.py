"""ran2_s of the reference (src/mod_ranstate.f90:171-191), host side.

The reference draws every Monte Carlo random number from this NR-F90
combined generator (subtract-with-borrow + xorshift + multiply-with-carry)
and returns REAL(SP).  The device carries the same five state words per
chain; this host copy seeds them and replays draws made during set-up
(``init_boson_field``).
"""
from __future__ import annotations

import numpy as np

_AMM = np.float32(np.float32(1.0) - np.float32(2.0 ** -24)) / np.float32(-2147483648.0)
_M32 = 0xFFFFFFFF


def _s32(v: int) -> int:
    v &= _M32
    return v - (1 << 32) if v & 0x80000000 else v


def seed_words(seed: int) -> list[int]:
    """init_rng_by_seed(iseed) (src/mod_ranstate.f90:267-283): ran_seed(put=)
    sets all five words to iseed, then forces words 1-3 non-negative and
    words 4-5 non-zero (:119-122)."""
    w = [int(seed)] * 5
    for k in range(3):
        if w[k] < 0:
            w[k] = ~w[k]
    for k in (3, 4):
        if w[k] == 0:
            w[k] = 1
    return w


class Ran2:
    def __init__(self, words):
        self.iran, self.jran, self.kran, self.mran, self.nran = (int(x) for x in words)

    @classmethod
    def from_seed(cls, seed: int) -> "Ran2":
        return cls(seed_words(seed))

    @property
    def words(self) -> list[int]:
        return [self.iran, self.jran, self.kran, self.mran, self.nran]

    def next(self) -> np.float32:
        rans = _s32(self.iran - self.kran)
        if rans < 0:
            rans = _s32(rans + 2147483579)
        self.iran, self.jran, self.kran = self.jran, self.kran, rans
        n = self.nran & _M32
        n ^= (n << 13) & _M32
        n ^= n >> 17
        n ^= (n << 5) & _M32
        self.nran = _s32(n)
        m = self.mran & _M32
        lo = m & 65535
        m = ((((3533 * (m >> 16) + lo) << 16) & _M32) + 3533 * lo + 820265819) & _M32
        self.mran = _s32(m)
        r = _s32(((self.nran & _M32) ^ (self.kran & _M32)) + (self.mran & _M32))
        v = r if r < 0 else ~r
        return np.float32(_AMM * np.float32(v))

    def rands(self) -> np.float32:
        return self.next()

    def ran_sysm(self) -> np.float32:
        r = self.next()
        return np.float32(np.float32(r * np.float32(2.0)) - np.float32(1.0))
