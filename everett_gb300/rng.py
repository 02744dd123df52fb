"""xoshiro256++ seeded through SplitMix64: a restatement of everett's Rng
(src/rng.rs:10-58), used by the circuit generators and the host side of the
engine so that seeds mean the same thing as in the reference."""
from __future__ import annotations

_M = (1 << 64) - 1


def _rotl(x: int, r: int) -> int:
    return ((x << r) | (x >> (64 - r))) & _M


class Rng:
    __slots__ = ("s",)

    def __init__(self, s: list[int]):
        self.s = s

    @classmethod
    def seed_from_u64(cls, seed: int) -> "Rng":
        seed &= _M
        words = []
        for _ in range(4):
            seed = (seed + 0x9E3779B97F4A7C15) & _M
            z = seed
            z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _M
            z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _M
            words.append(z ^ (z >> 31))
        return cls(words)

    def next_u64(self) -> int:
        s = self.s
        result = (_rotl((s[0] + s[3]) & _M, 23) + s[0]) & _M
        t = (s[1] << 17) & _M
        s[2] ^= s[0]
        s[3] ^= s[1]
        s[1] ^= s[2]
        s[0] ^= s[3]
        s[2] ^= t
        s[3] = _rotl(s[3], 45)
        return result

    def next_f64(self) -> float:
        return (self.next_u64() >> 11) * (1.0 / (1 << 53))
