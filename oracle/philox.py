"""Philox-4x32-10 in Python — TEST INFRASTRUCTURE ONLY.

The counter-based generator of Salmon, Moraes, Dror and Shaw, "Parallel
random numbers: as easy as 1, 2, 3" (SC 2011), restated from the paper:
ten rounds, each two 32 x 32 -> 64-bit multiplies (0xD2511F53 on word 0,
0xCD9E8D57 on word 2) whose high halves are mixed with the other words and
the key, the key bumped by the Weyl constants (0x9E3779B9, 0xBB67AE85)
between rounds. Pinned by the known-answer vectors the authors publish
(tests/test_device_sample_host.py). The device scene sampler
(csrc/sample.cu) is checked against it, and jitter() restates how that
sampler turns the generator's words into a particle's offsets.
"""
from __future__ import annotations

M0, M1 = 0xD2511F53, 0xCD9E8D57
W0, W1 = 0x9E3779B9, 0xBB67AE85
MASK = 0xFFFFFFFF


def philox4x32_10(counter, key):
    c = [int(x) & MASK for x in counter]
    k0, k1 = int(key[0]) & MASK, int(key[1]) & MASK
    for _ in range(10):
        p0 = M0 * c[0]
        p1 = M1 * c[2]
        hi0, lo0 = p0 >> 32, p0 & MASK
        hi1, lo1 = p1 >> 32, p1 & MASK
        c = [(hi1 ^ c[1] ^ k0) & MASK, lo1, (hi0 ^ c[3] ^ k1) & MASK, lo0]
        k0 = (k0 + W0) & MASK
        k1 = (k1 + W1) & MASK
    return c


def unit_double(a: int, b: int) -> float:
    """A double in [0, 1) from two words (27 + 26 high bits)."""
    return ((a >> 5) * 67108864.0 + (b >> 6)) * (1.0 / 9007199254740992.0)


def uniforms(particle: int, seed: int):
    """The three uniforms of particle number `particle` (x, y, z)."""
    k = (seed & MASK, (seed >> 32) & MASK)
    a = philox4x32_10((particle, 0, 0, 0), k)
    b = philox4x32_10((particle, 1, 0, 0), k)
    return unit_double(a[0], a[1]), unit_double(a[2], a[3]), unit_double(b[0], b[1])


def jitter(point, particle: int, seed: int, jitter_h: float):
    """The sampled coordinates: point + (u - 0.5) * (jitter * h), each in f64."""
    u = uniforms(particle, seed)
    return [p + (x - 0.5) * jitter_h for p, x in zip(point, u)]
