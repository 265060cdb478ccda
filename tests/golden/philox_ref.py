"""Scalar Python Philox4x32-10 (test infrastructure).

Philox4x32-10 is the counter-based generator of Salmon, Moraes, Dror and Shaw,
"Parallel random numbers: as easy as 1, 2, 3" (SC 2011).  The project uses it
to draw pipe-respawn positions: one call per uniform, key = the scene seed,
counter = (draw, step, particle id, 0).  A uniform double in [0, 1) takes the
top 53 bits of the first two output words.
"""

M0 = 0xD2511F53
M1 = 0xCD9E8D57
W0 = 0x9E3779B9
W1 = 0xBB67AE85
MASK = 0xFFFFFFFF


def philox4x32_10(ctr, key):
    c0, c1, c2, c3 = (int(v) & MASK for v in ctr)
    k0, k1 = (int(v) & MASK for v in key)
    for r in range(10):
        p0 = M0 * c0
        p1 = M1 * c2
        hi0, lo0 = p0 >> 32, p0 & MASK
        hi1, lo1 = p1 >> 32, p1 & MASK
        c0, c1, c2, c3 = (hi1 ^ c1 ^ k0), lo1, (hi0 ^ c3 ^ k1), lo0
        if r != 9:
            k0 = (k0 + W0) & MASK
            k1 = (k1 + W1) & MASK
    return c0, c1, c2, c3


def philox_uniform_f64(seed: int, pid: int, step: int, draw: int) -> float:
    seed = int(seed) & 0xFFFFFFFFFFFFFFFF
    x0, x1, _, _ = philox4x32_10((draw, step, pid, 0), (seed & MASK, seed >> 32))
    bits53 = (x0 << 21) | (x1 >> 11)
    return bits53 * (1.0 / 9007199254740992.0)
