"""CPU: the shuffle's nextInt remainder by reciprocal multiplication.

k_world_init (betaseedfinder_gb300/csrc/bsf_stage0.cu) takes r % b, for the
non-power-of-two bounds b = 256 - i of the Fisher-Yates shuffle and 31-bit
draws r, as r - b * umulhi64(r, M[b]) with M[b] = floor(2^64 / b) + 1 (the host
fills the table as ~0 / b + 1). The quotient must equal r // b for every r the
LCG can produce; Java's rejection test then reads the same remainder.
"""
import numpy as np

MASK64 = (1 << 64) - 1


def magic(b):
    return (MASK64 // b + 1) & MASK64  # the host's ~0ULL / b + 1


def test_table_matches_floor_two_pow_64_over_b_plus_one():
    for b in range(3, 257):
        if b & (b - 1):
            assert magic(b) == (1 << 64) // b + 1  # b is no power of two: 2^64 / b is not an integer


def test_quotient_exact_for_all_bounds():
    rng = np.random.default_rng(3)
    for b in range(3, 256):
        if not b & (b - 1):
            continue
        m = magic(b)
        rs = set(int(x) for x in rng.integers(0, 2 ** 31, 4000))
        rs.update([0, 1, b - 1, b, b + 1, 2 ** 31 - 1, 2 ** 31 - 2])
        top = (2 ** 31 - 1) // b
        for k in list(range(1, 300)) + list(range(top - 300, top + 1)):
            for d in (-1, 0, 1):  # every multiple of b and its neighbours at both ends of the range
                r = k * b + d
                if 0 <= r < 2 ** 31:
                    rs.add(r)
        for r in rs:
            q = (r * m) >> 64  # umulhi64(r, m)
            assert q == r // b, (b, r)
            assert r - q * b == r % b


def test_overshoot_bound():
    # the argument: r * m / 2^64 - r / b < r / 2^64 <= 2^-33, while the fractional
    # part of r / b is at most 1 - 1/b <= 1 - 1/255
    for b in range(3, 256):
        if b & (b - 1):
            over = magic(b) * b - (1 << 64)  # b * (m - 2^64 / b), exactly: 0 < m - 2^64 / b <= 1
            assert 0 < over <= b
            # r * (m - 2^64/b) / 2^64 < 2^31 / 2^64 < 1 / b for every 31-bit r
            assert (1 << 31) * b < (1 << 64)
