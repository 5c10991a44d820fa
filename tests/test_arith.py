"""Exact-arithmetic checks of the device's division-free byte conversion (CPU only).

The tile kernel converts texel and framebuffer bytes to float as the reference does,
`(float)v / 255.0f`, but without a division: q = v * r with r = float(1/255), then one
Markstein correction q' = fma(fma(-q, 255, v), r, q). Here every byte value is checked
against the correctly rounded quotient with exact rational arithmetic, rounding each
step to float32 (round to nearest, ties to even) as the GPU's FMA and multiply do.
"""
from fractions import Fraction as Fr

import numpy as np


def round_f32(q: Fr) -> Fr:
    """Nearest float32 to the rational q (ties to even); normal range only."""
    if q == 0:
        return Fr(0)
    sign = -1 if q < 0 else 1
    q = abs(q)
    e = q.numerator.bit_length() - q.denominator.bit_length()
    while Fr(2) ** e > q:
        e -= 1
    while Fr(2) ** (e + 1) <= q:
        e += 1
    ulp = Fr(2) ** (e - 23)
    m = q / ulp
    fl = m.numerator // m.denominator
    rem = m - fl
    if rem > Fr(1, 2) or (rem == Fr(1, 2) and fl % 2 == 1):
        fl += 1
    return sign * fl * ulp


def test_reciprocal_constant():
    r = round_f32(Fr(1, 255))
    assert float(r) == float(np.float32(1) / np.float32(255)) == float.fromhex("0x1.010102p-8")


def test_byte_over_255_is_exact_for_every_byte():
    r = round_f32(Fr(1, 255))
    for v in range(256):
        q = round_f32(v * r)
        e = round_f32(-q * 255 + v)
        q2 = round_f32(e * r + q)
        assert q2 == round_f32(Fr(v, 255)), v
        assert float(q2) == float(np.float32(v) / np.float32(255)), v


def _c_mod(x, n):
    """C's % on int32: truncated division."""
    q = abs(x) // abs(n)
    q = q if (x >= 0) == (n >= 0) else -q
    return x - q * n


def test_texel_wrap_shortcuts_match_reference_rule():
    """wrap_coord / wrap_next (GL_REPEAT) against get_texel_wrapped's ((x % n) + n) % n."""
    xs = list(range(-5000, 5000)) + [-2**31, -2**31 + 1, -2**31 + 2, 2**31 - 128, 2**31 - 129]
    for n in (1, 2, 4, 8, 64, 256, 512, 2048, 3, 5, 100, 1000, 2047):
        pow2 = (n & (n - 1)) == 0
        for x in xs:
            ref = _c_mod(_c_mod(x, n) + n, n)
            fast = (x & (n - 1)) if pow2 else ref
            assert fast == ref, (x, n)
            if x + 1 < 2**31:
                nxt = 0 if fast + 1 == n else fast + 1
                assert nxt == _c_mod(_c_mod(x + 1, n) + n, n), (x, n)
