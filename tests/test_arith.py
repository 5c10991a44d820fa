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


def _bresenham(x0, y0, x1, y1):
    """draw_line_full's pixel loop (raster.c:107-241), positions only."""
    dx, dy = x1 - x0, y1 - y0
    adx, ady = abs(dx), abs(dy)
    sx, sy = (-1 if dx < 0 else 1), (-1 if dy < 0 else 1)
    err, cx, cy, out = adx - ady, x0, y0, []
    while True:
        out.append((cx, cy))
        if cx == x1 and cy == y1:
            return out
        e2 = 2 * err
        if e2 > -ady:
            err -= ady
            cx += sx
        if e2 < adx:
            err += adx
            cy += sy


def test_line_step_closed_form_matches_the_loop():
    """The tile kernel's closed form of the Bresenham step (shade_prim) against the loop."""
    n = 130
    for dx in range(-n, n + 1):
        for dy in range(-n, n + 1, 1 if abs(dx) < 20 else 7):
            pts = _bresenham(3, -5, 3 + dx, -5 + dy)
            adx, ady = abs(dx), abs(dy)
            sx, sy = (-1 if dx < 0 else 1), (-1 if dy < 0 else 1)
            assert len(pts) == max(adx, ady) + 1
            for k, (cx, cy) in enumerate(pts):
                if adx > ady:
                    want = (3 + sx * k, -5 + sy * ((2 * ady * k + adx - 1) // (2 * adx)))
                elif ady > 0:
                    want = (3 + sx * ((2 * adx * k + ady - 1) // (2 * ady)), -5 + sy * k)
                else:
                    want = (3, -5)
                assert (cx, cy) == want, (dx, dy, k)


def test_mip_blend_at_weight_one_returns_level_one():
    """sample_lod skips level 0 from lod 1 up: lerp_col(c0, c1, 1) = c0 * 0 + c1 * 1 is c1's
    channel value exactly, and packing a channel value back gives the byte: trunc(round(
    round(b / 255) * 255)) == b for every byte, computed here with exact rationals rounded
    to float32 at each step (the same steps as unpack_rgba / pack_rgba)."""
    for b in range(256):
        u = round_f32(Fr(b, 255))
        assert u * 0 + u * 1 == u
        back = round_f32(u * 255)
        assert back.numerator // back.denominator == b, b


def test_small_conversions_by_directed_rounding():
    """small_trunc / small_floor / small_u2f: adding 2^23 (1.5 * 2^23) rounded toward zero
    (down) leaves the integer part in the low mantissa bits. Checked on the boundaries and
    on random values with exact rationals, rounding as the GPU's fadd.rz / fadd.rm do."""
    def add_directed(a: Fr, b: Fr, mode: str) -> Fr:
        s = a + b  # positive, in [2^23, 2^24): float32 spacing is 1, so both modes floor
        assert mode in ("rz", "rd") and 2 ** 23 <= s < 2 ** 24
        return Fr(s.numerator // s.denominator)
    rng = np.random.default_rng(3)
    vals = [0.0, 0.5, 1.0, 254.999, 255.0, 2.0 ** 22 - 0.5] + list(rng.uniform(0, 2 ** 22, 200))
    for v in vals:
        f = Fr(float(np.float32(v)))
        t = add_directed(f, Fr(2 ** 23), "rz") - 2 ** 23
        assert t == int(float(f)), v
    for v in [-2.0 ** 22, -1.5, -1.0, -0.5, -1e-7, 0.0, 0.25, 7.75] + list(rng.uniform(-2 ** 22, 2 ** 22, 200)):
        f = Fr(float(np.float32(v)))
        s = add_directed(f, Fr(3 * 2 ** 22), "rd")
        assert s - 3 * 2 ** 22 == np.floor(float(f)), v
    for v in (0, 1, 255, 2 ** 23 - 1):
        assert np.array([0x4B000000 | v], np.uint32).view(np.float32)[0] - np.float32(2 ** 23) == v
