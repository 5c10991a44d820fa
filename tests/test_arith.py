"""Exact-arithmetic checks of the device's shortcuts (CPU only).

Each shortcut must give the reference's result bit for bit:
- the division-free byte conversion. The tile kernel converts texel and framebuffer bytes to
  float as the reference does, `(float)v / 255.0f`, but without a division: q = v * r with
  r = float(1/255), then one Markstein correction q' = fma(fma(-q, 255, v), r, q). Every byte
  value is checked against the correctly rounded quotient with exact rational arithmetic,
  rounding each step to float32 (round to nearest, ties to even) as the GPU's FMA and
  multiply do;
- the texel wrap shortcuts, the closed form of the line's Bresenham step, level 1 alone at
  mip weight 1, and small float/int conversions by directed-rounding additions;
- the exact coverage tests that let binning drop tiles and the tile kernel skip warp blocks.
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


# ---- exact coverage tests (binning per tile, the tile kernel per 8x4 block)

def _edges(x0, y0, x1, y1, x2, y2):
    """The record's edges as the tile kernel evaluates them: (ax, ay, A, B) with the edge
    function (px - ax) * A - (py - ay) * B, all float32 (integer-valued)."""
    f = np.float32
    X0, Y0, X1, Y1, X2, Y2 = (f(v) for v in (x0, y0, x1, y1, x2, y2))
    return [(X1, Y1, Y2 - Y1, X2 - X1), (X2, Y2, Y0 - Y2, X0 - X2), (X0, Y0, Y1 - Y0, X1 - X0)]


def _pixel_covered(edges, area, px, py):
    """The per-pixel coverage test in float32, as shade_pixel forms it."""
    f = np.float32
    e = [(f(px) - ax) * A - (f(py) - ay) * B for ax, ay, A, B in edges]
    return (area > 0 and all(v >= 0 for v in e)) or (area < 0 and all(v <= 0 for v in e))


def _block_mask_int(edges, area, tx0, ty0, box, ts=16):
    """block_mask (k_tile.cuh) for the tile at (tx0, ty0): (blocks the box meets, blocks the
    triangle is walked in), bit r * (ts / 8) + c for the 8x4 block at column c, row r."""
    mnx, mny, mxx, mxy = box
    kwx = ts // 8
    if mxx < tx0 or mnx > tx0 + ts - 1 or mxy < ty0 or mny > ty0 + ts - 1:
        return 0, 0
    c0, c1 = max(mnx - tx0, 0) >> 3, min(mxx - tx0, ts - 1) >> 3
    r0, r1 = max(mny - ty0, 0) >> 2, min(mxy - ty0, ts - 1) >> 2
    blocks = [(r, c) for r in range(r0, r1 + 1) for c in range(c0, c1 + 1)]
    boxbits = sum(1 << (r * kwx + c) for r, c in blocks)
    if not (area > 0 or area < 0):
        return boxbits, 0
    pos = area > 0
    steps = []
    for ax, ay, A, B in edges:
        if not all(abs(v) < 2 ** 24 for v in (ax, ay, A, B)):
            return boxbits, boxbits
        ax, ay, A, B = int(ax), int(ay), int(A), int(B)
        a, b = (A, B) if pos else (-A, -B)
        if max(abs(tx0 - ax), abs(tx0 + ts - 1 - ax)) * abs(a) >= 1 << 24 or \
                max(abs(ty0 - ay), abs(ty0 + ts - 1 - ay)) * abs(b) >= 1 << 24:
            return boxbits, boxbits
        e00 = (tx0 + (7 if a >= 0 else 0) - ax) * a - (ty0 + (0 if b >= 0 else 3) - ay) * b
        assert -(1 << 31) <= e00 < (1 << 31)
        steps.append((e00, 8 * a, 4 * b))
    mask = 0
    for r, c in blocks:
        if all(e00 + c * sx - r * sy >= 0 for e00, sx, sy in steps):
            mask |= 1 << (r * kwx + c)
    return boxbits, mask


def _tile_excluded_int(edges, area, tx0, ty0, tx1, ty1, ts):
    """The per-tile test of binning (k_bin.cu rec_tiles_of / tile_gets_pair): None when the
    per-record check fails (every tile kept), else the set of excluded tiles."""
    if (tx1 - tx0 + 1) * (ty1 - ty0 + 1) < 4:  # kTestMinTiles: small boxes keep every tile
        return None
    xl, xh, yl, yh = tx0 * ts, tx1 * ts + ts - 1, ty0 * ts, ty1 * ts + ts - 1
    pos = area > 0
    steps = []
    for ax, ay, A, B in edges:
        ax, ay, A, B = int(ax), int(ay), int(A), int(B)
        a, b = (A, B) if pos else (-A, -B)
        if max(abs(xl - ax), abs(xh - ax)) * abs(a) >= 1 << 24 or max(abs(yl - ay), abs(yh - ay)) * abs(b) >= 1 << 24:
            return None
        cx, cy = xl + (ts - 1 if a >= 0 else 0), yl + (0 if b >= 0 else ts - 1)
        e00 = (cx - ax) * a - (cy - ay) * b
        assert -(1 << 31) <= e00 < (1 << 31) and -(1 << 31) <= a * ts < (1 << 31)
        steps.append((e00, a * ts, b * ts))
    out = set()
    for ty in range(ty0, ty1 + 1):
        for tx in range(tx0, tx1 + 1):
            col, row = tx - tx0, ty - ty0
            if not all(e00 + col * sx - row * sy >= 0 for e00, sx, sy in steps):
                out.add((tx, ty))
    return out


def test_coverage_tests_never_drop_a_covered_pixel():
    """Random integer triangles (small, large, slivers, both orientations, some far off the
    pixels so that the exactness check is what decides): every 8x4 block the tile kernel
    skips and every tile binning drops holds no pixel the per-pixel float32 test covers, and
    a tile binning drops has no block the tile kernel walks."""
    rng = np.random.default_rng(7)
    ts = 16
    checked = dropped_blocks = dropped_tiles = 0
    for k in range(1500):
        scale = [6, 40, 300][k % 3]
        off = 0 if k % 7 else int(rng.integers(-3_000_000, 3_000_000))
        cx, cy = int(rng.integers(0, 200)), int(rng.integers(0, 200))
        xs = [cx + int(v) for v in rng.integers(-scale, scale + 1, 3)]
        ys = [cy + int(v) for v in rng.integers(-scale, scale + 1, 3)]
        if k % 11 == 0:
            xs[2] = xs[0] + (xs[1] - xs[0]) // 2 + 1  # near-degenerate sliver
        xs[0] += off
        f = np.float32
        area = (f(xs[2]) - f(xs[0])) * (f(ys[1]) - f(ys[0])) - (f(ys[2]) - f(ys[0])) * (f(xs[1]) - f(xs[0]))
        if abs(area) < 0.5:
            continue
        edges = _edges(xs[0], ys[0], xs[1], ys[1], xs[2], ys[2])
        minx, maxx = max(min(xs), 0), min(max(xs), 255)
        miny, maxy = max(min(ys), 0), min(max(ys), 255)
        if minx > maxx or miny > maxy:
            continue
        # the per-pixel float32 test over the box, vectorised (same operations, same order)
        gx, gy = np.meshgrid(np.arange(minx, maxx + 1, dtype=np.float32), np.arange(miny, maxy + 1, dtype=np.float32))
        e = [(gx - ax) * A - (gy - ay) * B for ax, ay, A, B in edges]
        cov = (e[0] >= 0) & (e[1] >= 0) & (e[2] >= 0) if area > 0 else (e[0] <= 0) & (e[1] <= 0) & (e[2] <= 0)

        def any_covered(x0_, x1_, y0_, y1_):
            x0_, y0_ = max(x0_, minx), max(y0_, miny)
            x1_, y1_ = min(x1_, maxx), min(y1_, maxy)
            return x0_ <= x1_ and y0_ <= y1_ and bool(cov[y0_ - miny:y1_ - miny + 1, x0_ - minx:x1_ - minx + 1].any())

        assert _pixel_covered(edges, area, int(gx.flat[0]), int(gy.flat[0])) == bool(cov.flat[0])
        box = (minx, miny, maxx, maxy)
        masks = {}
        for ty in range(miny // ts, maxy // ts + 1):
            for tx in range(minx // ts, maxx // ts + 1):
                boxbits, mask = _block_mask_int(edges, area, tx * ts, ty * ts, box, ts)
                masks[(tx, ty)] = mask
                assert mask & ~boxbits == 0
                for bit in range(ts * ts // 32):
                    if boxbits >> bit & 1 and not mask >> bit & 1:
                        dropped_blocks += 1
                        bx, by = tx * ts + 8 * (bit % (ts // 8)), ty * ts + 4 * (bit // (ts // 8))
                        assert not any_covered(bx, bx + 7, by, by + 3), (k, bx, by)
        tx0, ty0, tx1, ty1 = minx // ts, miny // ts, maxx // ts, maxy // ts
        ex = _tile_excluded_int(edges, area, tx0, ty0, tx1, ty1, ts)
        if ex is None:
            continue
        for tx, ty in ex:
            dropped_tiles += 1
            assert not any_covered(tx * ts, tx * ts + ts - 1, ty * ts, ty * ts + ts - 1), (k, tx, ty)
            assert masks[(tx, ty)] == 0, (k, tx, ty)
            checked += 1
    assert dropped_blocks > 2000 and dropped_tiles > 400 and checked > 400


# ---- the per-block depth bound (setup_fan_tri's depth plane, the tile kernel's bound)

def _depth_plane_f32(z, xs, ys, area, inv_area, minx, miny, maxx, maxy):
    """depth_plane (k_geom.cu), float32 operations in the same order."""
    f = np.float32
    z0, z1, z2 = (f(v) for v in z)
    fx0, fy0, fx1, fy1, fx2, fy2 = (f(v) for v in (xs[0], ys[0], xs[1], ys[1], xs[2], ys[2]))
    ea0, eb0, ea1, eb1, ea2, eb2 = fy2 - fy1, fx2 - fx1, fy0 - fy2, fx0 - fx2, fy1 - fy0, fx1 - fx0
    px, py = f(minx), f(miny)
    e0 = (px - fx1) * ea0 - (py - fy1) * eb0
    e1 = (px - fx2) * ea1 - (py - fy2) * eb1
    e2 = (px - fx0) * ea2 - (py - fy0) * eb2
    b0, b1, b2 = e0 * inv_area, e1 * inv_area, e2 * inv_area
    p0 = b0 * z0 + b1 * z1 + b2 * z2
    gx = (z0 * ea0 + z1 * ea1 + z2 * ea2) / area
    gy = -((z0 * eb0 + z1 * eb1 + z2 * eb2) / area)
    aa = abs(area)
    s0 = abs(b0 * z0) + abs(b1 * z1) + abs(b2 * z2)
    sx = (abs(z0 * ea0) + abs(z1 * ea1) + abs(z2 * ea2)) / aa
    sy = (abs(z0 * eb0) + abs(z1 * eb1) + abs(z2 * eb2)) / aa
    zabs = max(abs(z0), abs(z1), abs(z2))
    m = f(2.0 ** -20) * (s0 + sx * f(maxx - minx) + sy * f(maxy - miny) + zabs) + f(1e-37)
    if not all(np.isfinite(v) for v in (p0, gx, gy, m)):
        return f(0), f(0), f(0), f(np.inf)
    return p0, gx, gy, m


def _depth_plane_bound_f32(zp, minx, miny, xl, xh, yl, yh):
    """depth_plane_bound (mtgl_device.cuh) in float32."""
    f = np.float32
    p0, gx, gy, m = zp
    dx = f((xl if gx >= 0 else xh) - minx)
    dy = f((yl if gy >= 0 else yh) - miny)
    zz = (p0 + gx * dx) + gy * dy - m
    return (zz + f(1)) * f(0.5)


def test_depth_plane_bound_is_below_every_covered_fragment():
    """Random integer triangles (small to a few hundred pixels, slivers, both orientations)
    with vertex depths spread, nearly equal, or large: for every 8x4 block meeting the box,
    the bound over the block's part of the box is at most the depth the tile kernel computes
    for each covered pixel there (edge functions, b_i = e_i * inv_area, z = sum b_i z_i,
    (z + 1) * 0.5, all float32), and it is not vacuous on ordinary triangles."""
    f = np.float32
    rng = np.random.default_rng(11)
    blocks = tight = 0
    for k in range(900):
        scale = [5, 30, 120, 400][k % 4]
        cx, cy = int(rng.integers(0, 300)), int(rng.integers(0, 300))
        xs = [cx + int(v) for v in rng.integers(-scale, scale + 1, 3)]
        ys = [cy + int(v) for v in rng.integers(-scale, scale + 1, 3)]
        if k % 9 == 0:
            xs[2] = xs[0] + (xs[1] - xs[0]) // 2 + 1  # near-degenerate sliver
        kind = k % 5
        if kind == 0:
            z = rng.uniform(-1, 1, 3)
        elif kind == 1:
            z = 0.3 + rng.uniform(-1e-6, 1e-6, 3)
        elif kind == 2:
            z = rng.uniform(-1, 1, 3) * 1e4
        elif kind == 3:
            z = np.full(3, rng.uniform(-1, 1)) + np.array([0.0, 1e-7, -1e-7])
        else:
            z = rng.uniform(0.9, 1.0, 3)
        z = [f(v) for v in z]
        X0, Y0, X1, Y1, X2, Y2 = (f(v) for v in (xs[0], ys[0], xs[1], ys[1], xs[2], ys[2]))
        area = (X2 - X0) * (Y1 - Y0) - (Y2 - Y0) * (X1 - X0)
        if abs(area) < 0.5:
            continue
        sx_, sy_ = max(xs) - min(xs), max(ys) - min(ys)
        if sx_ and sy_ and sx_ * sy_ >= 1 << 23:
            continue  # depth_rejection's exactness condition: no plane
        inv_area = f(1) / area
        minx, maxx = max(min(xs), 0), min(max(xs), 511)
        miny, maxy = max(min(ys), 0), min(max(ys), 511)
        if minx > maxx or miny > maxy:
            continue
        zp = _depth_plane_f32(z, xs, ys, area, inv_area, minx, miny, maxx, maxy)
        edges = _edges(xs[0], ys[0], xs[1], ys[1], xs[2], ys[2])
        gx, gy = np.meshgrid(np.arange(minx, maxx + 1, dtype=np.float32), np.arange(miny, maxy + 1, dtype=np.float32))
        e = [(gx - ax) * A - (gy - ay) * B for ax, ay, A, B in edges]
        cov = (e[0] >= 0) & (e[1] >= 0) & (e[2] >= 0) if area > 0 else (e[0] <= 0) & (e[1] <= 0) & (e[2] <= 0)
        b = [ei * inv_area for ei in e]
        zz = b[0] * z[0] + b[1] * z[1] + b[2] * z[2]
        depth = (zz + f(1)) * f(0.5)
        for by in range(miny - miny % 4, maxy + 1, 4):
            for bx in range(minx - minx % 8, maxx + 1, 8):
                xl, xh, yl, yh = max(bx, minx), min(bx + 7, maxx), max(by, miny), min(by + 3, maxy)
                sub = cov[yl - miny:yh - miny + 1, xl - minx:xh - minx + 1]
                if not sub.any():
                    continue
                lo = _depth_plane_bound_f32(zp, minx, miny, xl, xh, yl, yh)
                dmin = depth[yl - miny:yh - miny + 1, xl - minx:xh - minx + 1][sub].min()
                assert lo <= dmin, (k, bx, by, float(lo), float(dmin))
                blocks += 1
                if kind == 0 and dmin - lo < 1e-4:
                    tight += 1
    assert blocks > 20000 and tight > 1000
