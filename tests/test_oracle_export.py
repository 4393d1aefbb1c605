"""CPU checks of the oracle's renderer-side arithmetic against an independent
numpy restatement (float32 numpy operations are IEEE round-to-nearest with no
multiply-add fusion, like the oracle)."""
from __future__ import annotations

import numpy as np

from conftest import assert_bitexact


def test_surface_matches_numpy(oracle):
    rng = np.random.default_rng(2)
    H, W = 23, 31
    b = rng.uniform(0, 10, (H, W)).astype(np.float32)
    d = np.maximum(0, rng.uniform(-1, 2, (H, W))).astype(np.float32)
    v = rng.uniform(-40, 40, (H, W, 2)).astype(np.float32)
    got = oracle.surface(b, d, v)
    f32 = np.float32
    h = (d + b).astype(np.float32)
    assert_bitexact(got["height"], h, "height")
    rh = (h - f32(0.1)).astype(np.float32)
    rh = np.where(d < f32(0.1), (rh - f32(10.0)).astype(np.float32), rh)
    assert_bitexact(got["render_height"], rh, "render_height")
    assert np.array_equal(got["dry"], (d < f32(0.1)).astype(np.uint8))
    A = (np.roll(h, -1, axis=0) - np.roll(h, 1, axis=0)).astype(np.float32)  # h(y+1) - h(y-1)
    B = (np.roll(h, -1, axis=1) - np.roll(h, 1, axis=1)).astype(np.float32)  # h(x+1) - h(x-1)
    # GLSL cross((0, A, 1), (1, B, 0)) product by product: (A*0 - B, 1, 0*B - A)
    zero = np.float32(0.0)
    nx, ny, nz = (A * zero - B).astype(np.float32), np.ones_like(B), (zero * B - A).astype(np.float32)
    ln = np.sqrt(((nx * nx + ny * ny) + nz * nz).astype(np.float32)).astype(np.float32)
    n = np.stack([nx / ln, ny / ln, nz / ln], axis=-1).astype(np.float32)
    assert_bitexact(got["normal"], n, "normal")
    fl = v.astype(np.float16).astype(np.float32)
    s2 = (fl[..., 0] * fl[..., 0] + fl[..., 1] * fl[..., 1]).astype(np.float32)
    assert_bitexact(got["flow_speed"], np.sqrt(s2).astype(np.float32), "flow_speed")
    assert_bitexact(got["foam"], np.clip(s2 * f32(0.00004), 0, 1).astype(np.float32), "foam")


def test_mips_match_numpy(oracle):
    rng = np.random.default_rng(3)
    H, W = 37, 52
    b = rng.uniform(0, 10, (H, W)).astype(np.float32)
    d = rng.uniform(0, 3, (H, W)).astype(np.float32)
    rgba, mips = oracle.terrain_mips(b, d, 3)
    want = np.stack([b, np.full_like(b, 0.3), np.full_like(b, 0.3), d], axis=-1)
    assert_bitexact(rgba, want, "rgba")
    src = want
    for m in mips:
        h2, w2 = src.shape[0] // 2, src.shape[1] // 2
        s = src[:2 * h2, :2 * w2]
        t00, t10 = s[0::2, 0::2], s[0::2, 1::2]
        t01, t11 = s[1::2, 0::2], s[1::2, 1::2]
        exp = (((t00 + t10).astype(np.float32) + (t01 + t11).astype(np.float32)).astype(np.float32)
               * np.float32(0.25)).astype(np.float32)
        assert_bitexact(m, exp, "mip")
        src = exp
