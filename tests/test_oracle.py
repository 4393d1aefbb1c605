"""CPU tests of the oracle: pinned to the reference's own shaders (golden
fixtures and, where the reference checkout exists, a live run), plus
known-answer tests derived from the shader arithmetic."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import assert_bitexact, load_golden


# ---------------------------------------------------------------- generator KATs

def test_pcg32_published_known_answer(oracle):
    # pcg32-demo (pcg-random.org) with pcg32_srandom_r(&rng, 42u, 54u).
    want = [0xa15c02b7, 0x7b47f409, 0xba1d3330, 0x83d2f293, 0xbfa4784b, 0xcbed606e]
    assert oracle.pcg32(42, 54, 6).tolist() == want


def test_pcg32_jump_ahead_matches_sequential(oracle):
    seq = oracle.pcg32(2026, 3, 1000)
    for skip in (0, 1, 7, 511, 999):
        assert oracle.pcg32(2026, 3, 1, skip=skip)[0] == seq[skip]


def test_terrain_definition(oracle):
    b, d = oracle.terrain(2026, 256, 256, 40.0, 15.0)
    assert b.dtype == np.float32 and b.shape == (256, 256)
    assert 0.0 <= b.min() and b.max() < 40.0
    assert_bitexact(d, np.maximum(np.float32(0), np.float32(15.0) - b), "depth")
    b2, _ = oracle.terrain(2026, 256, 256, 40.0, 15.0)
    assert_bitexact(b2, b, "determinism")
    b3, _ = oracle.terrain(2027, 256, 256, 40.0, 15.0)
    assert not np.array_equal(b3, b)


# ---------------------------------------------------------------- pinning to the reference

@pytest.mark.parametrize("case", ["ref_brush_64", "ref_bumps_48x32"])
def test_oracle_matches_reference_golden(oracle, case):
    g = load_golden(case)
    kf, ka, c = g["params"].tolist()
    b, d, f = g["b"].copy(), g["d0"].copy(), g["f0"].copy()
    H, W = b.shape
    v = np.zeros((H, W, 2), np.float32)
    if g["brush"].size:
        bx, by, intensity, size_sq = g["brush"].tolist()
        oracle.sources_f32(d, [(oracle.SOURCE_BRUSH, bx, by, size_sq, intensity)])
    oracle.step_f32(b, d, f, v, kf, ka, c, oracle.BOUNDARY_OPEN, nsteps=int(g["steps"]))
    assert_bitexact(d, g["d"], "depth")
    assert_bitexact(f, g["f"], "flux")
    assert np.array_equal(v.astype(np.float16).view(np.uint16), g["flowmap_f16"]), "flow map"


def _ref_or_skip(oracle):
    if not oracle.ref_available():
        pytest.skip("reference shaders not built here (no reference checkout)")


# The reference dispatches its brush as glDispatchCompute(N/32, N/32) with
# 32x32 workgroups (Terrain.cpp:167), so it reaches only floor(N/32)*32 cells
# per axis; the step shaders need N % 16 == 0 (Terrain.cpp:258, 264).  Sizes
# here are multiples of 32, where the brush covers the whole grid.
@pytest.mark.parametrize("W,H,seed", [(32, 32, 1), (32, 64, 2), (96, 64, 3), (128, 128, 4)])
def test_oracle_matches_reference_live(oracle, W, H, seed):
    _ref_or_skip(oracle)
    b, d = oracle.terrain(seed, W, H, 40.0, 15.0)
    rng = np.random.default_rng(seed)
    f = rng.uniform(0, 0.2, (H, W, 4)).astype(np.float32)
    kf, ka, c = oracle.params_reference(60.0, 0.97, 20.0, float(W), W)
    brush = (W * 0.37, H * 0.61, 2.5, 32.0)
    rd, rf, rfm = oracle.ref_steps(b, d, f, kf, ka, c, 40, brush=brush)
    od, of = d.copy(), f.copy()
    ov = np.zeros((H, W, 2), np.float32)
    oracle.sources_f32(od, [(oracle.SOURCE_BRUSH, brush[0], brush[1], brush[3], brush[2])])
    oracle.step_f32(b, od, of, ov, kf, ka, c, oracle.BOUNDARY_OPEN, nsteps=40)
    assert_bitexact(od, rd, "depth")
    assert_bitexact(of, rf, "flux")
    assert np.array_equal(ov.astype(np.float16).view(np.uint16), rfm)


# ---------------------------------------------------------------- known-answer tests

def _bench_params(oracle):
    kf, ka, c = oracle.params_physical(0.02, 9.81, 1.0, 1.0, 0.998)
    return np.float32(kf), np.float32(ka), np.float32(c)


def test_lake_at_rest_is_exact(oracle):
    """b + d = const everywhere -> every surface difference is 0, flux stays
    exactly 0 and depth is unchanged bit for bit (closed walls)."""
    rng = np.random.default_rng(7)
    b = (rng.integers(0, 40, (40, 56)) / 8.0).astype(np.float32)
    d = (np.float32(10.0) - b).astype(np.float32)
    assert np.all(d + b == np.float32(10.0))
    f = np.zeros((40, 56, 4), np.float32)
    v = np.zeros((40, 56, 2), np.float32)
    d0 = d.copy()
    oracle.step_f32(b, d, f, v, *_bench_params(oracle), boundary=oracle.BOUNDARY_CLOSED, nsteps=100)
    assert_bitexact(d, d0, "depth")
    assert not f.any() and not v.any()


def test_single_column_first_step(oracle):
    """One wet cell on flat dry ground: each outflow is Ka*d0 before scaling;
    the scaling engages iff 4*Ka*d0*C > d0; neighbours receive the outflow."""
    kf, ka, c = _bench_params(oracle)
    for d0 in (np.float32(1.0), np.float32(37.5)):
        for ka_s in (ka, np.float32(20.0)):   # 20 makes 4*Ka*C > 1 -> scaling
            W = H = 9
            b = np.zeros((H, W), np.float32)
            d = np.zeros((H, W), np.float32)
            d[4, 4] = d0
            f = np.zeros((H, W, 4), np.float32)
            v = np.zeros((H, W, 2), np.float32)
            oracle.step_f32(b, d, f, v, kf, ka_s, c, boundary=oracle.BOUNDARY_CLOSED, nsteps=1)
            nf = np.float32(d0 * ka_s)
            total = np.float32(np.float32(np.float32(np.float32(nf + nf) + nf) + nf) * c)
            if total > d0:
                nf = np.float32(nf * np.float32(d0 / total))
                assert 4 * ka_s * d0 * c > d0
            assert np.all(f[4, 4] == nf)
            out = np.float32(np.float32(np.float32(nf + nf) + nf) + nf)
            want_c = np.maximum(np.float32(0), np.float32(d0 + np.float32(np.float32(0) - out) * c))
            assert d[4, 4] == want_c
            for (y, x) in ((4, 5), (4, 3), (5, 4), (3, 4)):
                assert d[y, x] == np.float32(nf * c)
            rest = d.copy()
            rest[4, 3:6] = 0
            rest[3:6, 4] = 0
            assert not rest.any(), "water moved beyond the four neighbours in one step"


def test_volume_conserved_closed(oracle):
    b, d = oracle.terrain(5, 96, 64, 40.0, 15.0)
    f = np.zeros((64, 96, 4), np.float32)
    v0 = oracle.volume(d)
    oracle.step_f32(b, d, f, None, *_bench_params(oracle), boundary=oracle.BOUNDARY_CLOSED,
                    nsteps=500)
    assert abs(oracle.volume(d) - v0) <= 1e-6 * v0
    assert d.min() >= 0 and f.min() >= 0
    # FP64 path: conserved to round-off
    kf, ka, c = oracle.params_physical()
    b64, d64 = oracle.terrain(5, 96, 64, 40.0, 15.0)
    b64, d64 = b64.astype(np.float64), d64.astype(np.float64)
    f64 = np.zeros((64, 96, 4), np.float64)
    w0 = oracle.volume(d64)
    oracle.step_f64(b64, d64, f64, None, kf, ka, c, boundary=oracle.BOUNDARY_CLOSED, nsteps=500)
    assert abs(oracle.volume(d64) - w0) <= 1e-12 * w0


def test_rain_adds_exact_volume_closed(oracle):
    W = H = 64
    b, d = oracle.terrain(9, W, H, 40.0, 15.0)
    f = np.zeros((H, W, 4), np.float64)
    b, d = b.astype(np.float64), d.astype(np.float64)
    (cx, cy), = oracle.rain_centers(9, W, H, 8, 1)
    n_in = sum(1 for y in range(H) for x in range(W) if (x - cx) ** 2 + (y - cy) ** 2 <= 64)
    v0 = oracle.volume(d)
    oracle.step_f64(b, d, f, None, *oracle.params_physical(), boundary=oracle.BOUNDARY_CLOSED,
                    sources=[(oracle.SOURCE_DISK, cx, cy, 8, 0.01)], nsteps=50)
    assert abs(oracle.volume(d) - (v0 + 50 * 0.01 * n_in)) <= 1e-9 * v0


def test_mirror_symmetry(oracle):
    """An x-mirrored scene stays mirrored: +x/-x outflows swap, v.x changes
    sign, all bit for bit (the shaders' sums are commutative pairs)."""
    W, H = 64, 48
    b, _ = oracle.terrain(3, W // 2, H, 40.0, 15.0)
    b = np.ascontiguousarray(np.concatenate([b, b[:, ::-1]], axis=1))
    d = np.maximum(np.float32(0), np.float32(15.0) - b).astype(np.float32)
    f = np.zeros((H, W, 4), np.float32)
    v = np.zeros((H, W, 2), np.float32)
    oracle.step_f32(b, d, f, v, *_bench_params(oracle), boundary=oracle.BOUNDARY_CLOSED,
                    sources=[(oracle.SOURCE_BRUSH, (W - 1) / 2.0, 20.0, 30.0, 0.5)], nsteps=200)
    assert_bitexact(d, np.ascontiguousarray(d[:, ::-1]), "depth mirror")
    fm = f[:, ::-1]
    assert_bitexact(f[..., 0], np.ascontiguousarray(fm[..., 1]), "+x vs -x")
    assert_bitexact(f[..., 2], np.ascontiguousarray(fm[..., 2]), "+y")
    # (a - b) and -(b - a) are equal but differ in the sign of an exact zero
    assert np.array_equal(v[..., 0], -v[:, ::-1, 0]), "v.x"
    assert_bitexact(v[..., 1], np.ascontiguousarray(v[:, ::-1, 1]), "v.y")


def test_fp32_tracks_fp64(oracle):
    """The FP32 transcription stays close to the FP64 oracle on the 256^2
    benchmark scene (1000 steps, closed walls, rain disk r=16)."""
    W = H = 256
    b, d = oracle.terrain(2026, W, H, 40.0, 15.0)
    (cx, cy), = oracle.rain_centers(2026, W, H, 16, 1)
    src = [(oracle.SOURCE_DISK, cx, cy, 16, 0.01)]
    kf, ka, c = oracle.params_physical()
    b64, d64 = b.astype(np.float64), d.astype(np.float64)
    f32 = np.zeros((H, W, 4), np.float32)
    f64 = np.zeros((H, W, 4), np.float64)
    oracle.step_f32(b, d, f32, None, np.float32(kf), np.float32(ka), np.float32(c),
                    boundary=oracle.BOUNDARY_CLOSED, sources=src, nsteps=1000)
    oracle.step_f64(b64, d64, f64, None, kf, ka, c, boundary=oracle.BOUNDARY_CLOSED, sources=src,
                    nsteps=1000)
    v32, v64 = oracle.volume(d), oracle.volume(d64)
    assert abs(v32 - v64) / v64 < 1e-5
    assert np.abs(d - d64).max() < 1e-2 * max(1.0, d64.max())


def test_fp16_storage_mode_quantizes(oracle):
    W = H = 64
    b, d = oracle.terrain(2, W, H, 40.0, 15.0)
    f = np.zeros((H, W, 4), np.float32)
    oracle.step_f32(b, d, f, None, *_bench_params(oracle), boundary=oracle.BOUNDARY_CLOSED,
                    nsteps=20, flux_scale=32.0)
    q = f.copy()
    oracle.quantize_f16(q, 32.0)
    assert_bitexact(q, f, "stored flux is a scaled half")


def test_reference_parameter_derivation(oracle):
    # Terrain.cpp:175-198 at the app defaults: 60 steps/s, damping 0.98, accel 10,
    # world 1024 over 1024 cells.
    kf, ka, c = oracle.params_reference(60.0, 0.98, 10.0, 1024.0, 1024)
    step = np.float64(np.float32(1.0) / np.float32(60.0))
    assert kf == np.float32(np.power(np.float32(0.98), np.float32(step), dtype=np.float32)) or \
        abs(kf - 0.98 ** step) < 1e-7
    assert ka == np.float32(step * 10.0 * 1.0)
    assert c == np.float32(step / 1.0)


# ------------------------------------------------------------ the reference's noise scene

def test_reference_noise_scene_matches_fixture(oracle):
    """The restated noise table and scene equal the reference's own
    Random.cpp / NoiseGenerator.cpp output (tests/golden/ref_noise_scene_96.npz)."""
    g = load_golden("ref_noise_scene_96")
    for gen in (0, 1):
        t = oracle.reference_noise_table(int(g["seed"]), gen)
        assert np.array_equal(t.view(np.uint32), g[f"table{gen}"].view(np.uint32))
        b, d = oracle.reference_terrain(96, 96, float(g["height_scale"]), int(g["seed"]), gen)
        assert_bitexact(b, g[f"b{gen}"], f"terrain {gen}")
        assert_bitexact(d, g[f"d{gen}"], f"depth {gen}")
    assert (g["d0"] > 0).any() and (g["d0"] == 0).any()  # the central pool and dry land


@pytest.mark.parametrize("N,gen,seed", [(64, 0, 231656522), (257, 2, 231656522), (130, 1, 7)])
def test_reference_noise_scene_live(oracle, N, gen, seed):
    """Against the reference's noise code compiled here (make -C oracle ref)."""
    if not oracle.ref_noise_available():
        pytest.skip("reference checkout not available")
    R = oracle.ref_noise()
    rb = np.empty((N, N), np.float32)
    rd = np.empty((N, N), np.float32)
    R.tws_ref_reference_terrain(seed, gen, N, 300.0, oracle._fp(rb), oracle._fp(rd))
    b, d = oracle.reference_terrain(N, N, 300.0, seed, gen)
    assert_bitexact(b, rb, "terrain")
    assert_bitexact(d, rd, "depth")


# ---------------------------------------------------------------- the renderer's reads, pinned

RENDER_KEYS = ("height", "render_height", "normal", "flow_speed", "foam")


def test_oracle_surface_matches_reference_render_golden(oracle):
    """The oracle's renderer-side arithmetic against the reference's own
    water-rendering shader code (waterRender.vert, .eval main(), .frag
    ComputeHeightmapNormal and flow speed), run on the CPU by make_golden.py."""
    import sys
    sys.path.insert(0, str(__import__("pathlib").Path(__file__).parent / "golden"))
    import make_golden

    g = load_golden("ref_render_64")
    b, d, v = make_golden.render_case_state()
    assert_bitexact(b, g["b"], "terrain")
    assert_bitexact(d, g["d"], "depth")
    assert_bitexact(v, g["v"], "flow map (float)")
    assert g["out_dry"].any() and (g["out_flow_speed"] > 0).any()  # the case exercises both
    got = oracle.surface(g["b"], g["d"], g["v"])
    for k in RENDER_KEYS:
        assert_bitexact(got[k], g["out_" + k], k)
    assert np.array_equal(got["dry"], g["out_dry"])


@pytest.mark.parametrize("N,seed", [(32, 5), (64, 6), (128, 7)])
def test_oracle_surface_matches_reference_render_live(oracle, N, seed):
    if not oracle.ref_render_available():
        pytest.skip("reference render shaders not built here (no reference checkout)")
    rng = np.random.default_rng(seed)
    b = rng.uniform(0.0, 10.0, (N, N)).astype(np.float32)
    d = np.maximum(0.0, rng.uniform(-1.0, 2.0, (N, N))).astype(np.float32)
    d[: N // 4] = 0.0
    b[: N // 8] = 3.0  # flat dry rows: zero slopes, whose signs the normal keeps
    v = rng.uniform(-40.0, 40.0, (N, N, 2)).astype(np.float32)
    want = oracle.ref_surface(b, d, v.astype(np.float16).view(np.uint16))
    got = oracle.surface(b, d, v)
    for k in RENDER_KEYS:
        assert not np.isnan(want[k]).any(), k  # every sample was a texel centre
        assert_bitexact(got[k], want[k], k)
    assert np.array_equal(got["dry"], want["dry"])


# ---------------------------------------------------------------- DISK rain rounding

@pytest.mark.parametrize("depth", [3.0, 12.0, 20.0, 40.0, 100.0])
def test_disk_rain_rounding_is_unbiased(oracle, depth):
    """Round to nearest biases d + 0.01 by a fixed fraction of an ulp of d in
    each binade (+2.3e-5 of the rain on 8-32 m, -1.7e-4 on 32-64 m); the DISK
    source's unbiased rounding adds the rate exactly in expectation, and is
    deterministic."""
    N, reps = 64, 400
    d = np.full((N, N), np.float32(depth))
    rate = np.float32(0.01)
    src = [(oracle.SOURCE_DISK, 32, 32, 100, 0.01)]  # every cell
    d2 = d.copy()
    for _ in range(reps):
        oracle.sources_f32(d, src)
        oracle.sources_f32(d2, src)
    assert_bitexact(d, d2, "determinism")
    added = float(np.sum(d, dtype=np.float64) - N * N * float(np.float32(depth)))
    want = reps * N * N * float(rate)
    # round to nearest on the same adds, for scale
    rn = np.full((N, N), np.float32(depth))
    for _ in range(reps):
        rn = (rn + rate).astype(np.float32)
    rn_bias = abs(float(np.sum(rn, dtype=np.float64)) - N * N * float(np.float32(depth)) - want)
    assert abs(added - want) / want < 2e-6, (added, want)
    assert abs(added - want) < 0.1 * rn_bias or rn_bias == 0.0
