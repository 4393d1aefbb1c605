"""GPU parity tests: the fused sm_103a step through the C ABI against the
oracle (bit-exact for FP32 storage) and against the reference-pinned golden
fixtures; full-size properties at 4096^2."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import assert_bitexact, load_golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def tws():
    import terrainwatersim_gb300 as t
    t.lib()
    return t


def oracle_run(O, b, d, f, params, sources, steps, boundary, flux_scale=0.0):
    b, d, f = b.copy(), d.copy(), f.copy()
    H, W = b.shape
    v = np.zeros((H, W, 2), np.float32)
    kf, ka, c = params
    O.step_f32(b, d, f, v, kf, ka, c, boundary, [(s[0], s[1], s[2], s[3], s[4]) for s in sources],
               nsteps=steps, flux_scale=flux_scale)
    return d, f, v


def gpu_run(tws, b, d, f, params, sources, steps, k, flux_storage=0, one_shot=None):
    H, W = b.shape
    with tws.Grid(W, H, params, flux_storage) as g:
        g.upload(b, d, f)
        if one_shot is not None:
            g.apply_source(one_shot)
        g.set_sources(sources)
        g.set_steps_per_launch(k)
        g.step(steps)
        g.sync()
        out = g.download()
        vol = g.volume()
        scale = g.buffers().flux_scale
    return out + (vol, scale)


# ------------------------------------------------------------ reference-pinned fixtures

@pytest.mark.parametrize("k", [1, 2, 3, 4])
@pytest.mark.parametrize("case", ["ref_brush_64", "ref_bumps_48x32"])
def test_golden_reference_fixtures(tws, case, k):
    g = load_golden(case)
    H, W = g["b"].shape
    kf, ka, c = g["params"].tolist()
    p = tws.SimParams(kf, ka, c, 1.0, tws.BOUNDARY_OPEN)
    one_shot = None
    if g["brush"].size:
        bx, by, intensity, size_sq = g["brush"].tolist()
        one_shot = (tws.SOURCE_BRUSH, bx, by, size_sq, intensity)
    d, f, v, _, _ = gpu_run(tws, g["b"], g["d0"], g["f0"], p, [], int(g["steps"]), k,
                            one_shot=one_shot)
    assert_bitexact(d, g["d"], "depth")
    assert_bitexact(f, g["f"], "flux")
    assert np.array_equal(v.astype(np.float16).view(np.uint16), g["flowmap_f16"]), "flow map"


# ------------------------------------------------------------ the 256^2 configuration

@pytest.mark.parametrize("k", [1, 2, 3, 4])
def test_baseline_256_config_bitexact(tws, oracle, k):
    """256^2, l=1, A=1, g=9.81, dt=0.02, damping 0.998/step, closed walls,
    rain disk r=16 at +0.01 m/step, 1000 steps."""
    W = H = 256
    p = tws.params_physical(0.02, 9.81, 1.0, 1.0, 0.998, tws.BOUNDARY_CLOSED)
    b, d = oracle.terrain(2026, W, H, 40.0, 15.0)
    rain = tws.rain_disks(2026, W, H, 16, 0.01, 1)
    f = np.zeros((H, W, 4), np.float32)
    gd, gf, gv, gvol, _ = gpu_run(tws, b, d, f, p, rain, 1000, k)
    od, of, ov = oracle_run(oracle, b, d, f, p.as_tuple(), rain, 1000, oracle.BOUNDARY_CLOSED)
    assert_bitexact(gd, od, "depth")
    assert_bitexact(gf, of, "flux")
    assert_bitexact(gv, ov, "velocity")
    ovol = oracle.volume(od)
    assert abs(gvol - ovol) <= 1e-12 * ovol
    # within the stated tolerance of the FP32 transcription by construction
    # (identical bits); also close to the FP64 oracle
    b64, d64 = b.astype(np.float64), d.astype(np.float64)
    f64 = np.zeros((H, W, 4), np.float64)
    kf, ka, c = oracle.params_physical()
    oracle.step_f64(b64, d64, f64, None, kf, ka, c, oracle.BOUNDARY_CLOSED,
                    [(s[0], s[1], s[2], s[3], 0.01) for s in rain], nsteps=1000)
    assert abs(gvol - oracle.volume(d64)) / oracle.volume(d64) < 1e-5


# ------------------------------------------------------------ seams, ragged sizes, borders

SIZES = [(1, 1), (1, 37), (37, 1), (2, 3), (33, 17), (64, 32), (97, 130), (200, 3), (129, 65)]


@pytest.mark.parametrize("boundary", [0, 1])
@pytest.mark.parametrize("k", [1, 2, 3, 4])
@pytest.mark.parametrize("W,H", SIZES)
def test_ragged_sizes_bitexact(tws, oracle, W, H, k, boundary):
    rng = np.random.default_rng(W * 1000 + H)
    b = rng.uniform(0, 6, (H, W)).astype(np.float32)
    d = np.maximum(0, rng.uniform(-2, 5, (H, W))).astype(np.float32)
    f = rng.uniform(0, 0.3, (H, W, 4)).astype(np.float32)
    p = tws.params_physical(0.02, 9.81, 1.0, 1.0, 0.998, boundary)
    srcs = [(tws.SOURCE_DISK, W // 2, H // 2, max(1, min(W, H) // 3), 0.05),
            (tws.SOURCE_BRUSH, W * 0.3, H * 0.7, 20.0, 0.2)]
    gd, gf, gv, _, _ = gpu_run(tws, b, d, f, p, srcs, 9, k)
    od, of, ov = oracle_run(oracle, b, d, f, p.as_tuple(), srcs, 9, boundary)
    assert_bitexact(gd, od, "depth")
    assert_bitexact(gf, of, "flux")
    assert_bitexact(gv, ov, "velocity")


@pytest.mark.parametrize("W,H", [(64, 64), (100, 37), (4096, 64)])
def test_scene_generator_matches_oracle(tws, oracle, W, H):
    with tws.Grid(W, H) as g:
        g.generate_scene(2026, 40.0, 15.0)
        b = g.download_terrain()
        d, f, v = g.download()
    ob, od = oracle.terrain(2026, W, H, 40.0, 15.0)
    assert_bitexact(b, ob, "terrain")
    assert_bitexact(d, od, "depth")
    assert not f.any() and not v.any()


def test_one_shot_brush_matches_oracle(tws, oracle):
    W, H = 96, 80
    b, d = oracle.terrain(3, W, H, 40.0, 15.0)
    brush = (tws.SOURCE_BRUSH, 31.7, 44.2, 32.0, 5.0)
    with tws.Grid(W, H) as g:
        g.upload(b, d)
        g.apply_source(brush)
        g.apply_source((tws.SOURCE_DISK, 90, 2, 7, 0.25))
        gd, _, _ = g.download(flux=False, velocity=False)
    od = d.copy()
    oracle.sources_f32(od, [brush, (oracle.SOURCE_DISK, 90, 2, 7, 0.25)])
    assert_bitexact(gd, od, "depth")


def test_lake_at_rest_gpu(tws):
    rng = np.random.default_rng(11)
    H, W = 200, 300
    b = (rng.integers(0, 40, (H, W)) / 8.0).astype(np.float32)
    d = (np.float32(10.0) - b).astype(np.float32)
    p = tws.params_physical(boundary=tws.BOUNDARY_CLOSED)
    for k in (1, 4):
        gd, gf, gv, _, _ = gpu_run(tws, b, d, np.zeros((H, W, 4), np.float32), p, [], 100, k)
        assert_bitexact(gd, d, "depth")
        assert not gf.any() and not gv.any()


def test_reference_setters_between_steps(tws, oracle):
    """Parameters changed between steps (Terrain.cpp:175-198 setters) take
    effect at the next step, as in the reference."""
    W = H = 128
    b, d = oracle.terrain(8, W, H, 40.0, 15.0)
    p1 = tws.params_reference(60.0, 0.98, 10.0, float(W), W, tws.BOUNDARY_OPEN)
    p2 = tws.params_reference(60.0, 0.96, 30.0, float(W), W, tws.BOUNDARY_OPEN)
    with tws.Grid(W, H, p1) as g:
        g.upload(b, d)
        g.step(30)
        g.set_params(p2)
        g.step(30)
        gd, gf, gv = g.download()
    od, of, ov = oracle_run(oracle, b, d, np.zeros((H, W, 4), np.float32), p1.as_tuple(), [], 30,
                            oracle.BOUNDARY_OPEN)
    od, of, ov = oracle_run(oracle, b, od, of, p2.as_tuple(), [], 30, oracle.BOUNDARY_OPEN)
    assert_bitexact(gd, od, "depth")
    assert_bitexact(gf, of, "flux")


# ------------------------------------------------------------ FP16 flux storage

@pytest.mark.parametrize("k", [1, 2, 4])
def test_f16_storage_matches_oracle_f16_mode(tws, oracle, k):
    W, H = 192, 160
    p = tws.params_physical(boundary=tws.BOUNDARY_CLOSED)
    b, d = oracle.terrain(5, W, H, 40.0, 15.0)
    rain = tws.rain_disks(5, W, H, 12, 0.02, 1)
    f = np.zeros((H, W, 4), np.float32)
    gd, gf, gv, gvol, scale = gpu_run(tws, b, d, f, p, rain, 300, k, flux_storage=tws.FLUX_F16)
    assert scale > 0 and np.log2(scale) == int(np.log2(scale))
    od, of, ov = oracle_run(oracle, b, d, f, p.as_tuple(), rain, 300, oracle.BOUNDARY_CLOSED,
                            flux_scale=scale)
    assert_bitexact(gd, od, "depth")
    assert_bitexact(gf, of, "flux")
    assert_bitexact(gv, ov, "velocity")
    # against the FP64 oracle: volume drift within 1e-4
    b64, d64 = b.astype(np.float64), d.astype(np.float64)
    f64 = np.zeros((H, W, 4), np.float64)
    kf, ka, c = oracle.params_physical()
    oracle.step_f64(b64, d64, f64, None, kf, ka, c, oracle.BOUNDARY_CLOSED,
                    [(s[0], s[1], s[2], s[3], 0.02) for s in rain], nsteps=300)
    v64 = oracle.volume(d64)
    assert abs(gvol - v64) / v64 <= 1e-4


def test_rain_on_deep_water_conserves_volume(tws, oracle):
    """Rain on 40 m of water (a binade where round to nearest would lose 1.7e-4
    of every 0.01 m increment): the DISK source's unbiased rounding keeps the
    FP64 volume within 2e-6 of the exact bookkeeping after 3000 steps, and the
    state equals the oracle's bit for bit."""
    W = H = 256
    b = np.zeros((H, W), np.float32)
    b[:, : W // 2] = 1.0  # a step in the bed, so the water moves
    d = (np.float32(41.0) - b).astype(np.float32)
    f = np.zeros((H, W, 4), np.float32)
    p = tws.params_physical(boundary=tws.BOUNDARY_CLOSED)
    r = 60
    rain = [(tws.SOURCE_DISK, W // 2, H // 2, r, 0.01)]
    steps = 3000
    gd, gf, gv, gvol, _ = gpu_run(tws, b, d, f, p, rain, steps, 2)
    od, of, ov = oracle_run(oracle, b, d, f, p.as_tuple(), rain, steps, oracle.BOUNDARY_CLOSED)
    assert_bitexact(gd, od, "depth")
    assert_bitexact(gf, of, "flux")
    yy, xx = np.mgrid[-r:r + 1, -r:r + 1]
    n = int(np.count_nonzero(xx * xx + yy * yy <= r * r))
    exact = float(np.sum(d, dtype=np.float64)) + steps * float(np.float32(0.01)) * n
    assert abs(gvol - exact) / exact < 2e-6, (gvol, exact)


# ------------------------------------------------------------ full size (4096^2)

def test_full_size_4096_bitexact_and_k_invariant(tws, oracle):
    """4096^2 benchmark scene with rain r=64: every temporal depth gives the
    same bits as the oracle after 12 steps."""
    W = H = 4096
    p = tws.params_physical(boundary=tws.BOUNDARY_CLOSED)
    rain = tws.rain_disks(2026, W, H, 64, 0.01, 1)
    b, d = oracle.terrain(2026, W, H, 40.0, 15.0)
    od, of, ov = oracle_run(oracle, b, d, np.zeros((H, W, 4), np.float32), p.as_tuple(), rain, 12,
                            oracle.BOUNDARY_CLOSED)
    with tws.Grid(W, H, p) as g:
        g.set_sources(rain)
        for k in (1, 2, 3, 4):
            g.generate_scene(2026, 40.0, 15.0)
            g.set_steps_per_launch(k)
            g.step(12)
            g.sync()
            gd, gf, gv = g.download()
            assert_bitexact(gd, od, f"depth k={k}")
            assert_bitexact(gf, of, f"flux k={k}")
            assert_bitexact(gv, ov, f"velocity k={k}")


def test_full_size_volume_conservation_and_positivity(tws):
    """4096^2, closed walls, no rain: total volume (FP64 reduction) stays
    within 1e-6 relative over 2000 steps; depth and flux stay non-negative."""
    W = H = 4096
    with tws.Grid(W, H, tws.params_physical(boundary=tws.BOUNDARY_CLOSED)) as g:
        g.generate_scene(7, 40.0, 15.0)
        v0 = g.volume()
        g.step(2000)
        g.sync()
        v1 = g.volume()
        d, f, _ = g.download(velocity=False)
    assert abs(v1 - v0) <= 1e-6 * v0
    assert d.min() >= 0 and f.min() >= 0


def test_volume_reduction_matches_fp64_sum(tws):
    rng = np.random.default_rng(1)
    for (W, H) in ((1, 1), (33, 5000), (3000, 7)):
        b = np.zeros((H, W), np.float32)
        d = rng.uniform(0, 100, (H, W)).astype(np.float32)
        with tws.Grid(W, H) as g:
            g.upload(b, d)
            v = g.volume()
        want = float(np.sum(d.astype(np.float64)))
        assert abs(v - want) <= 1e-12 * want


def test_error_paths(tws):
    with tws.Grid(16, 16) as g:
        with pytest.raises(tws.TwsError):
            g.step(-1)
        with pytest.raises(tws.TwsError):
            g.set_steps_per_launch(5)
        with pytest.raises(tws.TwsError):
            g.set_sources([(7, 0, 0, 1, 1)])
        with pytest.raises(tws.TwsError):
            g.set_sources([(0, 1, 1, 1, 1)] * 9)
        g.step(3)
        g.sync()  # no device-side error after normal work
        buf = g.buffers()
        assert buf.pitch % 32 == 0 and buf.width == 16 and buf.depth


# ------------------------------------------------------------ variants and autotuner

@pytest.mark.parametrize("W,H", [(97, 130), (300, 41), (1, 70), (260, 200)])
def test_every_kernel_variant_bitexact(tws, oracle, W, H):
    """Every (temporal depth, tile) variant, with a step count that leaves a
    remainder for the shallower kernels, matches the oracle bit for bit.
    260 x 200 gives every tile shape interior tiles, some under the source."""
    rng = np.random.default_rng(W + 7 * H)
    b = rng.uniform(0, 6, (H, W)).astype(np.float32)
    d = np.maximum(0, rng.uniform(-2, 5, (H, W))).astype(np.float32)
    f = rng.uniform(0, 0.3, (H, W, 4)).astype(np.float32)
    p = tws.params_physical(boundary=tws.BOUNDARY_CLOSED)
    srcs = [(tws.SOURCE_DISK, W // 3, H // 2, 5, 0.05)]
    od, of, ov = oracle_run(oracle, b, d, f, p.as_tuple(), srcs, 13, oracle.BOUNDARY_CLOSED)
    for vi in range(len(tws.variants())):
        with tws.Grid(W, H, p) as g:
            g.upload(b, d, f)
            g.set_sources(srcs)
            g.set_variant(vi)
            g.step(13)
            gd, gf, gv = g.download()
        assert_bitexact(gd, od, f"depth variant {vi}")
        assert_bitexact(gf, of, f"flux variant {vi}")
        assert_bitexact(gv, ov, f"velocity variant {vi}")


def test_signed_zeros_bitexact_every_variant(tws, oracle):
    """A patch where terrain, depth and flux are zeros of random sign, in
    a grid with interior tiles: surface differences of -0, flux terms of -0
    and dry cells that must scale to zero.  Every variant keeps the signs the
    shaders give (max(0, v) of -0 is +0; a dry cell's scale is its depth)."""
    W, H = 200, 160
    rng = np.random.default_rng(17)
    b = rng.uniform(0, 3, (H, W)).astype(np.float32)
    d = rng.uniform(0, 2, (H, W)).astype(np.float32)
    f = rng.uniform(0, 0.2, (H, W, 4)).astype(np.float32)

    def signed_zeros(shape):
        return np.where(rng.random(shape) < 0.5, np.float32(-0.0), np.float32(0.0))

    ys, xs = slice(40, 120), slice(50, 150)
    b[ys, xs] = signed_zeros(b[ys, xs].shape)
    d[ys, xs] = signed_zeros(d[ys, xs].shape)
    f[ys, xs] = signed_zeros(f[ys, xs].shape)
    # scattered dry cells with signed-zero depth elsewhere
    dry = rng.random((H, W)) < 0.2
    d[dry] = signed_zeros(int(dry.sum()))
    assert np.signbit(d).any() and np.signbit(f).any()
    p = tws.params_physical(boundary=tws.BOUNDARY_CLOSED)
    for steps in (1, 4):
        od, of, ov = oracle_run(oracle, b, d, f, p.as_tuple(), [], steps, oracle.BOUNDARY_CLOSED)
        for vi in range(len(tws.variants())):
            with tws.Grid(W, H, p) as g:
                g.upload(b, d, f)
                g.set_variant(vi)
                g.step(steps)
                gd, gf, gv = g.download()
            assert_bitexact(gd, od, f"depth variant {vi}, {steps} steps")
            assert_bitexact(gf, of, f"flux variant {vi}, {steps} steps")
            assert_bitexact(gv, ov, f"velocity variant {vi}, {steps} steps")


def test_autotune_preserves_state_and_pins_a_variant(tws, oracle):
    W, H = 512, 384
    p = tws.params_physical(boundary=tws.BOUNDARY_CLOSED)
    rain = tws.rain_disks(3, W, H, 20, 0.01, 1)
    b, d = oracle.terrain(3, W, H, 40.0, 15.0)
    with tws.Grid(W, H, p) as g:
        g.upload(b, d)
        g.set_sources(rain)
        g.step(5)
        best = g.autotune(12)
        assert 0 <= best < len(tws.variants())
        g.step(7)
        gd, gf, gv = g.download()
    od, of, ov = oracle_run(oracle, b, d, np.zeros((H, W, 4), np.float32), p.as_tuple(), rain, 12,
                            oracle.BOUNDARY_CLOSED)
    assert_bitexact(gd, od, "depth")
    assert_bitexact(gf, of, "flux")
    assert_bitexact(gv, ov, "velocity")
