"""GPU parity of the row-sweep kernels (tws_sweep.cu) with the oracle, bit for
bit: every sweep variant on grids with interior and edge strips and bands,
odd widths, grids narrower than one strip, both borders, both source kinds,
FP16 flux storage, and the 4096^2 benchmark scene."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import assert_bitexact

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def tws():
    import terrainwatersim_gb300 as t
    t.lib()
    return t


def sweep_variants(tws):
    return [i for i, v in enumerate(tws.variants()) if v[5] == tws.VARIANT_SWEEP]


def rough_state(W, H, seed):
    rng = np.random.default_rng(seed)
    b = rng.uniform(0, 6, (H, W)).astype(np.float32)
    d = np.maximum(0, rng.uniform(-2, 5, (H, W))).astype(np.float32)
    f = rng.uniform(0, 0.3, (H, W, 4)).astype(np.float32)
    return b, d, f


def oracle_run(O, b, d, f, params, sources, steps, boundary, flux_scale=0.0):
    b, d, f = b.copy(), d.copy(), f.copy()
    H, W = b.shape
    v = np.zeros((H, W, 2), np.float32)
    kf, ka, c = params
    O.step_f32(b, d, f, v, kf, ka, c, boundary, [tuple(s) for s in sources], nsteps=steps,
               flux_scale=flux_scale)
    return d, f, v


def gpu_run(tws, variant, b, d, f, params, sources, steps, flux_storage=0):
    H, W = b.shape
    with tws.Grid(W, H, params, flux_storage) as g:
        g.upload(b, d, f)
        g.set_sources(sources)
        g.set_variant(variant)
        g.step(steps)
        g.sync()
        out = g.download()
        scale = g.buffers().flux_scale
    return out + (scale,)


def test_sweep_variants_exist(tws):
    ks = {tws.variants()[i][0] for i in sweep_variants(tws)}
    assert ks == {2, 3, 4}


@pytest.mark.parametrize("W,H,boundary", [
    (700, 600, "closed"),   # interior strips and bands for every band height
    (333, 517, "open"),     # odd width: a strip ends on the grid's last column
    (45, 300, "closed"),    # narrower than one strip
    (130, 9, "open"),       # shallower than the band's halo
])
def test_every_sweep_variant_bitexact(tws, oracle, W, H, boundary):
    b, d, f = rough_state(W, H, W * 3 + H)
    bnd = tws.BOUNDARY_CLOSED if boundary == "closed" else tws.BOUNDARY_OPEN
    obnd = oracle.BOUNDARY_CLOSED if boundary == "closed" else oracle.BOUNDARY_OPEN
    p = tws.params_physical(boundary=bnd)
    srcs = [(tws.SOURCE_DISK, W // 3, H // 2, 7, 0.05),
            (tws.SOURCE_BRUSH, W * 0.7, H * 0.25, 30.0, 0.8)]
    steps = 13  # a remainder for every temporal depth
    od, of, ov = oracle_run(oracle, b, d, f, p.as_tuple(), srcs, steps, obnd)
    for vi in sweep_variants(tws):
        gd, gf, gv, _ = gpu_run(tws, vi, b, d, f, p, srcs, steps)
        assert_bitexact(gd, od, f"depth variant {vi}")
        assert_bitexact(gf, of, f"flux variant {vi}")
        assert_bitexact(gv, ov, f"flow map variant {vi}")


@pytest.mark.parametrize("W,H", [(400, 300), (257, 129)])
def test_every_sweep_variant_fp16_storage(tws, oracle, W, H):
    b, d = oracle.terrain(9, W, H, 40.0, 15.0)
    rng = np.random.default_rng(W)
    d = (d + np.maximum(0, rng.uniform(-1, 2, (H, W)))).astype(np.float32)
    f = np.zeros((H, W, 4), np.float32)
    p = tws.params_physical(boundary=tws.BOUNDARY_CLOSED)
    rain = tws.rain_disks(9, W, H, 12, 0.02, 1)
    ref = None
    for vi in sweep_variants(tws):
        gd, gf, gv, scale = gpu_run(tws, vi, b, d, f, p, rain, 20, tws.FLUX_F16)
        if ref is None:
            ref = oracle_run(oracle, b, d, f, p.as_tuple(), rain, 20, oracle.BOUNDARY_CLOSED,
                             flux_scale=scale)
        assert_bitexact(gd, ref[0], f"depth variant {vi}")
        assert_bitexact(gf, ref[1], f"flux variant {vi}")
        assert_bitexact(gv, ref[2], f"flow map variant {vi}")


def test_sweep_full_size_4096(tws, oracle):
    """The 4096^2 benchmark scene with its rain disk: 12 steps of every sweep
    depth give the oracle's bits on the full grid."""
    W = H = 4096
    p = tws.params_physical(boundary=tws.BOUNDARY_CLOSED)
    rain = tws.rain_disks(2026, W, H, 64, 0.01, 1)
    b, d = oracle.terrain(2026, W, H, 40.0, 15.0)
    f = np.zeros((H, W, 4), np.float32)
    od, of, ov = oracle_run(oracle, b, d, f, p.as_tuple(), rain, 12, oracle.BOUNDARY_CLOSED)
    picks = {}
    for vi in sweep_variants(tws):
        picks.setdefault(tws.variants()[vi][0], vi)  # the first variant of each depth
    for k, vi in sorted(picks.items()):
        with tws.Grid(W, H, p) as g:
            g.generate_scene(2026, 40.0, 15.0)
            g.set_sources(rain)
            g.set_variant(vi)
            g.step(12)
            gd, gf, gv = g.download()
        assert_bitexact(gd, od, f"depth K={k}")
        assert_bitexact(gf, of, f"flux K={k}")
        assert_bitexact(gv, ov, f"flow map K={k}")


def test_large_fp32_grid_default_is_bitexact(tws, oracle):
    """A grid of at least 12 Mi cells with FP32 flux and nothing pinned runs the
    three-step sweep by default; 5 steps (one sweep launch and a two-step
    remainder) give the oracle's bits."""
    W, H = 3584, 3600
    p = tws.params_physical(boundary=tws.BOUNDARY_CLOSED)
    rain = tws.rain_disks(44, W, H, 40, 0.02, 2)
    b, d = oracle.terrain(44, W, H, 40.0, 15.0)
    f = np.zeros((H, W, 4), np.float32)
    od, of, ov = oracle_run(oracle, b, d, f, p.as_tuple(), rain, 5, oracle.BOUNDARY_CLOSED)
    with tws.Grid(W, H, p) as g:
        g.generate_scene(44, 40.0, 15.0)
        g.set_sources(rain)
        n0 = tws.lib().tws_launch_count()
        g.step(5)
        g.sync()
        launches = tws.lib().tws_launch_count() - n0
        gd, gf, gv = g.download()
    assert launches == 2  # a three-step and a two-step launch
    assert_bitexact(gd, od, "depth")
    assert_bitexact(gf, of, "flux")
    assert_bitexact(gv, ov, "flow map")


def test_tail_bands_bitexact(tws, oracle):
    """Sweep variants whose queue ends in short bands, on a grid with several
    full tall bands, a partial one and the tail: sources straddle the band
    edges; every result is the oracle's."""
    W, H = 1000, 2100
    b, d, f = rough_state(W, H, 77)
    p = tws.params_physical(boundary=tws.BOUNDARY_CLOSED)
    srcs = [(tws.SOURCE_DISK, 500, 384, 30, 0.05), (tws.SOURCE_DISK, 130, 1090, 40, 0.03),
            (tws.SOURCE_BRUSH, 800.0, 1700.0, 900.0, 0.5)]
    steps = 7
    od, of, ov = oracle_run(oracle, b, d, f, p.as_tuple(), srcs, steps, oracle.BOUNDARY_CLOSED)
    tails = [vi for vi in sweep_variants(tws) if tws.variant_tail_rows(vi) > 0]
    assert tails
    for vi in tails:
        gd, gf, gv, _ = gpu_run(tws, vi, b, d, f, p, srcs, steps)
        assert_bitexact(gd, od, f"depth variant {vi}")
        assert_bitexact(gf, of, f"flux variant {vi}")
        assert_bitexact(gv, ov, f"flow map variant {vi}")


@pytest.mark.parametrize("N,flux,k,rows,tail", [
    (4096, 0, 3, 40, 0),      # FP32: three-step sweep, uniform 40-row bands
    (8192, 0, 3, 192, 48),    # larger grids: tall bands ending in short ones
    (4096, 1, 2, None, None), # FP16 below 32 Mi cells: the two-step tiles
    (8192, 1, 3, 192, 48),    # FP16 from 32 Mi cells: the sweep as for FP32
])
def test_default_variant_ladder(tws, N, flux, k, rows, tail):
    """The automatic choice per size and flux storage (the band heights are
    the measured rungs for a 152-SM GB300)."""
    import torch
    p = tws.params_physical(boundary=tws.BOUNDARY_CLOSED)
    with tws.Grid(N, N, p, flux) as g:
        vi = g.current_variant()
    v = tws.variants()[vi]
    assert v[0] == k
    if rows is None:
        assert v[5] == tws.VARIANT_TILE
        return
    assert v[5] == tws.VARIANT_SWEEP
    if torch.cuda.get_device_properties(0).multi_processor_count == 152:
        assert (v[2], tws.variant_tail_rows(vi)) == (rows, tail)
