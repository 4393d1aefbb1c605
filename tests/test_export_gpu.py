"""GPU tests of what the renderer reads: the water shaders' per-texel
arithmetic (surface height, dry mask, tessellated height, heightmap normal,
flow speed, foam) and the reference's texture layouts (RGBA32F TerrainData
with its mip pyramid, RG16F FlowMap), bit for bit against the oracle."""
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


@pytest.mark.parametrize("W,H", [(96, 80), (260, 130), (33, 257), (1, 5)])
def test_surface_outputs_match_oracle(tws, oracle, W, H):
    import torch
    p = tws.params_physical(boundary=tws.BOUNDARY_OPEN)
    with tws.Grid(W, H, p) as g:
        g.generate_scene(12, 40.0, 15.0)
        g.apply_source((tws.SOURCE_BRUSH, W * 0.4, H * 0.3, 40.0, 6.0))
        g.step(25)
        d, _, v = g.download(flux=False)
        b = g.download_terrain()
        bufs = {k: torch.zeros((H, W), dtype=torch.float32, device="cuda")
                for k in ("height", "render_height", "flow_speed", "foam")}
        bufs["normal"] = torch.zeros((H, W, 3), dtype=torch.float32, device="cuda")
        bufs["dry"] = torch.zeros((H, W), dtype=torch.uint8, device="cuda")
        torch.cuda.synchronize()
        out = tws.SurfaceOut(*[bufs[k].data_ptr() for k in
                               ("height", "render_height", "normal", "flow_speed", "foam", "dry")])
        g.surface(out)
        g.sync()
        got = {k: t.cpu().numpy() for k, t in bufs.items()}
    want = oracle.surface(b, d, v)
    for k in ("height", "render_height", "normal", "flow_speed", "foam"):
        assert_bitexact(got[k], want[k], k)
    assert np.array_equal(got["dry"], want["dry"])
    if W > 1:  # (a 1-wide open grid has drained by now)
        assert got["dry"].any() and (got["flow_speed"] > 0).any()


def test_surface_matches_reference_render_fixture(tws):
    """tws_surface against the reference's own water-rendering shader code
    (tests/golden/ref_render_64.npz, made by running waterRender.vert, the
    main() of waterRender.eval and waterRender.frag's ComputeHeightmapNormal
    and flow-speed lines on the CPU): the same state on the GPU, then every
    output bit for bit."""
    import torch
    g0 = load_golden("ref_render_64")
    N = int(g0["case_N"])
    bx, by, size_sq, intensity = g0["case_brush"].tolist()
    p = tws.params_physical(boundary=tws.BOUNDARY_OPEN)
    with tws.Grid(N, N, p) as g:
        g.generate_scene(int(g0["case_seed"]), 40.0, float(g0["case_fill"]))
        g.apply_source((tws.SOURCE_BRUSH, bx, by, size_sq, intensity))
        g.step(int(g0["case_steps"]))
        d, _, v = g.download(flux=False)
        assert_bitexact(d, g0["d"], "depth")
        assert_bitexact(v, g0["v"], "flow map")
        bufs = {k: torch.zeros((N, N), dtype=torch.float32, device="cuda")
                for k in ("height", "render_height", "flow_speed", "foam")}
        bufs["normal"] = torch.zeros((N, N, 3), dtype=torch.float32, device="cuda")
        bufs["dry"] = torch.zeros((N, N), dtype=torch.uint8, device="cuda")
        torch.cuda.synchronize()
        out = tws.SurfaceOut(*[bufs[k].data_ptr() for k in
                               ("height", "render_height", "normal", "flow_speed", "foam", "dry")])
        g.surface(out)
        g.sync()
        got = {k: t.cpu().numpy() for k, t in bufs.items()}
    for k in ("height", "render_height", "normal", "flow_speed", "foam"):
        assert_bitexact(got[k], g0["out_" + k], k)
    assert np.array_equal(got["dry"], g0["out_dry"])


@pytest.mark.parametrize("W,H,levels", [(64, 48, 3), (100, 37, 2), (38, 21, 2), (256, 256, 8),
                                          (200, 136, 7), (640, 382, 8)])
def test_texture_export_matches_oracle(tws, oracle, W, H, levels):
    import torch
    with tws.Grid(W, H) as g:
        g.generate_scene(4, 40.0, 15.0)
        g.set_sources(tws.rain_disks(4, W, H, 5, 0.05, 1))
        g.step(9)
        d, _, v = g.download(flux=False)
        b = g.download_terrain()
        rgba = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
        fm = torch.zeros((H, W, 2), dtype=torch.int16, device="cuda")
        n = 0
        w, h = W, H
        for _ in range(levels):
            w, h = w // 2, h // 2
            n += 4 * w * h
        mips = torch.zeros(max(1, n), dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        g.export_textures(rgba.data_ptr(), fm.data_ptr(), levels, mips.data_ptr())
        g.sync()
        got_rgba, got_fm, got_mips = rgba.cpu().numpy(), fm.cpu().numpy(), mips.cpu().numpy()
        with pytest.raises(tws.TwsError):
            g.export_textures(rgba.data_ptr(), None, 20, mips.data_ptr())  # past 1x1
    want_rgba, want_mips = oracle.terrain_mips(b, d, levels)
    assert_bitexact(got_rgba, want_rgba, "TerrainData")
    assert np.array_equal(got_fm.view(np.uint16), v.astype(np.float16).view(np.uint16))
    off = 0
    for lvl, m in enumerate(want_mips, 1):
        assert_bitexact(got_mips[off:off + m.size].reshape(m.shape), m, f"mip {lvl}")
        off += m.size


def test_unaligned_outputs(tws, oracle):
    """Surface outputs 4 bytes past a 16-byte boundary are written one cell at
    a time (the four-cell kernels need aligned rows), with the same values; so
    is a 4-byte aligned flow map.  RGBA32F buffers that are not 16-byte
    aligned are refused before any launch."""
    import torch
    W, H = 96, 40
    with tws.Grid(W, H) as g:
        g.generate_scene(5, 40.0, 15.0)
        g.set_sources(tws.rain_disks(5, W, H, 6, 0.05, 1))
        g.step(11)
        d, _, v = g.download(flux=False)
        b = g.download_terrain()
        raw = torch.zeros(W * H + 4, dtype=torch.float32, device="cuda")
        height = raw[1:1 + W * H]  # 4 bytes past an aligned start
        fm_raw = torch.zeros(2 * W * H + 2, dtype=torch.int16, device="cuda")
        flowmap = fm_raw[2:2 + 2 * W * H]  # 4 bytes past an aligned start
        rgba_raw = torch.zeros(W * H * 4 + 4, dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        g.surface(tws.SurfaceOut(height.data_ptr(), None, None, None, None, None))
        g.export_textures(None, flowmap.data_ptr(), 0, None)
        with pytest.raises(tws.TwsError) as e:
            g.export_textures(rgba_raw.data_ptr() + 4, None, 0, None)
        assert e.value.code == tws.ERR_INVALID
        with pytest.raises(tws.TwsError) as e:
            g.surface(tws.SurfaceOut(raw.data_ptr() + 2, None, None, None, None, None))
        assert e.value.code == tws.ERR_INVALID
        g.sync()
        got_h = height.cpu().numpy().reshape(H, W)
        got_fm = flowmap.cpu().numpy().reshape(H, W, 2)
    want = oracle.surface(b, d, v)
    assert_bitexact(got_h, want["height"], "height")
    assert np.array_equal(got_fm.view(np.uint16), v.astype(np.float16).view(np.uint16))
