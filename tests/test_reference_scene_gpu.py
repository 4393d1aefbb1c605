"""The reference's own noise scene (Terrain::CreateHeightmapFromNoiseAndResetSim)
generated on the GPU: bit for bit the oracle's restatement, which is itself
pinned to the reference's Random.cpp and NoiseGenerator.cpp (test_oracle.py and
the fixture tests/golden/ref_noise_scene_96.npz)."""
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


def test_reference_scene_matches_fixture(tws):
    g0 = load_golden("ref_noise_scene_96")
    N = 96
    with tws.Grid(N, N) as g:
        for gen in (0, 1):
            g.generate_reference_scene(int(g0["seed"]), gen, float(g0["height_scale"]))
            b = g.download_terrain()
            d, f, v = g.download()
            assert_bitexact(b, g0[f"b{gen}"], f"terrain, scene {gen}")
            assert_bitexact(d, g0[f"d{gen}"], f"depth, scene {gen}")
            assert not f.any() and not v.any()


@pytest.mark.parametrize("W,H,gen,hs", [(1024, 1024, 0, 300.0), (300, 200, 2, 40.0),
                                        (2, 2, 0, 300.0), (4097, 33, 1, 120.0)])
@pytest.mark.parametrize("flux_storage", [0, 1])
def test_reference_scene_matches_oracle(tws, oracle, W, H, gen, hs, flux_storage):
    with tws.Grid(W, H, tws.params_physical(), flux_storage) as g:
        g.generate_reference_scene(tws.REFERENCE_NOISE_SEED, gen, hs)
        b = g.download_terrain()
        d, f, _ = g.download(velocity=False)
    ob, od = oracle.reference_terrain(W, H, hs, generation=gen)
    assert_bitexact(b, ob, "terrain")
    assert_bitexact(d, od, "depth")
    assert not f.any()


def test_reference_scene_rejects_bad_input(tws):
    with tws.Grid(1, 8) as g:
        with pytest.raises(tws.TwsError):
            g.generate_reference_scene()
    with tws.Grid(8, 8) as g:
        with pytest.raises(tws.TwsError):
            g.generate_reference_scene(generation=-1)
