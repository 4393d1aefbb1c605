"""Failure detection on the GPU without a fault: every tile load arms its
barrier but issues no copy (tws_test_drop_tile_loads, include/tws_testing.h),
so each kernel's bounded barrier wait runs out with nothing in flight.  The kernel records the time-out in the grid's error word and returns;
tws_sync reports TWS_ERR_TIMEOUT once, and the same grid and context then
run a normal step that matches the oracle bit for bit."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import assert_bitexact

pytestmark = pytest.mark.gpu

WAIT_LIMIT = 2_000_000  # SM clocks, about a millisecond


@pytest.fixture(scope="module")
def tws():
    import terrainwatersim_gb300 as t
    t.lib()
    return t


def _state(oracle, W, H):
    b, d = oracle.terrain(11, W, H, 40.0, 15.0)
    f = np.zeros((H, W, 4), np.float32)
    return b, d, f


def _tile_variants(tws):
    """Tile variants (those that stage tiles in shared memory): the first
    K=1 and K=2 one-CTA-per-tile variants, the first persistent one and the
    last one in the table."""
    tiled = [(i, v) for i, v in enumerate(tws.variants()) if v[5] == tws.VARIANT_TILE]
    picks = [next(i for i, v in tiled if v[0] == 1 and v[3] == 1),
             next(i for i, v in tiled if v[0] == 2 and v[3] == 1),
             next(i for i, v in tiled if v[3] == 2),
             tiled[-1][0]]
    return list(dict.fromkeys(picks))


@pytest.mark.parametrize("pick", range(4))
def test_lost_tile_load_times_out_and_grid_recovers(tws, oracle, pick):
    variants = _tile_variants(tws)
    if pick >= len(variants):
        pytest.skip("fewer tile variants")
    variant = variants[pick]
    W, H = 96, 64
    b, d, f = _state(oracle, W, H)
    p = tws.params_physical(0.02, 9.81, 1.0, 1.0, 0.998, tws.BOUNDARY_CLOSED)
    with tws.Grid(W, H, p) as g:
        g.set_variant(variant)
        g.upload(b, d, f)
        g.set_wait_limit(WAIT_LIMIT)
        g.test_drop_tile_loads(True)
        g.step(2)
        with pytest.raises(tws.TwsError) as e:
            g.sync()
        assert e.value.code == tws.ERR_TIMEOUT
        # reported once: the word is clear again
        g.sync()
        # the context and grid stay usable: reload and run normally
        g.test_drop_tile_loads(False)
        g.set_wait_limit(0)
        g.upload(b, d, f)
        g.step(6)
        g.sync()
        gd, gf, gv = g.download()
    od, of = d.copy(), f.copy()
    ov = np.zeros((H, W, 2), np.float32)
    kf, ka, c = p.as_tuple()
    oracle.step_f32(b.copy(), od, of, ov, kf, ka, c, oracle.BOUNDARY_CLOSED, [], nsteps=6)
    assert_bitexact(gd, od, "depth")
    assert_bitexact(gf, of, "flux")
    assert_bitexact(gv, ov, "velocity")


def test_batched_lost_tile_load_times_out_and_recovers(tws, oracle):
    W, H = 80, 48
    b, d, f = _state(oracle, W, H)
    p = tws.params_physical(0.02, 9.81, 1.0, 1.0, 0.998, tws.BOUNDARY_CLOSED)
    with tws.Batch() as batch, tws.Grid(W, H, p) as g:
        g.upload(b, d, f)
        g.set_wait_limit(WAIT_LIMIT)
        g.test_drop_tile_loads(True)
        batch.add(g)
        batch.step(4)
        with pytest.raises(tws.TwsError) as e:
            batch.sync()
        assert e.value.code == tws.ERR_TIMEOUT
        batch.sync()
        batch.remove(g)
        g.test_drop_tile_loads(False)
        g.set_wait_limit(0)
        g.upload(b, d, f)
        batch.add(g)
        batch.step(4)
        batch.sync()
        batch.remove(g)
        gd, gf, _ = g.download()
    od, of = d.copy(), f.copy()
    kf, ka, c = p.as_tuple()
    oracle.step_f32(b.copy(), od, of, None, kf, ka, c, oracle.BOUNDARY_CLOSED, [], nsteps=4)
    assert_bitexact(gd, od, "depth")
    assert_bitexact(gf, of, "flux")


def test_hook_arguments_checked(tws):
    with tws.Grid(16, 16) as g:
        for bad in (-1, 2, 16):
            assert tws.lib().tws_test_drop_tile_loads(g._h, bad) == tws.ERR_INVALID
        with pytest.raises(tws.TwsError):
            g.set_wait_limit(-1)
