"""GPU tests of the asynchronous host I/O (tws_upload_async,
tws_download_async, tws_io_wait): every result is bit-exact with the oracle
run on the same input, including when several uploads, step chains and
downloads are queued back to back so that the copy streams, the staging
buffers and the grid's stream overlap."""
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


def pinned(shape):
    """A page-locked float32 host array (so that the copies are asynchronous)."""
    import torch
    return torch.empty(shape, dtype=torch.float32, pin_memory=True).numpy()


def oracle_state(O, b, d, f, params, sources, steps, flux_scale=0.0):
    b, d, f = b.copy(), d.copy(), f.copy()
    H, W = b.shape
    v = np.zeros((H, W, 2), np.float32)
    kf, ka, c = params
    O.step_f32(b, d, f, v, kf, ka, c, O.BOUNDARY_CLOSED,
               [(s[0], s[1], s[2], s[3], s[4]) for s in sources], nsteps=steps,
               flux_scale=flux_scale)
    return d, f, v


def scene(O, tws, seed, W, H, flux=False):
    b, d = O.terrain(seed, W, H, 40.0, 15.0)
    rng = np.random.default_rng(seed)
    f = (rng.random((H, W, 4), dtype=np.float32) * 0.5 if flux
         else np.zeros((H, W, 4), np.float32))
    return b, d, f


@pytest.mark.parametrize("flux_storage", [0, 1])
def test_async_round_trip_matches_oracle(tws, oracle, flux_storage):
    W, H = 200, 160
    p = tws.params_physical(0.02, 9.81, 1.0, 1.0, 0.998, tws.BOUNDARY_CLOSED)
    rain = tws.rain_disks(7, W, H, 12, 0.01, 2)
    b, d, f = scene(oracle, tws, 7, W, H)
    out = (pinned((H, W)), pinned((H, W, 4)), pinned((H, W, 2)))
    hb, hd, hf = pinned((H, W)), pinned((H, W)), pinned((H, W, 4))
    hb[...], hd[...], hf[...] = b, d, f
    with tws.Grid(W, H, p, flux_storage) as g:
        g.set_sources(rain)
        g.upload_async(hb, hd, hf)
        g.step(37)
        g.download_async(out)
        g.io_wait()
        scale = g.buffers().flux_scale if flux_storage else 0.0
    od, of, ov = oracle_state(oracle, b, d, f, p.as_tuple(), rain, 37, flux_scale=scale)
    assert_bitexact(out[0], od, "depth")
    assert_bitexact(out[1], of, "flux")
    assert_bitexact(out[2], ov, "velocity")


@pytest.mark.parametrize("flux_storage", [0, 1])
def test_async_pipeline_each_result_matches_its_input(tws, oracle, flux_storage):
    """Four different inputs queued without a host wait: upload i+1 runs
    while the steps of i do, download i while the steps of i+1 do.  Each
    output must be the oracle's state for its own input.  (FP16 storage
    starts from zero flux, which its storage holds exactly.)"""
    W, H = 257, 130
    steps = 20
    p = tws.params_physical(0.02, 9.81, 1.0, 1.0, 0.998, tws.BOUNDARY_CLOSED)
    rain = tws.rain_disks(11, W, H, 9, 0.02, 1)
    inputs, outs = [], []
    for i in range(4):
        b, d, f = scene(oracle, tws, 100 + i, W, H, flux=flux_storage == 0)
        hb, hd, hf = pinned((H, W)), pinned((H, W)), pinned((H, W, 4))
        hb[...], hd[...], hf[...] = b, d, f
        inputs.append((hb, hd, hf))
        outs.append((pinned((H, W)), pinned((H, W, 4)), pinned((H, W, 2))))
    with tws.Grid(W, H, p, flux_storage) as g:
        g.set_sources(rain)
        g.set_steps_per_launch(2)
        for i in range(4):
            g.upload_async(*inputs[i])
            g.step(steps)
            g.download_async(outs[i])
        g.io_wait()
        scale = g.buffers().flux_scale if flux_storage else 0.0
    for i in range(4):
        od, of, ov = oracle_state(oracle, *[a.copy() for a in inputs[i]], p.as_tuple(), rain,
                                  steps, flux_scale=scale)
        assert_bitexact(outs[i][0], od, f"depth {i}")
        assert_bitexact(outs[i][1], of, f"flux {i}")
        assert_bitexact(outs[i][2], ov, f"velocity {i}")


def test_async_optional_arrays_and_sync(tws, oracle):
    """NULL depth and flux upload as zeros (as tws_upload does); a download
    may ask for any subset; tws_sync also waits for the copies; pageable
    arrays work too."""
    W, H = 96, 72
    p = tws.params_physical(0.02, 9.81, 1.0, 1.0, 0.998, tws.BOUNDARY_OPEN)
    b, _, _ = scene(oracle, tws, 3, W, H)
    rain = tws.rain_disks(3, W, H, 20, 0.05, 1)
    dep = np.empty((H, W), np.float32)  # pageable
    vel = pinned((H, W, 2))
    with tws.Grid(W, H, p) as g:
        g.set_sources(rain)
        g.upload_async(b)
        g.step(9)
        g.download_async((dep, None, vel))
        g.sync()
        sd, sf, sv = g.download()
    kf, ka, c = p.as_tuple()
    zd, zf = np.zeros((H, W), np.float32), np.zeros((H, W, 4), np.float32)
    od, of, ov = zd.copy(), zf.copy(), np.zeros((H, W, 2), np.float32)
    oracle.step_f32(b.copy(), od, of, ov, kf, ka, c, oracle.BOUNDARY_OPEN,
                    [(s[0], s[1], s[2], s[3], s[4]) for s in rain], nsteps=9)
    assert_bitexact(dep, od, "depth")
    assert_bitexact(vel, ov, "velocity")
    assert_bitexact(sd, od, "depth (synchronous download)")
    assert_bitexact(sf, of, "flux (synchronous download)")


def test_async_then_sync_calls_keep_order(tws, oracle):
    """A synchronous upload after an asynchronous one wins; an asynchronous
    download after synchronous steps sees them."""
    W, H = 64, 64
    p = tws.params_physical(0.02, 9.81, 1.0, 1.0, 0.998, tws.BOUNDARY_CLOSED)
    b1, d1, f1 = scene(oracle, tws, 21, W, H)
    b2, d2, f2 = scene(oracle, tws, 22, W, H)
    out = (pinned((H, W)), pinned((H, W, 4)), pinned((H, W, 2)))
    with tws.Grid(W, H, p) as g:
        g.upload_async(b1, d1, f1)
        g.step(3)
        g.upload(b2, d2, f2)
        g.step(5)
        g.download_async(out)
        g.io_wait()
    od, of, ov = oracle_state(oracle, b2, d2, f2, p.as_tuple(), [], 5)
    assert_bitexact(out[0], od, "depth")
    assert_bitexact(out[1], of, "flux")
    assert_bitexact(out[2], ov, "velocity")


def test_async_rejects_bad_arguments(tws):
    with tws.Grid(32, 32) as g:
        with pytest.raises(ValueError):
            g.download_async((np.empty((32, 32), np.float64), None, None))
        with pytest.raises(ValueError):
            g.download_async((np.empty((32, 31), np.float32), None, None))
        assert tws.lib().tws_upload_async(g.handle, None, None, None) == tws.ERR_INVALID
    assert tws.lib().tws_io_wait(None) == tws.ERR_INVALID


def test_async_io_on_batch_members(tws, oracle):
    """Grids of a batch take asynchronous uploads and downloads on the
    batch's stream order: each result is its own grid's oracle state."""
    sizes = [(96, 64), (130, 70), (64, 160)]
    p = tws.params_physical(0.02, 9.81, 1.0, 1.0, 0.998, tws.BOUNDARY_CLOSED)
    grids, inputs, outs = [], [], []
    with tws.Batch() as batch:
        for k, (W, H) in enumerate(sizes):
            b, d, f = scene(oracle, tws, 40 + k, W, H)
            g = tws.Grid(W, H, p)
            g.set_sources(tws.rain_disks(40 + k, W, H, 6, 0.01, 1))
            batch.add(g)
            g.upload_async(b, d, f)
            grids.append(g)
            inputs.append((b, d, f))
            outs.append((pinned((H, W)), pinned((H, W, 4)), pinned((H, W, 2))))
        batch.step(24)
        for g, o in zip(grids, outs):
            g.download_async(o)
        for g in grids:
            g.io_wait()
        batch.sync()
        for g in grids:
            batch.remove(g)
    for k, (W, H) in enumerate(sizes):
        rain = tws.rain_disks(40 + k, W, H, 6, 0.01, 1)
        od, of, ov = oracle_state(oracle, *inputs[k], p.as_tuple(), rain, 24)
        assert_bitexact(outs[k][0], od, f"depth grid {k}")
        assert_bitexact(outs[k][1], of, f"flux grid {k}")
        assert_bitexact(outs[k][2], ov, f"velocity grid {k}")
    for g in grids:
        g.close()


def test_timeout_during_pipelined_io_is_reported_and_recovers(tws, oracle):
    """A tile load that never completes (the test hook) inside a pipelined
    upload / steps / download sequence: the copies still finish, tws_sync
    reports the time-out once, and the next pipelined round trip is exact."""
    W, H = 96, 64
    p = tws.params_physical(0.02, 9.81, 1.0, 1.0, 0.998, tws.BOUNDARY_CLOSED)
    b, d, f = scene(oracle, tws, 61, W, H)
    out = (pinned((H, W)), pinned((H, W, 4)), pinned((H, W, 2)))
    with tws.Grid(W, H, p) as g:
        g.set_steps_per_launch(2)
        g.set_wait_limit(2_000_000)
        g.test_drop_tile_loads(True)
        g.upload_async(b, d, f)
        g.step(4)
        g.download_async(out)
        g.io_wait()
        with pytest.raises(tws.TwsError) as e:
            g.sync()
        assert e.value.code == tws.ERR_TIMEOUT
        g.sync()  # reported once
        g.test_drop_tile_loads(False)
        g.upload_async(b, d, f)
        g.step(6)
        g.download_async(out)
        g.sync()
    od, of, ov = oracle_state(oracle, b, d, f, p.as_tuple(), [], 6)
    assert_bitexact(out[0], od, "depth")
    assert_bitexact(out[1], of, "flux")
    assert_bitexact(out[2], ov, "velocity")
