"""GPU parity tests of the resident kernel (the whole grid in the shared
memory of one thread-block cluster, many steps per launch, edge rows
exchanged through distributed shared memory): bit-exact with the oracle for
both boundaries, both sources, FP16 flux storage, uneven row splits over the
cluster's CTAs, and step counts beyond one launch."""
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


def oracle_run(O, b, d, f, params, sources, steps, boundary, flux_scale=0.0):
    b, d, f = b.copy(), d.copy(), f.copy()
    H, W = b.shape
    v = np.zeros((H, W, 2), np.float32)
    kf, ka, c = params
    O.step_f32(b, d, f, v, kf, ka, c, boundary, [(s[0], s[1], s[2], s[3], s[4]) for s in sources],
               nsteps=steps, flux_scale=flux_scale)
    return d, f, v


def random_state(W, H, seed):
    rng = np.random.default_rng(seed)
    b = rng.uniform(0, 6, (H, W)).astype(np.float32)
    d = np.maximum(0, rng.uniform(-2, 5, (H, W))).astype(np.float32)
    f = rng.uniform(0, 0.3, (H, W, 4)).astype(np.float32)
    return b, d, f


def resident_run(tws, b, d, f, p, sources, steps, flux_storage=0, calls=1):
    H, W = b.shape
    with tws.Grid(W, H, p, flux_storage) as g:
        g.upload(b, d, f)
        g.set_sources(sources)
        g.set_resident(True)
        for _ in range(calls):
            g.step(steps // calls)
        g.sync()
        out = g.download()
        scale = g.buffers().flux_scale
    return out + (scale,)


def test_c1_configuration_bitexact(tws, oracle):
    """256^2, closed walls, rain disk r=16 at +0.01 m/step, 1000 steps."""
    W = H = 256
    assert tws.resident_fits(W, H)
    p = tws.params_physical(0.02, 9.81, 1.0, 1.0, 0.998, tws.BOUNDARY_CLOSED)
    b, d = oracle.terrain(2026, W, H, 40.0, 15.0)
    f = np.zeros((H, W, 4), np.float32)
    rain = tws.rain_disks(2026, W, H, 16, 0.01, 1)
    gd, gf, gv, _ = resident_run(tws, b, d, f, p, rain, 1000)
    od, of, ov = oracle_run(oracle, b, d, f, p.as_tuple(), rain, 1000, oracle.BOUNDARY_CLOSED)
    assert_bitexact(gd, od, "depth")
    assert_bitexact(gf, of, "flux")
    assert_bitexact(gv, ov, "velocity")


@pytest.mark.parametrize("W,H", [(97, 130), (300, 41), (600, 40), (33, 17), (1, 70), (70, 1),
                                 (5, 3)])
@pytest.mark.parametrize("boundary", [0, 1])
def test_shapes_and_boundaries_bitexact(tws, oracle, W, H, boundary):
    """Row splits that leave the last CTAs with fewer or no rows, single rows
    and columns, both boundaries, a disk and a brush source."""
    b, d, f = random_state(W, H, W * 31 + H)
    p = tws.params_physical(boundary=boundary)
    srcs = [(tws.SOURCE_DISK, W // 3, H // 2, 5, 0.05),
            (tws.SOURCE_BRUSH, W * 0.6, H * 0.4, 32.0, 0.02)]
    gd, gf, gv, _ = resident_run(tws, b, d, f, p, srcs, 13)
    ob = oracle.BOUNDARY_CLOSED if boundary == 0 else oracle.BOUNDARY_OPEN
    od, of, ov = oracle_run(oracle, b, d, f, p.as_tuple(), srcs, 13, ob)
    assert_bitexact(gd, od, "depth")
    assert_bitexact(gf, of, "flux")
    assert_bitexact(gv, ov, "velocity")


@pytest.mark.parametrize("ctas", [1, 2, 4, 8, 16])
@pytest.mark.parametrize("W,H", [(60, 50), (33, 17)])
def test_every_cluster_size_bitexact(tws, oracle, W, H, ctas):
    """Each cluster size, including splits where CTAs get one row or none."""
    b, d, f = random_state(W, H, 7 * W + H + ctas)
    p = tws.params_physical(boundary=tws.BOUNDARY_CLOSED)
    srcs = [(tws.SOURCE_DISK, W // 2, H // 3, 4, 0.05)]
    with tws.Grid(W, H, p) as g:
        g.upload(b, d, f)
        g.set_sources(srcs)
        g.set_resident(True, ctas)
        g.step(9)
        gd, gf, gv = g.download()
    od, of, ov = oracle_run(oracle, b, d, f, p.as_tuple(), srcs, 9, oracle.BOUNDARY_CLOSED)
    assert_bitexact(gd, od, f"depth ({ctas} CTAs)")
    assert_bitexact(gf, of, f"flux ({ctas} CTAs)")
    assert_bitexact(gv, ov, f"velocity ({ctas} CTAs)")


def test_fp16_flux_storage_bitexact(tws, oracle):
    W, H = 128, 96
    p = tws.params_physical(0.02, 9.81, 1.0, 1.0, 0.998, tws.BOUNDARY_CLOSED)
    b, d = oracle.terrain(5, W, H, 40.0, 15.0)
    f = np.zeros((H, W, 4), np.float32)
    rain = tws.rain_disks(5, W, H, 10, 0.01, 2)
    gd, gf, gv, scale = resident_run(tws, b, d, f, p, rain, 200, flux_storage=tws.FLUX_F16)
    od, of, ov = oracle_run(oracle, b, d, f, p.as_tuple(), rain, 200, oracle.BOUNDARY_CLOSED,
                            flux_scale=scale)
    assert_bitexact(gd, od, "depth")
    assert_bitexact(gf, of, "flux")
    assert_bitexact(gv, ov, "velocity")


def test_steps_beyond_one_launch_and_split_calls(tws, oracle):
    """5000 steps: one call (two launches, 4096 + 904) and five calls of 1000
    give the oracle's state."""
    W, H = 64, 48
    p = tws.params_physical(0.02, 9.81, 1.0, 1.0, 0.998, tws.BOUNDARY_CLOSED)
    b, d = oracle.terrain(9, W, H, 40.0, 15.0)
    f = np.zeros((H, W, 4), np.float32)
    rain = tws.rain_disks(9, W, H, 6, 0.01, 1)
    od, of, ov = oracle_run(oracle, b, d, f, p.as_tuple(), rain, 5000, oracle.BOUNDARY_CLOSED)
    for calls in (1, 5):
        gd, gf, gv, _ = resident_run(tws, b, d, f, p, rain, 5000, calls=calls)
        assert_bitexact(gd, od, f"depth ({calls} calls)")
        assert_bitexact(gf, of, f"flux ({calls} calls)")
        assert_bitexact(gv, ov, f"velocity ({calls} calls)")


def test_signed_zeros_bitexact(tws, oracle):
    W, H = 120, 90
    rng = np.random.default_rng(4)
    b, d, f = random_state(W, H, 4)

    def signed_zeros(shape):
        return np.where(rng.random(shape) < 0.5, np.float32(-0.0), np.float32(0.0))

    b[20:60, 30:90] = signed_zeros((40, 60))
    d[20:60, 30:90] = signed_zeros((40, 60))
    f[20:60, 30:90] = signed_zeros((40, 60, 4))
    p = tws.params_physical(boundary=tws.BOUNDARY_CLOSED)
    gd, gf, gv, _ = resident_run(tws, b, d, f, p, [], 4)
    od, of, ov = oracle_run(oracle, b, d, f, p.as_tuple(), [], 4, oracle.BOUNDARY_CLOSED)
    assert_bitexact(gd, od, "depth")
    assert_bitexact(gf, of, "flux")
    assert_bitexact(gv, ov, "velocity")


def test_dispatch_one_launch_per_call_and_pinning_turns_it_off(tws):
    W, H = 64, 64
    with tws.Grid(W, H) as g:
        g.set_resident(True)
        n0 = tws.lib().tws_launch_count()
        g.step(10)
        g.sync()
        assert tws.lib().tws_launch_count() - n0 == 1
        g.set_variant(0)  # the plain kernel: one launch per step again
        n0 = tws.lib().tws_launch_count()
        g.step(10)
        g.sync()
        assert tws.lib().tws_launch_count() - n0 == 10


def test_too_large_is_refused(tws):
    assert tws.resident_fits(1024, 1024) == 0
    assert tws.resident_fits(256, 256) == 16
    with tws.Grid(1024, 1024) as g:
        with pytest.raises(tws.TwsError) as e:
            g.set_resident(True)
        assert e.value.code == tws.ERR_UNSUPPORTED
    with tws.Grid(256, 256) as g:
        with pytest.raises(tws.TwsError) as e:
            g.set_resident(True, 2)  # 915 KB of state in two CTAs
        assert e.value.code == tws.ERR_UNSUPPORTED
        with pytest.raises(tws.TwsError) as e:
            g.set_resident(True, 3)
        assert e.value.code == tws.ERR_INVALID or e.value.code == tws.ERR_UNSUPPORTED


def test_autotune_considers_it_and_keeps_state(tws, oracle):
    W = H = 256
    p = tws.params_physical(0.02, 9.81, 1.0, 1.0, 0.998, tws.BOUNDARY_CLOSED)
    rain = tws.rain_disks(3, W, H, 16, 0.01, 1)
    b, d = oracle.terrain(3, W, H, 40.0, 15.0)
    with tws.Grid(W, H, p) as g:
        g.upload(b, d)
        g.set_sources(rain)
        g.step(5)
        best = g.autotune(12)
        assert best == tws.VARIANT_RESIDENT or 0 <= best < len(tws.variants())
        g.step(7)
        gd, gf, gv = g.download()
        if best == tws.VARIANT_RESIDENT:
            # long calls take one resident launch, short ones the tiled kernels
            n0 = tws.lib().tws_launch_count()
            g.step(40)
            g.sync()
            assert tws.lib().tws_launch_count() - n0 == 1
            n0 = tws.lib().tws_launch_count()
            g.step(1)
            g.sync()
            assert tws.lib().tws_launch_count() - n0 == 1
    od, of, ov = oracle_run(oracle, b, d, np.zeros((H, W, 4), np.float32), p.as_tuple(), rain, 12,
                            oracle.BOUNDARY_CLOSED)
    assert_bitexact(gd, od, "depth")
    assert_bitexact(gf, of, "flux")
    assert_bitexact(gv, ov, "velocity")


def test_reference_scene_with_pipelined_io(tws, oracle):
    """The reference's own noise scene (open border, the reference's brush
    parameters), advanced by the resident kernel in calls of 100 steps while
    each state is downloaded asynchronously: every download is the oracle's
    state after that many steps."""
    import torch
    W = H = 192
    p = tws.params_reference(60.0, 0.98, 10.0, 1024.0, W, tws.BOUNDARY_OPEN)
    brush = [(tws.SOURCE_BRUSH, 100.5, 80.25, 32.0, 0.5)]
    outs = [tuple(torch.empty(shape, dtype=torch.float32, pin_memory=True).numpy()
                  for shape in ((H, W), (H, W, 4), (H, W, 2))) for _ in range(3)]
    with tws.Grid(W, H, p) as g:
        g.generate_reference_scene()
        g.set_sources(brush)
        g.set_resident(True)
        for i in range(3):
            g.step(100)
            g.download_async(outs[i])
        g.io_wait()
    b, d = oracle.reference_terrain(W, H)
    f = np.zeros((H, W, 4), np.float32)
    v = np.zeros((H, W, 2), np.float32)
    kf, ka, c = p.as_tuple()
    for i in range(3):
        oracle.step_f32(b, d, f, v, kf, ka, c, oracle.BOUNDARY_OPEN,
                        [(s[0], s[1], s[2], s[3], s[4]) for s in brush], nsteps=100)
        assert_bitexact(outs[i][0], d, f"depth after {100 * (i + 1)} steps")
        assert_bitexact(outs[i][1], f, f"flux after {100 * (i + 1)} steps")
        assert_bitexact(outs[i][2], v, f"velocity after {100 * (i + 1)} steps")
