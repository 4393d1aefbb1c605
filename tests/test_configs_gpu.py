"""The benchmark configurations at their stated sizes on the GPU, checked
against the oracle bit for bit (with fewer steps than the benchmark runs, so
that the CPU oracle finishes in seconds):

* the 64 uneven grids of the batched configuration (sides 128-2048, aspect
  1-4, per-grid terrain, fill and rain) advanced together by the batched
  kernel;
* the 16384^2 grid of the mixed-precision configuration with FP16 flux
  storage and its 8 rain disks;
* requests of the serving stream (sides 64-4096, FP16 storage) served
  together, each compared with the oracle directly rather than with the same
  request run alone on the GPU."""
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


def oracle_state(O, seed, W, H, fill, sources, steps, flux_scale=0.0):
    b, d = O.terrain(seed, W, H, 40.0, fill)
    f = np.zeros((H, W, 4), np.float32)
    v = np.zeros((H, W, 2), np.float32)
    kf, ka, c = (np.float32(x) for x in O.params_physical())
    O.step_f32(b, d, f, v, kf, ka, c, O.BOUNDARY_CLOSED,
               [(s[0], s[1], s[2], s[3], s[4]) for s in sources], nsteps=steps,
               flux_scale=flux_scale)
    return d, f, v


def test_batched_configuration_all_64_grids(tws, oracle):
    import bench
    work = bench.c3_workload()
    assert len(work) == 64
    steps = 40
    p = tws.params_physical(0.02, 9.81, 1.0, 1.0, 0.998, tws.BOUNDARY_CLOSED)
    grids, srcs = [], []
    with tws.Batch() as batch:
        for w in work:
            g = tws.Grid(w["W"], w["H"], p)
            src = tws.rain_disks(w["seed"], w["W"], w["H"], w["radius"], w["rate"], 1)
            g.set_sources(src)
            g.generate_scene(w["seed"], 40.0, w["fill"])
            grids.append(g)
            srcs.append(src)
            batch.add(g)
        batch.step(steps)
        batch.sync()
        for g in grids:
            batch.remove(g)
    try:
        for w, g, src in zip(work, grids, srcs):
            gd, gf, gv = g.download()
            od, of, ov = oracle_state(oracle, w["seed"], w["W"], w["H"], w["fill"], src, steps)
            tag = f"grid {w['W']}x{w['H']}"
            assert_bitexact(gd, od, f"depth, {tag}")
            assert_bitexact(gf, of, f"flux, {tag}")
            assert_bitexact(gv, ov, f"flow map, {tag}")
    finally:
        for g in grids:
            g.close()


def test_mixed_precision_configuration_16384(tws, oracle):
    N, steps = 16384, 6
    p = tws.params_physical(0.02, 9.81, 1.0, 1.0, 0.998, tws.BOUNDARY_CLOSED)
    rain = tws.rain_disks(2026, N, N, 128, 0.01, 8)
    with tws.Grid(N, N, p, tws.FLUX_F16) as g:
        g.set_sources(rain)
        g.generate_scene(2026, 40.0, 15.0)
        g.step(steps)
        g.sync()
        scale = g.buffers().flux_scale
        gd, gf, gv = g.download()
        gvol = g.volume()
    od, of, ov = oracle_state(oracle, 2026, N, N, 15.0, rain, steps, flux_scale=scale)
    ovol = oracle.volume(od)
    assert_bitexact(gd, od, "depth")
    del gd, od
    assert_bitexact(gf, of, "flux")
    del gf, of
    assert_bitexact(gv, ov, "flow map")
    assert abs(gvol - ovol) <= 1e-9 * ovol, (gvol, ovol)  # the device's FP64 sum


def test_served_requests_match_the_oracle(tws, oracle):
    import bench
    from terrainwatersim_gb300 import serve
    work = bench.c5_workload(12, 20000)
    p = tws.params_physical(0.02, 9.81, 1.0, 1.0, 0.998, tws.BOUNDARY_CLOSED)
    reqs, srcs = [], {}
    for i, w in enumerate(work):
        src = tws.rain_disks(w["seed"], w["W"], w["H"], w["radius"], w["rate"], 1)
        steps = min(w["steps"], 60)  # the CPU oracle replays every request
        reqs.append(serve.make_request(i + 1, w["W"], w["H"], w["seed"], w["fill"], p, src, steps,
                                       0.0))
        srcs[i + 1] = (w, src, steps)
    with tws.Grid(64, 64, p, tws.FLUX_F16) as g:
        scale = g.buffers().flux_scale  # the per-grid scale FP16 storage picks
    with serve.Server(memory_budget_bytes=60e9, flux_storage=tws.FLUX_F16,
                      keep_grids=True) as srv:
        for r in reqs:
            srv.submit(r)
        srv.close_submissions()
        srv.run()
        results = {r.id: r for r in srv.results()}
        assert len(results) == len(reqs)
        for rid, (w, src, steps) in srcs.items():
            res = results[rid]
            assert res.status == 0 and res.steps == steps
            gd, gf, gv = res.grid.download()
            res.grid.close()
            od, of, ov = oracle_state(oracle, w["seed"], w["W"], w["H"], w["fill"], src, steps,
                                      flux_scale=scale)
            tag = f"request {rid} ({w['W']}x{w['H']}, {steps} steps)"
            assert_bitexact(gd, od, f"depth, {tag}")
            assert_bitexact(gf, of, f"flux, {tag}")
            assert_bitexact(gv, ov, f"flow map, {tag}")
            assert abs(res.volume - oracle.volume(od)) <= 1e-9 * oracle.volume(od)
