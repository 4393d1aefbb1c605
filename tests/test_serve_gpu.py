"""GPU tests of the serving loop: requests arrive over time, are admitted
against a memory budget, advance together in batch chains, and each result is
the same -- bit for bit -- as the request run alone."""
from __future__ import annotations

import threading

import numpy as np
import pytest

from conftest import assert_bitexact

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def tws():
    import terrainwatersim_gb300 as t
    t.lib()
    return t


def stream_of_requests(tws, serve, n=10, seed=5):
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(n):
        W = int(rng.integers(24, 200))
        H = int(rng.integers(24, 200))
        boundary = int(rng.integers(0, 2))
        p = tws.params_physical(0.02, 9.81, 1.0, 1.0, float(rng.uniform(0.99, 0.999)), boundary)
        rate = float(rng.uniform(0.002, 0.02))
        src = tws.rain_disks(100 + i, W, H, max(1, min(W, H) // 8), rate, 1)
        reqs.append(serve.make_request(i + 1, W, H, 100 + i, float(rng.uniform(8, 20)), p, src,
                                       int(rng.integers(5, 120)), float(rng.uniform(0, 0.05))))
    return reqs


def alone(tws, req, flux_storage):
    g = tws.Grid(req.width, req.height, req.params, flux_storage)
    g.generate_scene(req.seed, req.height_scale, req.fill)
    g.set_sources([(s.kind, s.cx, s.cy, s.radius, s.rate) for s in req.sources[:req.nsources]])
    g.step(req.steps)
    out = g.download()
    vol = g.volume()
    g.close()
    return out, vol


@pytest.mark.parametrize("flux_storage", [0, 1])
def test_served_results_equal_alone(tws, flux_storage):
    from terrainwatersim_gb300 import serve
    reqs = stream_of_requests(tws, serve)
    with serve.Server(memory_budget_bytes=4e9, flux_storage=flux_storage, keep_grids=True) as srv:
        for r in reqs:
            srv.submit(r)
        srv.close_submissions()
        srv.run()
        results = {r.id: r for r in srv.results()}
        assert len(results) == len(reqs)
        for req in reqs:
            res = results[req.id]
            assert res.status == 0 and res.steps == req.steps
            assert res.done_s >= res.admit_s >= res.arrival_s - 1e-3
            (d, f, v), vol = alone(tws, req, flux_storage)
            gd, gf, gv = res.grid.download()
            assert_bitexact(gd, d, f"depth of request {req.id}")
            assert_bitexact(gf, f, f"flux of request {req.id}")
            assert_bitexact(gv, v, f"velocity of request {req.id}")
            assert res.volume == vol
            res.grid.close()


def test_admission_respects_memory_budget(tws):
    from terrainwatersim_gb300 import serve
    reqs = stream_of_requests(tws, serve, n=8, seed=9)
    sizes = [serve.grid_bytes(r.width, r.height, 1) for r in reqs]
    budget = 2.2 * max(sizes)
    huge = serve.make_request(99, 8192, 8192, 1, 10.0, reqs[0].params, [], 10, 0.0)
    with serve.Server(memory_budget_bytes=budget, flux_storage=1) as srv:
        for r in reqs:
            srv.submit(r)
        srv.submit(huge)
        srv.close_submissions()
        srv.run()
        res = {r.id: r for r in srv.results()}
        st = srv.stats()
    assert st["peak_bytes"] <= budget
    assert res[99].status == tws.ERR_BUSY
    assert all(res[r.id].status == 0 and res[r.id].steps == r.steps for r in reqs)


def test_serial_baseline_gives_the_same_results(tws):
    from terrainwatersim_gb300 import serve
    reqs = stream_of_requests(tws, serve, n=6, seed=3)
    vols = {}
    for serial in (False, True):
        with serve.Server(memory_budget_bytes=4e9, flux_storage=0) as srv:
            for r in reqs:
                srv.submit(r)
            srv.close_submissions()
            srv.run(serial=serial)
            vols[serial] = {r.id: (r.status, r.volume) for r in srv.results()}
            assert srv.stats()["cell_steps"] == sum(r.width * r.height * r.steps for r in reqs)
    assert vols[False] == vols[True]


def test_submissions_from_another_thread(tws):
    from terrainwatersim_gb300 import serve
    reqs = stream_of_requests(tws, serve, n=5, seed=11)
    with serve.Server(memory_budget_bytes=4e9, flux_storage=1) as srv:
        t = threading.Thread(target=srv.run)
        t.start()
        for r in reqs:
            srv.submit(r)
        srv.close_submissions()
        t.join(timeout=120)
        assert not t.is_alive()
        res = srv.results()
    assert sorted(r.id for r in res) == [r.id for r in reqs]
    assert all(r.status == 0 for r in res)
