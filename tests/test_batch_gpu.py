"""GPU tests of batches: many uneven grids advanced by one launch per step
(chains replayed from CUDA graphs) give, grid by grid, the same bits
as the oracle -- alone or in the mix, with grids joining and leaving between
calls, with per-grid step counts, with graphs on or off."""
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


# uneven grids: ragged sizes, both borders, different constants and sources
SPECS = [
    # (W, H, boundary, damping, seed, rain radius, rain rate)
    (96, 80, 0, 0.998, 1, 10, 0.02),
    (257, 33, 1, 0.99, 2, 6, 0.05),
    (33, 190, 0, 0.995, 3, 5, 0.01),
    (1, 45, 0, 0.998, 4, 0, 0.0),
    (128, 128, 1, 0.97, 5, 20, 0.005),
    (70, 7, 0, 0.998, 6, 3, 0.1),
    (200, 160, 1, 0.998, 7, 30, 0.01),  # interior tiles for every tile shape
]


def make_grid(tws, oracle, spec, flux_storage=0):
    W, H, boundary, damping, seed, r, rate = spec
    p = tws.params_physical(0.02, 9.81, 1.0, 1.0, damping, boundary)
    b, d = oracle.terrain(seed, W, H, 40.0, 15.0)
    g = tws.Grid(W, H, p, flux_storage)
    g.upload(b, d)
    srcs = tws.rain_disks(seed, W, H, r, rate, 1) if r > 0 else []
    g.set_sources(srcs)
    return g, (b, d, p, srcs)


def oracle_state(oracle, setup, steps, flux_scale=0.0):
    b, d, p, srcs = setup
    H, W = b.shape
    d = d.copy()
    f = np.zeros((H, W, 4), np.float32)
    v = np.zeros((H, W, 2), np.float32)
    kf, ka, c = p.as_tuple()
    oracle.step_f32(b.copy(), d, f, v, kf, ka, c, p.boundary,
                    [(s[0], s[1], s[2], s[3], s[4]) for s in srcs], nsteps=steps,
                    flux_scale=flux_scale)
    return d, f, v


@pytest.mark.parametrize("variant", range(7))
def test_batch_variants_match_oracle_per_grid(tws, oracle, variant):
    if variant >= len(tws.batch_variants()):
        pytest.skip("no such batched variant")
    grids, setups = zip(*[make_grid(tws, oracle, s) for s in SPECS])
    with tws.Batch() as batch:
        for g in grids:
            batch.add(g)
        batch.set_variant(variant)
        batch.step(37)  # two full chains and a partial one; odd for K = 2
        batch.sync()
        for g, setup in zip(grids, setups):
            od, of, ov = oracle_state(oracle, setup, 37)
            gd, gf, gv = g.download()
            assert_bitexact(gd, od, f"depth {g.width}x{g.height}")
            assert_bitexact(gf, of, f"flux {g.width}x{g.height}")
            assert_bitexact(gv, ov, f"velocity {g.width}x{g.height}")
    for g in grids:
        g.close()


@pytest.mark.parametrize("graphs", [True, False])
def test_batch_step_each_and_join_leave(tws, oracle, graphs):
    """Grids join and leave between calls and advance by their own counts;
    each result equals the grid alone."""
    made = [make_grid(tws, oracle, s) for s in SPECS[:6]]
    grids = [m[0] for m in made]
    setups = [m[1] for m in made]
    done = {}
    with tws.Batch() as batch:
        batch.use_graphs(graphs)
        for g in grids[:3]:
            batch.add(g)
        batch.step_each([5, 21, 0])
        done[0] = 5
        batch.add(grids[3])
        batch.add(grids[4])
        batch.step_each([0, 11, 40, 17, 3])
        batch.remove(grids[0])          # leaves after 5 steps
        batch.add(grids[5])
        batch.step_each([1, 2, 3, 4, 16])
        batch.sync()
        totals = {1: 21 + 11 + 1, 2: 0 + 40 + 2, 3: 17 + 3, 4: 3 + 4, 5: 16}
        done.update(totals)
        chains, replayed = batch.stats()
        assert chains > 0
        assert (replayed > 0) == graphs
    for i, g in enumerate(grids):
        od, of, ov = oracle_state(oracle, setups[i], done[i])
        gd, gf, gv = g.download()
        assert_bitexact(gd, od, f"depth grid {i}")
        assert_bitexact(gf, of, f"flux grid {i}")
        assert_bitexact(gv, ov, f"velocity grid {i}")
        g.close()


@pytest.mark.parametrize("variant", [None, 1, 6])
def test_batch_fp16_storage_matches_oracle(tws, oracle, variant):
    made = [make_grid(tws, oracle, s, flux_storage=tws.FLUX_F16) for s in SPECS[:4] + SPECS[6:]]
    with tws.Batch(tws.FLUX_F16) as batch:
        if variant is not None:
            batch.set_variant(variant)
        for g, _ in made:
            batch.add(g)
        batch.step(24)
        batch.sync()
        for g, setup in made:
            scale = g.buffers().flux_scale
            od, of, ov = oracle_state(oracle, setup, 24, flux_scale=scale)
            gd, gf, gv = g.download()
            assert_bitexact(gd, od, "depth")
            assert_bitexact(gf, of, "flux")
            assert_bitexact(gv, ov, "velocity")
    for g, _ in made:
        g.close()


def test_batch_rejects_mixed_storage_and_double_membership(tws, oracle):
    g32, _ = make_grid(tws, oracle, SPECS[0])
    g16, _ = make_grid(tws, oracle, SPECS[1], flux_storage=tws.FLUX_F16)
    with tws.Batch() as b1, tws.Batch() as b2:
        b1.add(g32)
        with pytest.raises(tws.TwsError):
            b1.add(g16)
        with pytest.raises(tws.TwsError):
            b2.add(g32)
        with pytest.raises(tws.TwsError):
            b1.step_each([1, 2])
    g32.close()
    g16.close()


@pytest.mark.parametrize("variant", [1, 4])
def test_batch_reused_memory_new_tensor_maps(tws, oracle, variant):
    """A grid is destroyed and new grids take its memory from the pool with
    different contents and shapes: the tensor maps written into the reused
    memory must be the ones the batched kernel uses (the first chain after a
    write fences them), so every result matches the oracle bit for bit."""
    first = [make_grid(tws, oracle, s) for s in SPECS[:3]]
    with tws.Batch() as batch:
        batch.set_variant(variant)
        for g, _ in first:
            batch.add(g)
        batch.step(6)
        batch.sync()
        for g, _ in first:
            batch.remove(g)
            g.close()
        # similar sizes, different shapes and contents, likely in the freed memory
        respec = [(80, 96, 1, 0.99, 11, 9, 0.03), (33, 257, 0, 0.995, 12, 6, 0.02),
                  (190, 33, 1, 0.998, 13, 5, 0.04)]
        second = [make_grid(tws, oracle, s) for s in respec]
        for g, _ in second:
            batch.add(g)
        batch.step(10)
        batch.sync()
        for g, setup in second:
            od, of, ov = oracle_state(oracle, setup, 10)
            gd, gf, gv = g.download()
            assert_bitexact(gd, od, f"depth {g.width}x{g.height}")
            assert_bitexact(gf, of, f"flux {g.width}x{g.height}")
            assert_bitexact(gv, ov, f"velocity {g.width}x{g.height}")
    for g, _ in second:
        g.close()


@pytest.mark.parametrize("flux_storage", [0, 1])
def test_batch_large_grid_matches_single_grid_path(tws, flux_storage):
    """A 4096x2048 grid (8192 tiles) batched with small ones gives the same
    bits as the same grids stepped alone by the single-grid kernel."""
    specs = [(4096, 2048, 11), (300, 200, 12), (64, 1000, 13)]
    p = tws.params_physical(boundary=tws.BOUNDARY_CLOSED)

    def make():
        gs = []
        for W, H, seed in specs:
            g = tws.Grid(W, H, p, flux_storage)
            g.generate_scene(seed, 40.0, 15.0)
            g.set_sources(tws.rain_disks(seed, W, H, 24, 0.01, 1))
            gs.append(g)
        return gs

    alone = make()
    for g in alone:
        g.step(10)
    want = [g.download() for g in alone]
    for g in alone:
        g.close()
    batched = make()
    with tws.Batch(flux_storage) as batch:
        for g in batched:
            batch.add(g)
        batch.step(10)
        batch.sync()
        got = [g.download() for g in batched]
    for g in batched:
        g.close()
    for (W, H, _), w, gg in zip(specs, want, got):
        for name, a, b in zip(("depth", "flux", "velocity"), gg, w):
            assert_bitexact(a, b, f"{name} {W}x{H}")


def test_batch_autotune_preserves_state(tws, oracle):
    made = [make_grid(tws, oracle, s) for s in SPECS]
    with tws.Batch() as batch:
        for g, _ in made:
            batch.add(g)
        batch.step(3)
        v = batch.autotune(16)
        assert 0 <= v < len(tws.batch_variants())
        batch.step(5)
        batch.sync()
        for g, setup in made:
            od, of, ov = oracle_state(oracle, setup, 8)
            gd, gf, gv = g.download()
            assert_bitexact(gd, od, "depth")
            assert_bitexact(gf, of, "flux")
    for g, _ in made:
        g.close()


@pytest.mark.parametrize("variant", [4, 6])
def test_batch_uneven_steps_and_membership(tws, oracle, variant):
    """Members with different step counts (remainders that are not multiples
    of K run as one-step launches), a member joining between calls and one
    leaving, every result bit-exact."""
    made = [make_grid(tws, oracle, s) for s in SPECS]
    counts = [5, 17, 0, 33, 2, 11, 40]
    with tws.Batch() as batch:
        batch.set_variant(variant)
        for g, _ in made[:-1]:
            batch.add(g)
        batch.step_each(counts[:-1])
        batch.sync()
        batch.add(made[-1][0])  # joins
        batch.remove(made[0][0])  # leaves
        batch.step_each([4] * (len(made) - 1))
        batch.sync()
        for i, (g, setup) in enumerate(made):
            total = counts[i] + (4 if i > 0 else 0)
            if i == len(made) - 1:
                total = 4
            od, of, ov = oracle_state(oracle, setup, total)
            gd, gf, gv = g.download()
            assert_bitexact(gd, od, f"depth {g.width}x{g.height}")
            assert_bitexact(gf, of, f"flux {g.width}x{g.height}")
            assert_bitexact(gv, ov, f"velocity {g.width}x{g.height}")
    for g, _ in made:
        g.close()
