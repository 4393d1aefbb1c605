"""tws_volume_noalloc: the total-volume entry point that allocates nothing.

Some callers cannot allocate device memory: a renderer that owns all GPU
memory through its own pools, a frame loop that must not take the implicit
synchronisation of cudaMalloc/cudaFree, or code recording a CUDA graph.  This
entry point takes the depth buffer and an output pointer from the caller and
keeps its per-row partial sums in a fixed array inside libtws.so.  Its result
must agree with tws_volume (which uses scratch the grid allocated) within the
tolerance the other volume tests use, call after call.

The file name sorts last so that a run stopping at the first failure has run
every other test first.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL_TOL = 1e-12  # the volume tolerance of tests/test_step_gpu.py


@pytest.fixture(scope="module")
def tws():
    import terrainwatersim_gb300 as t
    t.lib()
    return t


def _noalloc(tws, g, out_ptr):
    """One call through the C ABI on the grid's stream."""
    buf = g.buffers()
    return tws.lib().tws_volume_noalloc(C.c_void_p(buf.depth), buf.width, buf.height, buf.pitch,
                                        float(g.params.cell_area), C.c_void_p(out_ptr),
                                        C.c_void_p(g.stream))


@pytest.mark.parametrize("W,H", [(300, 200), (517, 3000)])
def test_noalloc_volume_matches_tws_volume_twice_in_a_row(tws, W, H):
    import torch

    # The output lives in memory the caller owns (allocated here, by the test).
    out = torch.zeros(4, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    p = tws.params_physical(0.02, 9.81, 1.0, 1.0, 0.998, tws.BOUNDARY_CLOSED)
    with tws.Grid(W, H, p) as g:
        g.generate_scene(31, 40.0, 15.0)
        g.set_sources(tws.rain_disks(31, W, H, 20, 0.05, 1))
        g.step(9)
        want1 = g.volume()
        # two calls in a row on the same state
        assert _noalloc(tws, g, out.data_ptr()) == tws.TWS_OK
        assert _noalloc(tws, g, out.data_ptr() + 8) == tws.TWS_OK
        g.sync()
        # the state changes (rain), then two more calls
        g.step(5)
        want2 = g.volume()
        assert _noalloc(tws, g, out.data_ptr() + 16) == tws.TWS_OK
        assert _noalloc(tws, g, out.data_ptr() + 24) == tws.TWS_OK
        g.sync()
    got = out.cpu().numpy()
    assert want2 > want1 > 0
    for i, want in enumerate((want1, want1, want2, want2)):
        assert abs(got[i] - want) <= REL_TOL * want, (i, got[i], want)
    if H <= 1024:
        # same partition of the rows as tws_volume: identical bits
        assert got[0] == want1 and got[2] == want2


def test_noalloc_rejects_grids_beyond_its_scratch(tws):
    # Size checks happen before anything is enqueued: the pointers are never used.
    dummy = C.c_void_p(256)
    rc = tws.lib().tws_volume_noalloc(dummy, 8, tws.VOLUME_NOALLOC_MAX_ROWS + 1, 32, 1.0, dummy,
                                      None)
    assert rc == tws.ERR_TOO_LARGE
    assert b"TWS_VOLUME_NOALLOC_MAX_ROWS" in tws.lib().tws_error_string(rc)
    assert tws.lib().tws_volume_noalloc(None, 8, 8, 32, 1.0, dummy, None) == tws.ERR_INVALID
    assert tws.lib().tws_volume_noalloc(dummy, 64, 8, 32, 1.0, dummy, None) == tws.ERR_INVALID
    # misaligned depth (floats) or result (a double): refused before any launch
    assert tws.lib().tws_volume_noalloc(C.c_void_p(258), 8, 8, 32, 1.0, dummy,
                                        None) == tws.ERR_INVALID
    assert tws.lib().tws_volume_noalloc(dummy, 8, 8, 32, 1.0, C.c_void_p(260),
                                        None) == tws.ERR_INVALID
