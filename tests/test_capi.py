"""CPU tests of libtws.so's C ABI: the library loads, exports every entry
point include/tws.h declares, and its host-only helpers agree with the
oracle.  No kernel runs here."""
from __future__ import annotations

import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import ROOT


@pytest.fixture(scope="module")
def tws():
    from terrainwatersim_gb300 import build
    build.build()
    import terrainwatersim_gb300 as t
    return t


def declared_symbols():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            text = open(os.path.join(ROOT, "include", h)).read()
            names |= set(re.findall(r"TWS_API\s+[\w\s\*]+?\b(tws_\w+)\s*\(", text))
    return sorted(names)


def test_every_declared_symbol_is_exported(tws):
    names = declared_symbols()
    assert len(names) >= 20, names
    L = tws.lib()
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_params_physical_matches_oracle(tws, oracle):
    p = tws.params_physical(0.02, 9.81, 1.0, 1.0, 0.998)
    kf, ka, c = oracle.params_physical(0.02, 9.81, 1.0, 1.0, 0.998)
    assert p.as_tuple() == (np.float32(kf), np.float32(ka), np.float32(c))
    assert p.cell_area == 1.0 and p.boundary == tws.BOUNDARY_CLOSED
    q = tws.params_physical(0.01, 9.81, 2.0, 4.0, 0.99)
    assert q.water_acceleration_per_step == np.float32(0.01 * 9.81 * 2.0 / 4.0)
    assert q.cell_area_inv_time_scaled == np.float32(0.01 / 16.0)
    assert q.cell_area == 16.0


@pytest.mark.parametrize("sps,damp,acc,world,res", [(60.0, 0.98, 10.0, 1024.0, 1024),
                                                     (60.0, 0.96, 30.0, 1024.0, 512),
                                                     (120.0, 0.5, 3.0, 300.0, 1000)])
def test_params_reference_matches_oracle(tws, oracle, sps, damp, acc, world, res):
    p = tws.params_reference(sps, damp, acc, world, res)
    assert p.as_tuple() == oracle.params_reference(sps, damp, acc, world, res)


def test_rain_disks_match_oracle(tws, oracle):
    for (W, H, r, n) in ((256, 256, 16, 1), (4096, 4096, 64, 1), (16384, 16384, 128, 8),
                         (20, 10, 16, 2)):
        disks = tws.rain_disks(2026, W, H, r, 0.01, n)
        centres = oracle.rain_centers(2026, W, H, r, n)
        assert [(int(s[1]), int(s[2])) for s in disks] == centres
        assert all(s[0] == tws.SOURCE_DISK and s[3] == r for s in disks)


def test_invalid_arguments_rejected_without_touching_the_gpu(tws):
    L = tws.lib()
    p = tws.SimParams()
    assert L.tws_params_physical(-1.0, 9.81, 1.0, 1.0, 0.998, 0, C.byref(p)) == tws.ERR_INVALID
    assert L.tws_params_physical(0.02, 9.81, 1.0, 1.0, 0.998, 7, C.byref(p)) == tws.ERR_INVALID
    assert L.tws_params_reference(0.0, 0.98, 10.0, 1024.0, 1024, 0, C.byref(p)) == tws.ERR_INVALID
    good = tws.params_physical()
    h = C.c_void_p()
    assert L.tws_create(0, 16, C.byref(good), 0, None, C.byref(h)) == tws.ERR_INVALID
    assert L.tws_create(16, 16, C.byref(good), 5, None, C.byref(h)) == tws.ERR_INVALID
    bad = tws.SimParams(0.998, 0.1962, 0.02, 1.0, 9)
    assert L.tws_create(16, 16, C.byref(bad), 0, None, C.byref(h)) == tws.ERR_INVALID
    assert L.tws_error_string(tws.ERR_TIMEOUT) == b"device-side wait timed out"
    # asynchronous host I/O and the resident kernel: null handles
    assert L.tws_upload_async(None, None, None, None) == tws.ERR_INVALID
    assert L.tws_download_async(None, None, None, None) == tws.ERR_INVALID
    assert L.tws_io_wait(None) == tws.ERR_INVALID
    assert L.tws_set_resident(None, tws.RESIDENT_AUTO) == tws.ERR_INVALID
    assert L.tws_resident_fits(64, 64, 7) == 0  # no such flux storage
    v = C.c_int(-7)
    assert L.tws_current_variant(None, C.byref(v)) == tws.ERR_INVALID and v.value == -7
    assert L.tws_variant_tail_rows(-1) == tws.ERR_INVALID


def test_resident_fits_answers_no_without_a_gpu(tws):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    assert tws.resident_fits(256, 256) == 0
    assert tws.resident_fits(0, 0) == 0


def test_no_cpu_fallback(tws):
    """Without a GPU the library refuses to create a grid instead of running
    anywhere else."""
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    with pytest.raises(tws.TwsError) as ei:
        tws.Grid(64, 64)
    assert ei.value.code == tws.ERR_CUDA


def test_binding_raises_when_library_missing(tmp_path, monkeypatch):
    import terrainwatersim_gb300 as t
    monkeypatch.setattr(t, "_LIB_PATH", str(tmp_path / "nope.so"))
    monkeypatch.setattr(t, "_lib", None)
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        t.lib()


def test_variant_table(tws):
    v = tws.variants()
    assert len(v) >= 4
    assert {k for k, _, _, _, _, _ in v} == {1, 2, 3, 4}
    for k, tx, ty, stages, smem, kind in v:
        # TMA tile variants stage whole 16-byte units in shared memory; the
        # register-streaming variants (30-column strips) use none; the sweeps
        # yield 64 - 4K columns per warp strip and stage rows in shared memory
        assert ty >= 1 and stages in (1, 2) and 0 <= smem <= 227 * 1024
        if kind == tws.VARIANT_TILE:
            assert smem > 0 and tx % 4 == 0
        elif kind == tws.VARIANT_STREAM:
            assert smem == 0 and tx == 30 and k == 1
        else:
            assert kind == tws.VARIANT_SWEEP and 2 <= k <= 4 and tx == 64 - 4 * k and smem > 0
    assert any(x[5] == tws.VARIANT_SWEEP for x in v)
    assert tws.lib().tws_variant_kind(len(v)) == tws.ERR_INVALID
    # sweeps with a tail of short bands end their queue on units shorter
    # than the tall bands; every other variant has none
    tails = [tws.variant_tail_rows(i) for i in range(len(v))]
    assert any(t > 0 for t in tails)
    for (k, tx, ty, stages, smem, kind), t in zip(v, tails):
        assert t == 0 or (kind == tws.VARIANT_SWEEP and 0 < t < ty)
    assert tws.lib().tws_variant_tail_rows(len(v)) == tws.ERR_INVALID
    # entries 0..3 are the defaults for K = 1..4
    assert [v[i][0] for i in range(4)] == [1, 2, 3, 4]
    assert tws.lib().tws_variant_info(len(v), None, None, None, None, None) == tws.ERR_INVALID
