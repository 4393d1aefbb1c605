"""FP16 flux storage on a scene where the water moves everywhere, against the
FP64 oracle.

The benchmark scenes start as a lake at rest (d = max(0, 15 - b)), so away
from the rain disks the flux stays exactly zero and a depth comparison there
says nothing about the storage precision.  Here every cell starts out of
equilibrium: random bumps on the water surface and a random initial outflow
(the style of the reference-pinned fixture ref_bumps_48x32), on 1024^2 cells
with a rain disk, 300 steps, closed walls.

What is asserted:
* the GPU's FP16 mode equals the oracle's FP16 mode bit for bit, and the FP32
  storage equals the FP32 oracle bit for bit (the parity bar);
* against the FP64 oracle from the same (quantised) initial state, the total
  volume drifts by at most 1e-4 relative in both storage modes (the bound the
  precision mode is specified to);
* the FP64 comparison sees the storage: FP16 and FP32 give different max depth
  errors, and each stays inside a bound stated here from measurement (the
  oracle gives FP32 1.4e-3 of the largest depth, FP16 1.9e-2: half precision
  keeps 11 mantissa bits of each stored outflow, and the steep fronts of this
  scene turn that into a phase error of up to a few decimetres in a few
  cells, while the volume stays conserved to FP32 round-off).
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import assert_bitexact

pytestmark = pytest.mark.gpu

N, STEPS = 1024, 300
# relative max depth error against FP64 (max |d - d64| / max d64) allowed per
# storage mode; the oracle gives 1.4e-3 (FP32) and 1.9e-2 (FP16) on this scene
REL_DEPTH_BOUND = {"f32": 5e-3, "f16": 5e-2}
VOLUME_DRIFT_BOUND = 1e-4


@pytest.fixture(scope="module")
def tws():
    import terrainwatersim_gb300 as t
    t.lib()
    return t


def moving_scene(O):
    rng = np.random.default_rng(1024)
    b, d = O.terrain(31, N, N, 40.0, 15.0)
    d = (d + np.maximum(0.0, rng.uniform(-1.0, 3.0, (N, N)))).astype(np.float32)
    f = rng.uniform(0.0, 0.5, (N, N, 4)).astype(np.float32)
    return b, d, f


@pytest.fixture(scope="module")
def runs(tws, oracle):
    """GPU runs in both storage modes, the oracle in both FP32 modes, and the
    FP64 oracle, all from the same initial state (the flux quantised to what
    FP16 storage holds, so that the three start identical)."""
    O = oracle
    b, d, f = moving_scene(O)
    p = tws.params_physical(boundary=tws.BOUNDARY_CLOSED)
    rain = tws.rain_disks(77, N, N, 24, 0.01, 1)
    out = {}
    f0 = None
    for name, fs in (("f16", tws.FLUX_F16), ("f32", tws.FLUX_F32)):
        with tws.Grid(N, N, p, fs) as g:
            if f0 is None:  # the common initial flux: what FP16 storage holds
                scale = g.buffers().flux_scale
                f0 = f.copy()
                O.quantize_f16(f0, scale)
            g.upload(b, d, f0)
            g.set_sources(rain)
            g.step(STEPS)
            g.sync()
            gd, gf, gv = g.download()
            out[name] = dict(d=gd, f=gf, v=gv, vol=g.volume(), scale=g.buffers().flux_scale)
    src = [(s[0], s[1], s[2], s[3], s[4]) for s in rain]
    kf, ka, c = p.as_tuple()
    for name, sc in (("f16", out["f16"]["scale"]), ("f32", 0.0)):
        od, of = d.copy(), f0.copy()
        ov = np.zeros((N, N, 2), np.float32)
        O.step_f32(b, od, of, ov, kf, ka, c, O.BOUNDARY_CLOSED, src, nsteps=STEPS, flux_scale=sc)
        out["oracle_" + name] = dict(d=od, f=of, v=ov)
    b64, d64, f64 = b.astype(np.float64), d.astype(np.float64), f0.astype(np.float64)
    O.step_f64(b64, d64, f64, None, *O.params_physical(), O.BOUNDARY_CLOSED,
               [(s[0], s[1], s[2], s[3], 0.01) for s in rain], nsteps=STEPS)
    out["f64"] = dict(d=d64, vol=O.volume(d64))
    out["d0"] = d.astype(np.float64)
    return out


def test_the_scene_moves_everywhere(runs):
    moved = np.abs(runs["f64"]["d"] - runs["d0"]) > 1e-3
    assert moved.mean() > 0.9, f"only {moved.mean():.1%} of the cells changed by more than 1 mm"


@pytest.mark.parametrize("mode", ["f16", "f32"])
def test_storage_modes_match_the_oracle_bit_for_bit(runs, mode):
    got, want = runs[mode], runs["oracle_" + mode]
    assert_bitexact(got["d"], want["d"], f"{mode} depth")
    assert_bitexact(got["f"], want["f"], f"{mode} flux")
    assert_bitexact(got["v"], want["v"], f"{mode} flow map")


@pytest.mark.parametrize("mode", ["f16", "f32"])
def test_against_fp64(runs, mode):
    ref = runs["f64"]["d"]
    err = np.abs(runs[mode]["d"].astype(np.float64) - ref)
    rel = err.max() / np.abs(ref).max()
    drift = abs(runs[mode]["vol"] - runs["f64"]["vol"]) / runs["f64"]["vol"]
    print(f"{mode}: max depth error {err.max():.3e} m (relative {rel:.3e}), "
          f"mean {err.mean():.3e} m, volume drift {drift:.3e}")
    assert drift <= VOLUME_DRIFT_BOUND, drift
    assert rel <= REL_DEPTH_BOUND[mode], rel


def test_fp16_and_fp32_errors_differ(runs):
    ref = runs["f64"]["d"]
    e16 = np.abs(runs["f16"]["d"] - ref).max()
    e32 = np.abs(runs["f32"]["d"] - ref).max()
    assert e16 != e32
    assert e16 > e32, (e16, e32)  # the coarser storage shows in the error
