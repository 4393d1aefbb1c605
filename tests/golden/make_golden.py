"""Generate tests/golden/*.npz from the reference's own shader code.

The reference's compute shaders (terrainwatersim/shader/flowUpdate.comp,
flowApply.comp, waterBrush.comp) are compiled as C++ by `make -C oracle ref`
(see oracle/ref_glsl/glsl_emu.h) and run here on the CPU, dispatch by
dispatch, the way Terrain::PerformSimulationStep drives them
(Terrain.cpp:253-265).  Their outputs are stored as fixtures so that tests
can pin the oracle and the CUDA kernels without the reference checkout.

The reference's native border is the open sink (out-of-range image loads read
zero), so the fixtures use TWS_BOUNDARY_OPEN.

Run:  TWS_REFERENCE_ROOT=<reference checkout> python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402


def case_brush_64():
    """Benchmark terrain, reference parameters at the app's defaults
    (60 steps/s, damping 0.98, acceleration 10; Terrain.cpp:28-30) with one
    brush stroke (BrushSizeSq 32, Terrain.cpp:159), 300 steps."""
    W = H = 64
    b, d = O.terrain(11, W, H, 40.0, 15.0)
    f = np.zeros((H, W, 4), np.float32)
    kf, ka, c = O.params_reference(60.0, 0.98, 10.0, float(W), W)
    brush = (20.3, 40.7, 3.0, 32.0)
    return dict(name="ref_brush_64", b=b, d=d, f=f, params=np.array([kf, ka, c], np.float32),
                brush=np.array(brush, np.float32), steps=300)


def case_bumps_48x32():
    """Non-square grid, rough terrain, nonzero initial outflow, the newest
    screenshot's settings (damping 0.96, acceleration 30), 200 steps."""
    W, H = 48, 32
    rng = np.random.default_rng(4832)
    b = rng.uniform(0.0, 5.0, (H, W)).astype(np.float32)
    d = np.maximum(0.0, rng.uniform(-1.0, 3.0, (H, W))).astype(np.float32)
    d[10:20, 20:30] += 8.0
    f = rng.uniform(0.0, 0.5, (H, W, 4)).astype(np.float32)
    kf, ka, c = O.params_reference(60.0, 0.96, 30.0, float(W), W)
    return dict(name="ref_bumps_48x32", b=b, d=d, f=f, params=np.array([kf, ka, c], np.float32),
                brush=np.zeros(0, np.float32), steps=200)


def main():
    O.build(ref=True)
    if "--render-only" in sys.argv:
        write_render_case()
        return
    if not O.ref_available():
        raise SystemExit("reference library not built (no reference checkout?)")
    for case in (case_brush_64(), case_bumps_48x32()):
        kf, ka, c = case["params"].tolist()
        brush = tuple(case["brush"].tolist()) if case["brush"].size else None
        d_out, f_out, fm = O.ref_steps(case["b"], case["d"], case["f"], kf, ka, c, case["steps"],
                                       brush=brush)
        path = os.path.join(HERE, case["name"] + ".npz")
        np.savez_compressed(path, b=case["b"], d0=case["d"], f0=case["f"], params=case["params"],
                            brush=case["brush"], steps=np.int64(case["steps"]), d=d_out, f=f_out,
                            flowmap_f16=fm)
        print(f"wrote {path}: volume {O.volume(d_out):.6f}")
    write_reference_scene()
    write_render_case()


RENDER_CASE = dict(N=64, seed=12, fill=15.0, brush=(25.6, 19.2, 40.0, 6.0), steps=25)


def render_case_state():
    """The state the render fixture is taken on: the benchmark terrain (seed
    12) on 64 x 64 cells, open border, one brush stroke, 25 steps of the
    benchmark's physical parameters -- water flowing, some cells dry."""
    c = RENDER_CASE
    N = c["N"]
    b, d = O.terrain(c["seed"], N, N, 40.0, c["fill"])
    f = np.zeros((N, N, 4), np.float32)
    v = np.zeros((N, N, 2), np.float32)
    kf, ka, cc = O.params_physical()
    bx, by, size_sq, intensity = c["brush"]
    O.sources_f32(d, [(O.SOURCE_BRUSH, bx, by, size_sq, intensity)])
    O.step_f32(b, d, f, v, kf, ka, cc, O.BOUNDARY_OPEN, nsteps=c["steps"])
    return b, d, v


def write_render_case():
    """What the reference's water-rendering shaders compute from that state
    (their own code, compiled by `make -C oracle ref`; see
    oracle/ref_glsl/render_emu.h): surface and tessellated heights, the dry
    flag, the heightmap normal, the flow speed and the foam blend factor."""
    if not O.ref_render_available():
        raise SystemExit("reference render library not built")
    b, d, v = render_case_state()
    fm = v.astype(np.float16).view(np.uint16)
    r = O.ref_surface(b, d, fm)
    path = os.path.join(HERE, "ref_render_64.npz")
    np.savez_compressed(path, b=b, d=d, v=v, flowmap_f16=fm,
                        **{"out_" + k: val for k, val in r.items()},
                        **{"case_" + k: np.array(val) for k, val in RENDER_CASE.items()})
    print(f"wrote {path}")


def write_reference_scene():
    """The reference's own noise scene (Terrain::CreateHeightmapFromNoiseAndResetSim)
    from its own Random.cpp / NoiseGenerator.cpp, compiled by `make -C oracle
    ref`: the application's seed, the first and second scene after start-up,
    a 96x96 grid at the default height scale 300."""
    if not O.ref_noise_available():
        raise SystemExit("reference noise library not built")
    R = O.ref_noise()
    out = {}
    for gen in (0, 1):
        t = np.empty(4096, np.float32)
        R.tws_ref_noise_table(O.REFERENCE_NOISE_SEED, gen, O._fp(t))
        N = 96
        b = np.empty((N, N), np.float32)
        d = np.empty((N, N), np.float32)
        R.tws_ref_reference_terrain(O.REFERENCE_NOISE_SEED, gen, N, 300.0, O._fp(b), O._fp(d))
        out[f"table{gen}"], out[f"b{gen}"], out[f"d{gen}"] = t, b, d
    path = os.path.join(HERE, "ref_noise_scene_96.npz")
    np.savez_compressed(path, seed=np.uint32(O.REFERENCE_NOISE_SEED), height_scale=np.float32(300.0),
                        **out)
    print(f"wrote {path}")


if __name__ == "__main__":
    main()
