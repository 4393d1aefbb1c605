"""ctypes wrapper of the test oracle (TEST INFRASTRUCTURE, not the product).

Only tests/, the smoke check and bench.py's CPU-baseline arm import this
module.  It loads two CPU libraries built by oracle/Makefile:

* ``_build/libtws_oracle.so`` -- the restatement of the reference's step
  (flowUpdate.comp + flowApply.comp + waterBrush.comp), FP32 and FP64, OpenMP,
  plus the synthetic scene generator;
* ``_ref/libtws_ref.so`` -- the reference's own shader files run on the CPU
  through oracle/ref_glsl/glsl_emu.h.  It exists only where the reference
  checkout is present; ``ref_available()`` tells.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(HERE, "_build", "libtws_oracle.so")
_REF_PATH = os.path.join(HERE, "_ref", "libtws_ref.so")
_lock = threading.Lock()
_lib = None
_ref = None

BOUNDARY_CLOSED = 0
BOUNDARY_OPEN = 1
SOURCE_DISK = 0
SOURCE_BRUSH = 1


class Source(C.Structure):
    _fields_ = [("kind", C.c_int), ("pad_", C.c_int), ("cx", C.c_double), ("cy", C.c_double),
                ("radius", C.c_double), ("rate", C.c_double)]


def build(ref: bool = False) -> None:
    """Compile the oracle (and, with ref=True, the reference shaders) in place."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True)


def _fp(a):
    return a.ctypes.data_as(C.c_void_p)


def lib():
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(_LIB_PATH):
                build()
            L = C.CDLL(_LIB_PATH)
            L.tws_oracle_terrain.argtypes = [C.c_uint64, C.c_int, C.c_int, C.c_float, C.c_float,
                                             C.c_void_p, C.c_void_p]
            L.tws_oracle_rain_centers.argtypes = [C.c_uint64, C.c_int, C.c_int, C.c_int, C.c_int,
                                                  C.c_void_p, C.c_void_p]
            L.tws_oracle_pcg32.argtypes = [C.c_uint64, C.c_uint64, C.c_uint64, C.c_int, C.c_void_p]
            L.tws_oracle_params_physical.argtypes = [C.c_double] * 5 + [C.c_void_p]
            L.tws_oracle_params_reference.argtypes = [C.c_float] * 4 + [C.c_uint, C.c_void_p]
            L.tws_oracle_step_f32.argtypes = ([C.c_int, C.c_int, C.c_float, C.c_float, C.c_float,
                                               C.c_int, C.c_float] + [C.c_void_p] * 5
                                              + [C.c_int] * 3)
            L.tws_oracle_quantize_f16.argtypes = [C.c_void_p, C.c_longlong, C.c_float]
            L.tws_oracle_step_f32.restype = C.c_double
            L.tws_oracle_step_f64.argtypes = ([C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                               C.c_int] + [C.c_void_p] * 5 + [C.c_int] * 3)
            L.tws_oracle_step_f64.restype = C.c_double
            L.tws_oracle_sources_f32.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int]
            L.tws_oracle_volume_f32.argtypes = [C.c_void_p, C.c_longlong, C.c_double]
            L.tws_oracle_volume_f32.restype = C.c_double
            L.tws_oracle_volume_f64.argtypes = [C.c_void_p, C.c_longlong, C.c_double]
            L.tws_oracle_volume_f64.restype = C.c_double
            L.tws_oracle_max_threads.restype = C.c_int
            _lib = L
    return _lib


def ref_available() -> bool:
    return os.path.exists(_REF_PATH)


def ref():
    global _ref
    with _lock:
        if _ref is None:
            R = C.CDLL(_REF_PATH)
            R.tws_ref_flow_update.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p]
            R.tws_ref_flow_apply.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int,
                                             C.c_void_p]
            R.tws_ref_water_brush.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_float, C.c_float,
                                              C.c_float, C.c_float]
            _ref = R
    return _ref


# --------------------------------------------------------------------------- scene

def terrain(seed: int, W: int, H: int, height_scale: float = 40.0, fill: float = 15.0):
    """Benchmark terrain b and initial depth d = max(0, fill - b), float32 (H, W)."""
    b = np.empty((H, W), np.float32)
    d = np.empty((H, W), np.float32)
    lib().tws_oracle_terrain(seed, W, H, height_scale, fill, _fp(b), _fp(d))
    return b, d


def rain_centers(seed: int, W: int, H: int, radius: int, count: int = 1):
    cx = np.empty(count, np.int32)
    cy = np.empty(count, np.int32)
    lib().tws_oracle_rain_centers(seed, W, H, radius, count, _fp(cx), _fp(cy))
    return [(int(a), int(b)) for a, b in zip(cx, cy)]


def pcg32(initstate: int, initseq: int, n: int, skip: int = 0) -> np.ndarray:
    out = np.empty(n, np.uint32)
    lib().tws_oracle_pcg32(initstate, initseq, skip, n, _fp(out))
    return out


def params_physical(dt=0.02, g=9.81, A=1.0, l=1.0, damping=0.998):
    """(Kf, Ka, C) in double for the benchmark parameterisation."""
    out = np.empty(3, np.float64)
    lib().tws_oracle_params_physical(dt, g, A, l, damping, _fp(out))
    return tuple(float(x) for x in out)


def params_reference(steps_per_second=60.0, damping=0.98, accel=10.0, world=1024.0, res=1024):
    """(Kf, Ka, C) as float32, derived the way Terrain.cpp:175-198 does."""
    out = np.empty(3, np.float32)
    lib().tws_oracle_params_reference(steps_per_second, damping, accel, world, res, _fp(out))
    return tuple(out.tolist())


def make_sources(specs):
    """specs: list of (kind, cx, cy, radius_or_sizesq, rate)."""
    arr = (Source * max(1, len(specs)))()
    for i, (kind, cx, cy, r, rate) in enumerate(specs):
        arr[i] = Source(kind, 0, cx, cy, r, rate)
    return arr, len(specs)


# --------------------------------------------------------------------------- step

def step_f32(b, d, f, v, kf, ka, c, boundary=BOUNDARY_CLOSED, sources=(), nsteps=1, threads=0,
             flux_scale=0.0):
    """Advance in place: b (H,W) f32, d (H,W) f32, f (H,W,4) f32, v (H,W,2) f32 or None.
    flux_scale > 0 models FP16 flux storage with that scale.
    Returns the elapsed seconds of the step loop."""
    H, W = b.shape
    for a in (b, d, f) + ((v,) if v is not None else ()):
        assert a.dtype == np.float32 and a.flags.c_contiguous
    src, n = make_sources(list(sources))
    return lib().tws_oracle_step_f32(W, H, np.float32(kf), np.float32(ka), np.float32(c),
                                     1 if boundary == BOUNDARY_CLOSED else 0, flux_scale,
                                     _fp(b), _fp(d), _fp(f), _fp(v) if v is not None else None,
                                     src, n, nsteps, threads)


def step_f64(b, d, f, v, kf, ka, c, boundary=BOUNDARY_CLOSED, sources=(), nsteps=1, threads=0):
    H, W = b.shape
    for a in (b, d, f) + ((v,) if v is not None else ()):
        assert a.dtype == np.float64 and a.flags.c_contiguous
    src, n = make_sources(list(sources))
    return lib().tws_oracle_step_f64(W, H, kf, ka, c, 1 if boundary == BOUNDARY_CLOSED else 0,
                                     _fp(b), _fp(d), _fp(f), _fp(v) if v is not None else None,
                                     src, n, nsteps, threads)


def quantize_f16(f, scale):
    """In place: the values an FP16-stored flux array reads back as."""
    assert f.dtype == np.float32 and f.flags.c_contiguous
    lib().tws_oracle_quantize_f16(_fp(f), f.size, scale)


def sources_f32(d, sources):
    H, W = d.shape
    src, n = make_sources(list(sources))
    lib().tws_oracle_sources_f32(W, H, _fp(d), src, n)


def volume(d, cell_area=1.0) -> float:
    d = np.ascontiguousarray(d)
    if d.dtype == np.float64:
        return lib().tws_oracle_volume_f64(_fp(d), d.size, cell_area)
    assert d.dtype == np.float32
    return lib().tws_oracle_volume_f32(_fp(d), d.size, cell_area)


def max_threads() -> int:
    return lib().tws_oracle_max_threads()


def surface(b, d, v):
    """The renderer's per-texel arithmetic (see tws_oracle_surface)."""
    H, W = b.shape
    out = {"height": np.empty((H, W), np.float32), "render_height": np.empty((H, W), np.float32),
           "normal": np.empty((H, W, 3), np.float32), "flow_speed": np.empty((H, W), np.float32),
           "foam": np.empty((H, W), np.float32), "dry": np.empty((H, W), np.uint8)}
    L = lib()
    L.tws_oracle_surface.argtypes = [C.c_int, C.c_int] + [C.c_void_p] * 9
    b, d, v = (np.ascontiguousarray(a, dtype=np.float32) for a in (b, d, v))
    L.tws_oracle_surface(W, H, _fp(b), _fp(d), _fp(v), *[_fp(out[k]) for k in
                         ("height", "render_height", "normal", "flow_speed", "foam", "dry")])
    return out


def terrain_mips(b, d, levels):
    """(RGBA32F TerrainData, [mip level 1..levels]) as the reference lays them out."""
    H, W = b.shape
    sizes, w, h = [], W, H
    for _ in range(levels):
        w, h = w // 2, h // 2
        sizes.append((h, w))
    rgba = np.empty((H, W, 4), np.float32)
    mips = np.empty(max(1, sum(4 * hh * ww for hh, ww in sizes)), np.float32)
    L = lib()
    L.tws_oracle_terrain_mips.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int,
                                          C.c_void_p, C.c_void_p]
    b, d = (np.ascontiguousarray(a, dtype=np.float32) for a in (b, d))
    L.tws_oracle_terrain_mips(W, H, _fp(b), _fp(d), levels, _fp(rgba), _fp(mips))
    out, off = [], 0
    for hh, ww in sizes:
        out.append(mips[off:off + 4 * hh * ww].reshape(hh, ww, 4))
        off += 4 * hh * ww
    return rgba, out


# --------------------------------------------------------------------------- reference run

def ref_steps(b, d, f, kf, ka, c, nsteps, brush=None):
    """Run the reference's own shaders (open-sink border, its native semantics)
    for nsteps: optional one-shot brush (x, y, intensity, size_sq) before the
    first step, then per step flowUpdate + flowApply.  Returns (d, f, flowmap
    as uint16 (H,W,2) halves)."""
    H, W = b.shape
    td = np.zeros((H, W, 4), np.float32)
    td[..., 0] = b
    td[..., 1] = 0.3
    td[..., 2] = 0.3
    td[..., 3] = d
    fl = np.ascontiguousarray(f, dtype=np.float32).copy()
    fm = np.zeros((H, W, 2), np.uint16)
    p = np.array([kf, ka, c], np.float32)
    R = ref()
    if brush is not None:
        R.tws_ref_water_brush(_fp(td), W, H, *[float(x) for x in brush])
    for _ in range(nsteps):
        R.tws_ref_flow_update(_fp(td), _fp(fl), W, H, _fp(p))
        R.tws_ref_flow_apply(_fp(td), _fp(fl), _fp(fm), W, H, _fp(p))
    return td[..., 3].copy(), fl, fm


# --------------------------------------------------------------------------- reference noise scene

REFERENCE_NOISE_SEED = 231656522  # Application.cpp:57
_REF_NOISE_PATH = os.path.join(HERE, "_ref", "libtws_ref_noise.so")
_ref_noise = None


def reference_noise_table(seed: int = REFERENCE_NOISE_SEED, generation: int = 0) -> np.ndarray:
    """The 4096-entry white-noise table of the reference's NoiseGenerator after
    Random::Init(seed) and `generation` earlier generators (the restatement)."""
    L = lib()
    L.tws_oracle_reference_noise_table.argtypes = [C.c_uint32, C.c_int, C.c_void_p]
    t = np.empty(4096, np.float32)
    L.tws_oracle_reference_noise_table(seed, generation, _fp(t))
    return t


def reference_terrain(W: int, H: int, height_scale: float = 300.0,
                      seed: int = REFERENCE_NOISE_SEED, generation: int = 0):
    """The reference's own scene (Terrain::CreateHeightmapFromNoiseAndResetSim),
    b and d float32 (H, W), from the restatement."""
    L = lib()
    L.tws_oracle_reference_terrain.argtypes = [C.c_uint32, C.c_int, C.c_int, C.c_int, C.c_float,
                                               C.c_void_p, C.c_void_p]
    b = np.empty((H, W), np.float32)
    d = np.empty((H, W), np.float32)
    L.tws_oracle_reference_terrain(seed, generation, W, H, height_scale, _fp(b), _fp(d))
    return b, d


def ref_noise_available() -> bool:
    return os.path.exists(_REF_NOISE_PATH)


def ref_noise():
    """The reference's own Random.cpp and NoiseGenerator.cpp, built by
    `make -C oracle ref` (square grids, as the reference)."""
    global _ref_noise
    with _lock:
        if _ref_noise is None:
            R = C.CDLL(_REF_NOISE_PATH)
            R.tws_ref_noise_table.argtypes = [C.c_uint, C.c_int, C.c_void_p]
            R.tws_ref_reference_terrain.argtypes = [C.c_uint, C.c_int, C.c_int, C.c_float,
                                                    C.c_void_p, C.c_void_p]
            _ref_noise = R
    return _ref_noise


# --------------------------------------------------------------------------- reference render shaders

_REF_RENDER_PATH = os.path.join(HERE, "_ref", "libtws_ref_render.so")
_ref_render = None


def ref_render_available() -> bool:
    return os.path.exists(_REF_RENDER_PATH)


def ref_render():
    """The parts of the reference's water-rendering shaders that read the
    simulation's textures (waterRender.vert, .eval's main(), .frag's
    ComputeHeightmapNormal and flow-speed lines), built by `make -C oracle
    ref` (see ref_glsl/render_emu.h)."""
    global _ref_render
    with _lock:
        if _ref_render is None:
            R = C.CDLL(_REF_RENDER_PATH)
            R.tws_ref_water_vert.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
            R.tws_ref_water_eval.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p]
            R.tws_ref_water_frag.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p,
                                             C.c_void_p, C.c_void_p]
            _ref_render = R
    return _ref_render


def ref_surface(b, d, flowmap_f16):
    """The reference's own shader code on a square grid's state: b, d (N, N)
    float32 and the RG16F flow map as (N, N, 2) uint16.  Returns the same keys
    as surface()."""
    H, W = b.shape
    assert H == W, "the fragment shader's texel size is one number: square grids"
    R = ref_render()
    rgba = np.empty((H, W, 4), np.float32)
    rgba[..., 0] = b
    rgba[..., 1] = 0.3
    rgba[..., 2] = 0.3
    rgba[..., 3] = d
    fm = np.ascontiguousarray(flowmap_f16, dtype=np.uint16)
    height = np.empty((H, W), np.float32)
    under = np.empty((H, W), np.int32)
    render = np.empty((H, W), np.float32)
    normal = np.empty((H, W, 3), np.float32)
    speed = np.empty((H, W), np.float32)
    foam = np.empty((H, W), np.float32)
    R.tws_ref_water_vert(_fp(rgba), W, H, _fp(height), _fp(under))
    R.tws_ref_water_eval(_fp(rgba), W, H, _fp(render))
    R.tws_ref_water_frag(_fp(rgba), _fp(fm), W, _fp(normal), _fp(speed), _fp(foam))
    return {"height": height, "render_height": render, "normal": normal, "flow_speed": speed,
            "foam": foam, "dry": under.astype(np.uint8)}
