"""terrainwatersim_gb300 -- GB300-native virtual-pipe shallow-water step.

Python binding (ctypes) of the C ABI in include/tws.h.  The computation runs
in libtws.so (hand-written sm_103a kernels); this module only marshals
arguments.  There is no CPU fallback: if libtws.so has not been built, or no
sm_103a GPU is present, the calls raise.

The names follow the reference's `Terrain` class
(terrainwatersim/source/scene/Terrain.h:15-153): a `Grid` is created from a
heightmap, advanced with `step`, given water with `apply_source` (the
reference's brush) or per-step `set_sources` (the benchmark's rain), and
exposes its depth / flux / flow-map buffers.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

import numpy as np

__all__ = [
    "TwsError", "SimParams", "Source", "Buffers", "Grid", "lib", "library_path",
    "params_physical", "params_reference", "rain_disks", "variants",
    "BOUNDARY_CLOSED", "BOUNDARY_OPEN", "FLUX_F32", "FLUX_F16", "SOURCE_DISK", "SOURCE_BRUSH",
    "MAX_SOURCES",
]

BOUNDARY_CLOSED = 0
BOUNDARY_OPEN = 1
FLUX_F32 = 0
FLUX_F16 = 1
SOURCE_DISK = 0
SOURCE_BRUSH = 1
MAX_SOURCES = 8

TWS_OK = 0
ERR_INVALID = -1
ERR_CUDA = -2
ERR_OOM = -3
ERR_TIMEOUT = -4
REFERENCE_NOISE_SEED = 231656522  # the seed the reference application uses
ERR_UNSUPPORTED = -5
ERR_BUSY = -6
ERR_TOO_LARGE = -7
VOLUME_NOALLOC_MAX_ROWS = 16384
VARIANT_RESIDENT = -2  # tws_autotune's answer when the resident kernel is fastest
RESIDENT_AUTO = -1     # tws_set_resident: the automatic cluster size

_PKG = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_PKG, "_build", "libtws.so")
_lock = threading.Lock()
_lib = None


class TwsError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"tws error {code}: {message}")
        self.code = code


class SimParams(C.Structure):
    _fields_ = [("flow_friction_per_step", C.c_float),
                ("water_acceleration_per_step", C.c_float),
                ("cell_area_inv_time_scaled", C.c_float),
                ("cell_area", C.c_float),
                ("boundary", C.c_int)]

    def as_tuple(self):
        return (self.flow_friction_per_step, self.water_acceleration_per_step,
                self.cell_area_inv_time_scaled)


class Source(C.Structure):
    _fields_ = [("kind", C.c_int), ("cx", C.c_float), ("cy", C.c_float),
                ("radius", C.c_float), ("rate", C.c_float)]


class SurfaceOut(C.Structure):
    _fields_ = [("height", C.c_void_p), ("render_height", C.c_void_p), ("normal", C.c_void_p),
                ("flow_speed", C.c_void_p), ("foam", C.c_void_p), ("dry", C.c_void_p)]


class Buffers(C.Structure):
    _fields_ = [("terrain", C.c_void_p), ("depth", C.c_void_p), ("flux", C.c_void_p),
                ("velocity", C.c_void_p), ("width", C.c_int), ("height", C.c_int),
                ("pitch", C.c_int), ("flux_storage", C.c_int), ("flux_scale", C.c_float)]


def library_path() -> str:
    return _LIB_PATH


def _declare(L):
    vp, i, f, d, u64 = C.c_void_p, C.c_int, C.c_float, C.c_double, C.c_uint64
    sig = {
        "tws_params_physical": ([d, d, d, d, d, i, vp], i),
        "tws_params_reference": ([f, f, f, f, C.c_uint, i, vp], i),
        "tws_create": ([i, i, vp, i, vp, vp], i),
        "tws_destroy": ([vp], i),
        "tws_upload": ([vp, vp, vp, vp], i),
        "tws_upload_device": ([vp, vp, vp, vp], i),
        "tws_generate_scene": ([vp, u64, f, f], i),
        "tws_generate_reference_scene": ([vp, C.c_uint32, i, f], i),
        "tws_scene_rain_disks": ([u64, i, i, i, f, i, vp], i),
        "tws_set_params": ([vp, vp], i),
        "tws_set_sources": ([vp, vp, i], i),
        "tws_apply_source": ([vp, vp], i),
        "tws_set_steps_per_launch": ([vp, i], i),
        "tws_variant_count": ([], i),
        "tws_variant_info": ([i, vp, vp, vp, vp, vp], i),
        "tws_variant_kind": ([i], i),
        "tws_variant_tail_rows": ([i], i),
        "tws_current_variant": ([vp, vp], i),
        "tws_set_variant": ([vp, i], i),
        "tws_set_wait_limit": ([vp, C.c_longlong], i),
        "tws_test_drop_tile_loads": ([vp, i], i),
        "tws_autotune": ([vp, i, vp], i),
        "tws_resident_fits": ([i, i, i], i),
        "tws_set_resident": ([vp, i], i),
        "tws_step": ([vp, i], i),
        "tws_volume": ([vp, vp], i),
        "tws_volume_noalloc": ([vp, i, i, i, d, vp, vp], i),
        "tws_download": ([vp, vp, vp, vp], i),
        "tws_download_terrain": ([vp, vp], i),
        "tws_upload_async": ([vp, vp, vp, vp], i),
        "tws_download_async": ([vp, vp, vp, vp], i),
        "tws_io_wait": ([vp], i),
        "tws_get_buffers": ([vp, vp], i),
        "tws_sync": ([vp], i),
        "tws_stream": ([vp], vp),
        "tws_error_string": ([i], C.c_char_p),
        "tws_last_error": ([vp], C.c_char_p),
        "tws_launch_count": ([], u64),
        "tws_batch_create": ([i, vp, vp], i),
        "tws_batch_destroy": ([vp], i),
        "tws_batch_add": ([vp, vp], i),
        "tws_batch_remove": ([vp, vp], i),
        "tws_batch_size": ([vp], i),
        "tws_batch_variant_count": ([], i),
        "tws_batch_variant_info": ([i, vp, vp, vp], i),
        "tws_batch_set_variant": ([vp, i], i),
        "tws_batch_autotune": ([vp, i, vp], i),
        "tws_batch_use_graphs": ([vp, i], i),
        "tws_batch_step": ([vp, i], i),
        "tws_batch_step_each": ([vp, vp, i], i),
        "tws_batch_sync": ([vp], i),
        "tws_batch_stream": ([vp], vp),
        "tws_batch_last_error": ([vp], C.c_char_p),
        "tws_batch_stats": ([vp, vp, vp], i),
        "tws_server_create": ([vp, vp], i),
        "tws_server_destroy": ([vp], i),
        "tws_server_submit": ([vp, vp], i),
        "tws_server_close": ([vp], i),
        "tws_server_run": ([vp, i], i),
        "tws_server_result_count": ([vp], i),
        "tws_server_result": ([vp, i, vp], i),
        "tws_server_stats": ([vp, vp, vp, vp, vp], i),
        "tws_grid_bytes": ([i, i, i], d),
        "tws_surface": ([vp, vp], i),
        "tws_export_textures": ([vp, vp, vp, i, vp], i),
        "tws_version": ([], C.c_char_p),
    }
    for name, (args, res) in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res


def lib():
    """Load libtws.so (built by terrainwatersim_gb300.build).  Raises if absent."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(_LIB_PATH):
                raise RuntimeError(
                    f"{_LIB_PATH} is missing: build it with "
                    "`python -c 'import __graft_entry__ as g; g.build()'` (there is no CPU fallback)")
            L = C.CDLL(_LIB_PATH)
            _declare(L)
            _lib = L
    return _lib


def _check(code: int, grid_handle=None):
    if code != TWS_OK:
        L = lib()
        msg = L.tws_last_error(grid_handle).decode() if grid_handle else ""
        raise TwsError(code, f"{L.tws_error_string(code).decode()}: {msg}")


def params_physical(dt=0.02, gravity=9.81, pipe_area=1.0, cell_size=1.0, damping_per_step=0.998,
                    boundary=BOUNDARY_CLOSED) -> SimParams:
    p = SimParams()
    _check(lib().tws_params_physical(dt, gravity, pipe_area, cell_size, damping_per_step, boundary,
                                     C.byref(p)))
    return p


def params_reference(steps_per_second=60.0, flow_damping=0.98, flow_acceleration=10.0,
                     grid_world_size=1024.0, grid_resolution=1024,
                     boundary=BOUNDARY_OPEN) -> SimParams:
    p = SimParams()
    _check(lib().tws_params_reference(steps_per_second, flow_damping, flow_acceleration,
                                      grid_world_size, grid_resolution, boundary, C.byref(p)))
    return p


def rain_disks(seed: int, width: int, height: int, radius: int, rate: float, count: int = 1):
    arr = (Source * max(1, count))()
    _check(lib().tws_scene_rain_disks(seed, width, height, radius, rate, count, arr))
    return [(s.kind, s.cx, s.cy, s.radius, s.rate) for s in arr[:count]]


VARIANT_TILE, VARIANT_STREAM, VARIANT_SWEEP = 0, 1, 2


def variants():
    """[(steps_per_launch, tile_x, tile_y, stages, shared_bytes, kind)] of the
    step kernel (kind: VARIANT_TILE, VARIANT_STREAM or VARIANT_SWEEP)."""
    L = lib()
    out = []
    for i in range(L.tws_variant_count()):
        k, tx, ty, st, sm = C.c_int(), C.c_int(), C.c_int(), C.c_int(), C.c_size_t()
        _check(L.tws_variant_info(i, C.byref(k), C.byref(tx), C.byref(ty), C.byref(st),
                                  C.byref(sm)))
        kind = L.tws_variant_kind(i)
        _check(min(kind, 0))
        out.append((k.value, tx.value, ty.value, st.value, sm.value, kind))
    return out


def variant_tail_rows(variant: int) -> int:
    """Rows of the short bands that end a sweep variant's work queue (0: all
    bands are tile_y rows)."""
    r = lib().tws_variant_tail_rows(variant)
    _check(min(r, 0))
    return int(r)


def resident_fits(width: int, height: int, flux_storage: int = FLUX_F32) -> int:
    """The resident kernel's automatic cluster size (CTAs) for a grid of this
    size on this device, or 0 if the grid does not fit it."""
    return int(lib().tws_resident_fits(width, height, flux_storage))


def _host_f32(a, shape):
    a = np.ascontiguousarray(a, dtype=np.float32)
    if a.shape != shape:
        raise ValueError(f"expected shape {shape}, got {a.shape}")
    return a


def _check_out_f32(a, shape):
    """An output array the library writes in place: no conversion allowed."""
    if not isinstance(a, np.ndarray) or a.dtype != np.float32 or not a.flags.c_contiguous \
            or not a.flags.writeable:
        raise ValueError("outputs must be writeable C-contiguous float32 numpy arrays")
    if a.shape != shape:
        raise ValueError(f"expected shape {shape}, got {a.shape}")


class Grid:
    """One simulated grid resident on the GPU (the simulation half of Terrain)."""

    def __init__(self, width: int, height: int, params: SimParams | None = None,
                 flux_storage: int = FLUX_F32, stream: int | None = None):
        self.width, self.height = int(width), int(height)
        self.params = params if params is not None else params_physical()
        self.flux_storage = flux_storage
        h = C.c_void_p()
        _check(lib().tws_create(self.width, self.height, C.byref(self.params), flux_storage,
                                C.c_void_p(stream) if stream else None, C.byref(h)))
        self._h = h
        self._io_refs = []  # host arrays of asynchronous copies not yet waited for

    # -- lifecycle
    def close(self):
        if getattr(self, "_h", None):
            lib().tws_destroy(self._h)  # waits for the asynchronous copies
            self._h = None
            self._io_refs = []

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    @property
    def stream(self) -> int:
        return lib().tws_stream(self._h) or 0

    # -- state
    def upload(self, terrain, depth=None, flux=None):
        H, W = self.height, self.width
        b = _host_f32(terrain, (H, W))
        d = _host_f32(depth, (H, W)) if depth is not None else None
        f = _host_f32(flux, (H, W, 4)) if flux is not None else None
        _check(lib().tws_upload(self._h, b.ctypes.data,
                                d.ctypes.data if d is not None else None,
                                f.ctypes.data if f is not None else None), self._h)

    def upload_async(self, terrain, depth=None, flux=None):
        """tws_upload_async: the state is replaced by these arrays before any
        step queued later; returns at once.  The arrays are kept referenced
        until io_wait/sync and must not change before then (pinned arrays,
        e.g. from torch's pin_memory, make the copy asynchronous)."""
        H, W = self.height, self.width
        b = _host_f32(terrain, (H, W))
        d = _host_f32(depth, (H, W)) if depth is not None else None
        f = _host_f32(flux, (H, W, 4)) if flux is not None else None
        _check(lib().tws_upload_async(self._h, b.ctypes.data,
                                      d.ctypes.data if d is not None else None,
                                      f.ctypes.data if f is not None else None), self._h)
        self._io_refs.append((b, d, f))

    def download_async(self, out):
        """tws_download_async into the preallocated (d, f, v) float32 arrays
        (any may be None): the state after every step queued so far.  The
        arrays hold it once io_wait/sync returns."""
        H, W = self.height, self.width
        d, f, v = out
        shapes = ((H, W), (H, W, 4), (H, W, 2))
        for a, shape in zip(out, shapes):
            if a is not None:
                _check_out_f32(a, shape)
        _check(lib().tws_download_async(self._h, d.ctypes.data if d is not None else None,
                                        f.ctypes.data if f is not None else None,
                                        v.ctypes.data if v is not None else None), self._h)
        self._io_refs.append((d, f, v))

    def io_wait(self):
        """Block until every asynchronous upload and download has completed."""
        _check(lib().tws_io_wait(self._h), self._h)
        self._io_refs = []

    def upload_device(self, terrain_ptr: int, depth_ptr: int | None = None,
                      flux_ptr: int | None = None):
        _check(lib().tws_upload_device(self._h, terrain_ptr, depth_ptr, flux_ptr), self._h)

    def generate_scene(self, seed: int, height_scale: float = 40.0, fill: float = 15.0):
        _check(lib().tws_generate_scene(self._h, seed, height_scale, fill), self._h)

    def generate_reference_scene(self, seed: int = REFERENCE_NOISE_SEED, generation: int = 0,
                                 height_scale: float = 300.0):
        """The reference's own noise terrain and central pool
        (Terrain::CreateHeightmapFromNoiseAndResetSim)."""
        _check(lib().tws_generate_reference_scene(self._h, seed, generation, height_scale),
               self._h)

    def set_params(self, params: SimParams):
        _check(lib().tws_set_params(self._h, C.byref(params)), self._h)
        self.params = params

    def set_sources(self, sources):
        srcs = list(sources)
        arr = (Source * max(1, len(srcs)))()
        for k, s in enumerate(srcs):
            arr[k] = Source(*s)
        _check(lib().tws_set_sources(self._h, arr, len(srcs)), self._h)

    def apply_source(self, source):
        s = Source(*source)
        _check(lib().tws_apply_source(self._h, C.byref(s)), self._h)

    def set_steps_per_launch(self, k: int):
        _check(lib().tws_set_steps_per_launch(self._h, k), self._h)

    def set_variant(self, variant: int):
        _check(lib().tws_set_variant(self._h, variant), self._h)

    def current_variant(self) -> int:
        """The variant tws_step launches for this grid now (tws_current_variant)."""
        v = C.c_int()
        _check(lib().tws_current_variant(self._h, C.byref(v)), self._h)
        return v.value

    def set_wait_limit(self, sm_cycles: int):
        """SM clocks a tile-load wait may take before the kernel gives up
        (0: the default)."""
        _check(lib().tws_set_wait_limit(self._h, sm_cycles), self._h)

    def test_drop_tile_loads(self, drop: bool = True):
        """Test hook (tws_testing.h): every tile load arms its barrier but
        issues no copy, so its bounded wait runs out with nothing in flight
        (False turns it off)."""
        _check(lib().tws_test_drop_tile_loads(self._h, 1 if drop else 0), self._h)

    def set_resident(self, on: bool = True, ctas: int | None = None):
        """Run the steps with the resident kernel (the whole grid in one
        cluster's shared memory), on `ctas` CTAs (1, 2, 4, 8 or 16; None:
        the automatic size); raises if the grid does not fit it."""
        mode = 0 if not on else (RESIDENT_AUTO if ctas is None else int(ctas))
        _check(lib().tws_set_resident(self._h, mode), self._h)

    def autotune(self, trial_steps: int = 24) -> int:
        """Time every kernel variant (and the resident kernel, where the grid
        fits it) on this grid's state (restored after) and use the fastest;
        returns its index, or VARIANT_RESIDENT."""
        out = C.c_int()
        _check(lib().tws_autotune(self._h, trial_steps, C.byref(out)), self._h)
        return out.value

    def step(self, nsteps: int = 1):
        _check(lib().tws_step(self._h, nsteps), self._h)

    def volume(self) -> float:
        out = C.c_double()
        _check(lib().tws_volume(self._h, C.byref(out)), self._h)
        return out.value

    def sync(self):
        _check(lib().tws_sync(self._h), self._h)
        self._io_refs = []

    def download(self, depth=True, flux=True, velocity=True, out=None):
        """Return (d, f, v) as float32 host arrays (None where not requested).
        `out` may supply preallocated (d, f, v) arrays."""
        H, W = self.height, self.width
        if out is not None:
            d, f, v = out
        else:
            d = np.empty((H, W), np.float32) if depth else None
            f = np.empty((H, W, 4), np.float32) if flux else None
            v = np.empty((H, W, 2), np.float32) if velocity else None
        _check(lib().tws_download(self._h, d.ctypes.data if d is not None else None,
                                  f.ctypes.data if f is not None else None,
                                  v.ctypes.data if v is not None else None), self._h)
        return d, f, v

    def surface(self, out: "SurfaceOut"):
        """The renderer's per-texel outputs into caller-owned device buffers."""
        _check(lib().tws_surface(self._h, C.byref(out)), self._h)

    def export_textures(self, terrain_rgba_ptr, flowmap_ptr, mip_levels=0, mips_ptr=None):
        """The reference's RGBA32F TerrainData (+ mips) and RG16F FlowMap into
        caller-owned device buffers."""
        _check(lib().tws_export_textures(self._h, terrain_rgba_ptr, flowmap_ptr, mip_levels,
                                         mips_ptr), self._h)

    def download_terrain(self):
        b = np.empty((self.height, self.width), np.float32)
        _check(lib().tws_download_terrain(self._h, b.ctypes.data), self._h)
        return b

    def buffers(self) -> Buffers:
        out = Buffers()
        _check(lib().tws_get_buffers(self._h, C.byref(out)), self._h)
        return out


def batch_variants():
    """[(steps_per_launch, tile_x, tile_y)] of the batched kernel."""
    L = lib()
    out = []
    for i in range(L.tws_batch_variant_count()):
        k, tx, ty = C.c_int(), C.c_int(), C.c_int()
        _check(L.tws_batch_variant_info(i, C.byref(k), C.byref(tx), C.byref(ty)))
        out.append((k.value, tx.value, ty.value))
    return out


class Batch:
    """Many grids advanced together by one persistent launch per step, chains
    of 16 steps replayed from CUDA graphs (tws_batch_* in include/tws.h)."""

    def __init__(self, flux_storage: int = FLUX_F32, stream: int | None = None):
        h = C.c_void_p()
        _check(lib().tws_batch_create(flux_storage, C.c_void_p(stream) if stream else None,
                                      C.byref(h)))
        self._h = h
        self.grids = []

    def _check(self, code):
        if code != TWS_OK:
            L = lib()
            raise TwsError(code, f"{L.tws_error_string(code).decode()}: "
                                 f"{L.tws_batch_last_error(self._h).decode()}")

    def close(self):
        if getattr(self, "_h", None):
            lib().tws_batch_destroy(self._h)
            self._h = None
            self.grids = []

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self) -> int:
        return lib().tws_batch_stream(self._h) or 0

    def add(self, grid: Grid):
        self._check(lib().tws_batch_add(self._h, grid.handle))
        self.grids.append(grid)

    def remove(self, grid: Grid):
        self._check(lib().tws_batch_remove(self._h, grid.handle))
        self.grids.remove(grid)

    def __len__(self):
        return lib().tws_batch_size(self._h)

    def set_variant(self, variant: int):
        self._check(lib().tws_batch_set_variant(self._h, variant))

    def use_graphs(self, enable: bool):
        self._check(lib().tws_batch_use_graphs(self._h, 1 if enable else 0))

    def autotune(self, trial_steps: int = 32) -> int:
        out = C.c_int()
        self._check(lib().tws_batch_autotune(self._h, trial_steps, C.byref(out)))
        return out.value

    def step(self, nsteps: int):
        self._check(lib().tws_batch_step(self._h, nsteps))

    def step_each(self, nsteps):
        arr = (C.c_int * max(1, len(nsteps)))(*[int(n) for n in nsteps])
        self._check(lib().tws_batch_step_each(self._h, arr, len(nsteps)))

    def sync(self):
        self._check(lib().tws_batch_sync(self._h))

    def stats(self):
        a, b = C.c_uint64(), C.c_uint64()
        self._check(lib().tws_batch_stats(self._h, C.byref(a), C.byref(b)))
        return a.value, b.value
