"""Python binding of the serving loop (tws_server_* in include/tws.h).

The loop itself is native (terrainwatersim_gb300/csrc/tws_serve.cpp); this
module marshals requests and results.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

from . import FLUX_F16, SimParams, Source, TwsError, Grid, lib, MAX_SOURCES, TWS_OK


class ServerConfig(C.Structure):
    _fields_ = [("memory_budget_bytes", C.c_double), ("flux_storage", C.c_int),
                ("chain_steps", C.c_int), ("batch_variant", C.c_int), ("keep_grids", C.c_int)]


class Request(C.Structure):
    _fields_ = [("id", C.c_uint64), ("width", C.c_int), ("height", C.c_int),
                ("seed", C.c_uint64), ("height_scale", C.c_float), ("fill", C.c_float),
                ("params", SimParams), ("nsources", C.c_int),
                ("sources", Source * MAX_SOURCES), ("steps", C.c_int),
                ("arrival_s", C.c_double)]


class _Result(C.Structure):
    _fields_ = [("id", C.c_uint64), ("status", C.c_int), ("steps", C.c_int),
                ("arrival_s", C.c_double), ("admit_s", C.c_double), ("done_s", C.c_double),
                ("volume", C.c_double), ("grid", C.c_void_p)]


@dataclass
class Result:
    id: int
    status: int
    steps: int
    arrival_s: float
    admit_s: float
    done_s: float
    volume: float
    grid: object  # a Grid when keep_grids, else None

    @property
    def latency_s(self) -> float:
        return self.done_s - self.arrival_s


class _KeptGrid(Grid):
    """A finished grid handed back by the server (keep_grids)."""

    def __init__(self, handle, width, height, params, flux_storage):  # noqa: D401
        self._h = C.c_void_p(handle)
        self.width, self.height = width, height
        self.params = params
        self.flux_storage = flux_storage


def make_request(rid, width, height, seed, fill, params, sources, steps, arrival_s,
                 height_scale=40.0) -> Request:
    r = Request()
    r.id, r.width, r.height, r.seed = rid, width, height, seed
    r.height_scale, r.fill = height_scale, fill
    r.params = params
    srcs = list(sources)
    r.nsources = len(srcs)
    for k, s in enumerate(srcs):
        r.sources[k] = Source(*s)
    r.steps, r.arrival_s = steps, arrival_s
    return r


class Server:
    def __init__(self, memory_budget_bytes=120e9, flux_storage=FLUX_F16, chain_steps=0,
                 batch_variant=4, keep_grids=False):
        """chain_steps <= 0 sizes each chain to about 1.5e9 cell-steps.
        batch_variant: the batched kernel (default 4: two steps per launch on
        unified-layout 32x32 tiles, the library's default); -1 autotunes on
        the first chain."""
        self.cfg = ServerConfig(memory_budget_bytes, flux_storage, chain_steps, batch_variant,
                                1 if keep_grids else 0)
        h = C.c_void_p()
        code = lib().tws_server_create(C.byref(self.cfg), C.byref(h))
        if code != TWS_OK:
            raise TwsError(code, "tws_server_create")
        self._h = h
        self._requests = {}

    def close(self):
        if getattr(self, "_h", None):
            lib().tws_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def submit(self, request: Request):
        code = lib().tws_server_submit(self._h, C.byref(request))
        if code != TWS_OK:
            raise TwsError(code, "tws_server_submit")
        self._requests[request.id] = request

    def close_submissions(self):
        lib().tws_server_close(self._h)

    def run(self, serial: bool = False):
        code = lib().tws_server_run(self._h, 1 if serial else 0)
        if code != TWS_OK:
            raise TwsError(code, "tws_server_run")

    def results(self):
        out = []
        for i in range(lib().tws_server_result_count(self._h)):
            r = _Result()
            lib().tws_server_result(self._h, i, C.byref(r))
            grid = None
            if r.grid:
                req = self._requests.get(r.id)
                grid = _KeptGrid(r.grid, req.width, req.height, req.params, self.cfg.flux_storage)
            out.append(Result(r.id, r.status, r.steps, r.arrival_s, r.admit_s, r.done_s,
                              r.volume, grid))
        return out

    def stats(self):
        cs, sec, peak, ch = C.c_double(), C.c_double(), C.c_double(), C.c_uint64()
        lib().tws_server_stats(self._h, C.byref(cs), C.byref(sec), C.byref(peak), C.byref(ch))
        return {"cell_steps": cs.value, "seconds": sec.value, "peak_bytes": peak.value,
                "chains": ch.value}


def grid_bytes(width, height, flux_storage) -> float:
    return lib().tws_grid_bytes(width, height, flux_storage)
