"""Benchmark of the GB300 virtual-pipe shallow-water step.

Workload (the single-GPU configuration the headline metric is quoted on):
one 4096 x 4096 FP32 grid, seeded PCG32 fBm terrain scaled to 0-40 m, initial
depth max(0, 15 - b), closed walls, l = 1 m, A = 1 m^2, g = 9.81, dt = 0.02 s,
damping 0.998 per step, one rain disk of radius 64 cells adding 0.01 m per
step.  A benchmark "step" is a chain of `--chain` simulation steps (default
200, so the default 50 timed steps make the configuration's 10,000 steps).

Printed JSON line (rank 0):
  value          Gcell-steps/s with the state resident in HBM (all ranks)
  e2e            same metric through the C ABI with host buffers: per bench
                 step, upload b/d/f from pinned host memory, the chain of steps,
                 download d/f/v to pinned host memory; `value` pipelined (the
                 asynchronous calls), `serial_value` with the synchronous ones
  roofline       the step kernel: algorithmic bytes (52 B per cell-step for
                 FP32 state) per launch / measured launch time, against the
                 measured HBM copy bandwidth
  cpu_baseline   the FP32 oracle (a CPU port of the reference shaders) on the
                 host cores, bounded sample of the same grid; its state is
                 compared with the GPU's for the same steps (full grid)
  plain/blocked  the plain kernel (1 step per launch) and the temporally
                 blocked kernel, both timed
  batched_vs_plain  64 uneven grids (2000 steps) in one batched launch per
                 step against the plain kernel one grid at a time, with FP64
                 checks on 4 sampled grids
  serving        the serving loop on the first --serving-requests requests of
                 the seeded Poisson stream: time-to-completion p50/p95/p99 and
                 aggregate rate against serial plain-kernel execution, at 70%
                 load and saturated
--impl reference times the CPU port of the reference's path on the host cores
(the reference itself is an OpenGL program that cannot run on this machine).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

W_DEFAULT = 4096
BYTES_PER_CELL_STEP_F32 = 52.0   # read b 4 + d 4 + f 16, write d 4 + f 16 + v 8
BYTES_PER_CELL_STEP_F16 = 36.0
METRIC = "Gcell-steps/s and % of HBM peak, batched vs plain at same error; p50/p99 latency"
L2_BYTES = 129e6


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--size", type=int, default=W_DEFAULT)
    ap.add_argument("--chain", type=int, default=200, help="simulation steps per bench step")
    ap.add_argument("--variant", type=int, default=-1,
                    help="kernel variant for the headline (-1: the library's autotuner picks)")
    ap.add_argument("--no-sweep", action="store_true", help="do not time every kernel variant")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end leg")
    ap.add_argument("--flux", choices=["f32", "f16"], default="f32")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-renderer", action="store_true",
                    help="skip timing the renderer-facing outputs")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--config", choices=["c1", "c2", "c3", "c4", "c5"], default="c2",
                    help="c2 (default): the 4096^2 headline; c1: 256^2; c3: 64 uneven grids "
                         "batched; c4: 16384^2 FP16 flux; c5: serving loop")
    ap.add_argument("--requests", type=int, default=2000, help="c5: requests in the stream")
    ap.add_argument("--max-steps", type=int, default=20000, help="c5: largest step count")
    ap.add_argument("--no-batched", action="store_true",
                    help="skip the batched-vs-plain leg (the 64-grid configuration)")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving leg")
    ap.add_argument("--c4-window-steps", type=int, default=1600,
                    help="c4: steps before the 1024^2 window is compared with the FP64 oracle")
    ap.add_argument("--serving-requests", type=int, default=300,
                    help="serving leg of the default run: the first N requests of the stream")
    return ap.parse_args()


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            p = json.load(fh)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def ncu_traffic_per_cell(k: int, flux: str, variant: int | None = None):
    """DRAM bytes per cell per launch of the step kernel from the committed ncu
    summary (profiles/step_kernel_traffic.txt): the line of this variant, else
    of the same temporal depth and flux storage; None if there is none."""
    path = os.path.join(ROOT, "profiles", "step_kernel_traffic.txt")
    if not os.path.exists(path):
        return None
    by_k = None
    for line in open(path):
        if line.startswith("#") or "=" not in line:
            continue
        kv = dict(tok.split("=", 1) for tok in line.split() if "=" in tok)
        try:
            if int(kv["k"]) != k or kv.get("flux", "f32") != flux:
                continue
            per_cell = float(kv["dram_bytes_per_launch"]) / float(kv["cells"])
            if variant is not None and int(kv.get("variant", -1)) == variant:
                return per_cell
            by_k = per_cell if by_k is None else by_k
        except (KeyError, ValueError):
            continue
    return by_k


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        # nvidia-smi numbers GPUs physically; map through CUDA_VISIBLE_DEVICES
        vis = [v.strip() for v in os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",") if v.strip()]
        self.index = vis[index] if index < len(vis) else str(index)
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        time.sleep(0.25)
        self.rows = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            for line in out.strip().splitlines():
                parts = [p.strip() for p in line.split(",")]
                if len(parts) == 8:
                    self.rows.append(parts)

    def summary(self):
        if not getattr(self, "rows", None):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(r[0]) for r in self.rows if num(r[0])]
        smax = [num(r[1]) for r in self.rows if num(r[1])]
        pw = [num(r[2]) for r in self.rows if num(r[2])]
        loaded = [s for s in sm if smax and s > 0.5 * max(smax)] or sm
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4)
                          if r[4 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(loaded) if loaded else None,
                "sm_max_mhz": max(smax) if smax else None,
                "power_w_max": max(pw) if pw else None,
                "samples": len(self.rows), "reasons": reasons}


# ------------------------------------------------------------------ distributed

def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def dist_init(ws, local):
    import torch
    import torch.distributed as dist
    torch.cuda.set_device(local)
    if ws > 1 and not dist.is_initialized():
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    return dist if ws > 1 else None


def barrier(dist):
    import torch
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, x: float, device: str = "cuda") -> float:
    """The slowest rank's time: the whole job is done when the last replica is."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_gcell_steps(cells: int, sim_steps: int, world_size: int, seconds: float) -> float:
    """Whole-job throughput: every rank advances its own replica of the grid
    (weak scaling), so the work is world_size x cells x steps over the
    slowest rank's time."""
    return float(cells) * sim_steps * world_size / seconds / 1e9


# ------------------------------------------------------------------ our arm

def variant_form(v, tail=0):
    """How a variant runs: one CTA per tile, persistent CTAs, register
    streaming, or a row sweep (with its rows per loop trip and the height of
    the short bands that end its queue)."""
    kind = v[5] if len(v) > 5 else 0
    if kind == 1:
        return "stream"
    if kind == 2:
        return f"sweep_u{v[3]}" + (f"_tail{tail}" if tail else "")
    return "persistent" if v[3] > 1 else "pertile"


def kernel_name(v):
    kind = v[5] if len(v) > 5 else 0
    return {1: "stream_kernel", 2: "sweep_kernel"}.get(kind, "step_kernel")


def kernel_label(v, tail=0):
    """e.g. sweep_kernel<K=3,52x256,tail 64> or step_kernel<K=2,32x32>."""
    return (f"{kernel_name(v)}<K={v[0]},{v[1]}x{v[2]}" + (f",tail {tail}" if tail else "")
            + ">")


def scene(tws, size):
    p = tws.params_physical(0.02, 9.81, 1.0, 1.0, 0.998, tws.BOUNDARY_CLOSED)
    rain = tws.rain_disks(2026, size, size, 64, 0.01, 1)
    return p, rain


def time_device(tws, torch, g, stream, variant, chain, steps, warmup, dist):
    """Timed region with the state resident in HBM.  Returns (seconds,
    per-bench-step ms list, launches)."""
    g.set_variant(variant)
    for _ in range(warmup):
        g.step(chain)
    barrier(dist)
    g.sync()
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
    L0 = tws.lib().tws_launch_count()
    evs[0].record(stream)
    for i in range(steps):
        g.step(chain)
        evs[i + 1].record(stream)
    torch.cuda.synchronize()
    launches = tws.lib().tws_launch_count() - L0
    per = [evs[i].elapsed_time(evs[i + 1]) for i in range(steps)]
    total = evs[0].elapsed_time(evs[steps]) / 1e3
    g.sync()
    return total, per, launches


def run_ours(args):
    import torch

    import terrainwatersim_gb300 as tws

    ws, rank, local = dist_env()
    dist = dist_init(ws, local)
    size, chain, steps, warmup = args.size, args.chain, args.steps, max(3, args.warmup)
    flux = tws.FLUX_F16 if args.flux == "f16" else tws.FLUX_F32
    bpc = BYTES_PER_CELL_STEP_F16 if args.flux == "f16" else BYTES_PER_CELL_STEP_F32
    cells = size * size
    peak, peak_kind = measured_peaks()
    p, rain = scene(tws, size)
    stream = torch.cuda.Stream()
    g = tws.Grid(size, size, p, flux, stream=stream.cuda_stream)
    g.generate_scene(2026, 40.0, 15.0)
    g.set_sources(rain)
    state_bytes = cells * (4 + 2 * 4 + 2 * (16 if flux == tws.FLUX_F32 else 8) + 8)

    # every kernel variant (plain and temporally blocked, several tiles), same workload
    vinfo = tws.variants()
    tails = [tws.variant_tail_rows(i) for i in range(len(vinfo))]
    variants = {}
    if not args.no_sweep:
        sweep_steps = max(3, steps // 5)
        for vi in range(len(vinfo)):
            g.generate_scene(2026, 40.0, 15.0)
            t, _, n = time_device(tws, torch, g, stream, vi, chain, sweep_steps, warmup, dist)
            variants[vi] = dict(seconds=max_over_ranks(dist, t), launches=n, steps=sweep_steps)
    # the library's autotuner picks the headline kernel on the workload's state
    g.generate_scene(2026, 40.0, 15.0)
    tuned = g.autotune(24) if args.variant < 0 else None
    best_v = tuned if args.variant < 0 else args.variant
    best_k = vinfo[best_v][0]

    # headline run of the chosen kernel with clocks sampled during it
    g.generate_scene(2026, 40.0, 15.0)
    with ClockSampler(local) as cs:
        total, per, launches = time_device(tws, torch, g, stream, best_v, chain, steps, warmup, dist)
    total = max_over_ranks(dist, total)
    clocks = cs.summary()
    value = aggregate_gcell_steps(cells, chain * steps, ws, total)
    launch_s = total / max(1, launches)  # only step kernels run in the timed region
    cell_steps_per_launch = cells * best_k
    # Compulsory HBM bytes of one launch: the state is read once and written
    # once whatever the launch's temporal depth K (52 B per cell for FP32
    # flux, 36 B for FP16).  The K-scaled "effective" rate is reported beside it.
    compulsory = bpc * cells
    achieved = compulsory / launch_s / 1e9
    effective = bpc * cell_steps_per_launch / launch_s / 1e9
    tpc = ncu_traffic_per_cell(best_k, args.flux, best_v)
    plain = variants.get(0)
    if plain is None:  # no sweep: time the plain kernel alone for its top-level keys
        g.generate_scene(2026, 40.0, 15.0)
        t, _, n = time_device(tws, torch, g, stream, 0, chain, max(3, steps // 5), warmup, dist)
        plain = dict(seconds=max_over_ranks(dist, t), launches=n, steps=max(3, steps // 5))
    plain_launch_s = plain["seconds"] / max(1, plain["launches"])
    plain_value = cells * chain * plain["steps"] * ws / plain["seconds"] / 1e9
    plain_gbs = bpc * cells / plain_launch_s / 1e9

    # end to end through the C ABI with pinned host buffers
    hb = torch.empty((size, size), dtype=torch.float32, pin_memory=True).numpy()
    hd = torch.empty((size, size), dtype=torch.float32, pin_memory=True).numpy()
    hf = torch.zeros((size, size, 4), dtype=torch.float32, pin_memory=True).numpy()
    od = torch.empty((size, size), dtype=torch.float32, pin_memory=True).numpy()
    of = torch.empty((size, size, 4), dtype=torch.float32, pin_memory=True).numpy()
    ov = torch.empty((size, size, 2), dtype=torch.float32, pin_memory=True).numpy()
    g.generate_scene(2026, 40.0, 15.0)
    hb[...] = g.download_terrain()
    g.download(out=(hd, None, None), flux=False, velocity=False)
    g.set_variant(best_v)
    e2e_steps = steps  # the same K bench steps as the headline, each with its copies
    e2e_value = e2e_serial = None
    if not args.no_e2e:
        # pipelined: each bench step queues its upload, its chain and its
        # download without a host wait, so the copies of one bench step
        # overlap the chain of the next (tws_upload_async/tws_download_async)
        for _ in range(2):
            g.upload_async(hb, hd, hf)
            g.step(chain)
            g.download_async((od, of, ov))
        g.io_wait()
        torch.cuda.synchronize()
        barrier(dist)
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            g.upload_async(hb, hd, hf)
            g.step(chain)
            g.download_async((od, of, ov))
        g.io_wait()
        torch.cuda.synchronize()
        e2e_s = max_over_ranks(dist, time.perf_counter() - t0)
        e2e_value = float(cells) * chain * e2e_steps * ws / e2e_s / 1e9
        # serial: the synchronous calls, each bench step waiting for its copies
        for _ in range(2):
            g.upload(hb, hd, hf)
            g.step(chain)
            g.download(out=(od, of, ov))
        barrier(dist)
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            g.upload(hb, hd, hf)
            g.step(chain)
            g.download(out=(od, of, ov))
        torch.cuda.synchronize()
        e2e_s = max_over_ranks(dist, time.perf_counter() - t0)
        e2e_serial = float(cells) * chain * e2e_steps * ws / e2e_s / 1e9

    result = None
    if rank == 0:
        per_sorted = sorted(per)
        result = {
            "metric": METRIC,
            "value": round(value, 3),
            "unit": "Gcell-steps/s",
            "n_gpus": ws,
            "steps": steps,
            "warmup": warmup,
            "ms_per_step": round(total / steps * 1e3, 4),
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f32" if flux == tws.FLUX_F32 else "f32 (f16 flux storage)",
            "data": "synthetic: seeded PCG32 fBm terrain 0-40 m, fill 15 m, rain disk r=64",
            "config": {
                "workload": f"{size}x{size} FP32 virtual-pipe grid, closed walls, rain r=64, "
                            f"{chain} simulation steps per bench step "
                            f"({chain * steps} timed steps)",
                "grid": [size, size],
                "sim_steps_per_bench_step": chain,
                "steps_per_launch": best_k,
                "variant": best_v,
                "tile": [vinfo[best_v][1], vinfo[best_v][2]],
                "flux_storage": args.flux,
                "l2": (f"state {state_bytes / 1e6:.0f} MB > L2 {L2_BYTES / 1e6:.0f} MB, no flush"
                       if state_bytes > L2_BYTES else
                       f"state {state_bytes / 1e6:.0f} MB fits the {L2_BYTES / 1e6:.0f} MB L2 "
                       "(no flush; the default 4096^2 workload does not fit)"),
                "parallelism": "replicas (one whole grid per GPU)" if ws > 1 else "single grid",
            },
            "hbm_frac_of_measured": round(achieved / peak, 4),
            "hbm_frac_of_8tbs_nominal": round(achieved / 8000.0, 4),
            "plain_gcell_steps_per_s": round(plain_value, 3),
            "plain_hbm_gbs": round(plain_gbs, 1),
            "plain_hbm_frac_of_measured": round(plain_gbs / peak, 4),
            "plain_kernel": "step_kernel<K=1,32x32> (variant 0): one step per launch, "
                            f"{bpc:.0f} B per cell-step compulsory",
            "p50_ms": round(per_sorted[len(per) // 2], 4),
            "p99_ms": round(per_sorted[min(len(per) - 1, int(0.99 * len(per)))], 4),
            "p50_p99_note": "per bench step (a chain of simulation steps) on the resident grid; "
                            "request time-to-completion percentiles are under 'serving'",
            "roofline": {
                "bound": "hbm",
                "achieved": round(achieved, 1),
                "peak": peak,
                "unit": "GB/s",
                "frac": round(achieved / peak, 4),
                "peak_kind": peak_kind,
                "algorithmic_bytes_per_launch": compulsory,
                "algorithmic_bytes_note": f"{bpc:.0f} B per cell x {cells} cells: the state read "
                                          f"and written once per launch (K = {best_k} steps "
                                          "per launch)",
                "effective_gbs": round(effective, 1),
                "effective_note": f"{bpc:.0f} B per cell-step x K cell-steps per cell per "
                                  "launch / launch time (an un-blocked kernel's traffic for the "
                                  "same work, not bytes moved)",
                "launch_us": round(launch_s * 1e6, 2),
                "traffic": round(tpc * cells, 0) if tpc else None,
                "dram_gbs": round(tpc * cells / launch_s / 1e9, 1) if tpc else None,
                "kernel": kernel_label(vinfo[best_v], tails[best_v]),
            },
            "roofline_by_kernel": {
                (f"{i}_{kernel_name(vinfo[i])}_k{vinfo[i][0]}_{vinfo[i][1]}x{vinfo[i][2]}"
                 + (f"_tail{tails[i]}" if tails[i] else "")): {
                    "launch_us": round(v["seconds"] / max(1, v["launches"]) * 1e6, 2),
                    "frac": round(bpc * cells / (v["seconds"] / max(1, v["launches"])) / 1e9
                                  / peak, 4),
                } for i, v in variants.items() if i in (0, 16, best_v)},
            "roofline_note": "frac = compulsory bytes (the state in and out once) per launch / "
                             "launch time / measured copy rate; a kernel advancing K steps per "
                             "launch moves the state once for K steps, so a faster deep kernel "
                             "can show a lower frac (the K = 3 sweep is bound by instruction "
                             "latency, not HBM: profiles/sweep_kernel_k3_40rows_4096.md)",
            "variants": {
                (f"{i}_{'plain' if vinfo[i][0] == 1 else 'blocked_k%d' % vinfo[i][0]}"
                 f"_{vinfo[i][1]}x{vinfo[i][2]}_{variant_form(vinfo[i], tails[i])}"): {
                    "variant": i,
                    "gcell_steps_per_s": round(cells * chain * v["steps"] * ws / v["seconds"] / 1e9,
                                               3),
                    "launch_us": round(v["seconds"] / max(1, v["launches"]) * 1e6, 2),
                    "effective_gbs": round(bpc * cells * vinfo[i][0]
                                           / (v["seconds"] / max(1, v["launches"])) / 1e9, 1),
                } for i, v in variants.items()},
            "autotuned_variant": tuned,
            "e2e": None if e2e_value is None else {
                "value": round(e2e_value, 3),
                "unit": "Gcell-steps/s",
                "h2d_bytes_per_step": int(hb.nbytes + hd.nbytes + hf.nbytes),
                "d2h_bytes_per_step": int(od.nbytes + of.nbytes + ov.nbytes),
                "steps": e2e_steps,
                "mode": "pipelined: the copies of one bench step overlap the chain of the "
                        "next (tws_upload_async, tws_download_async, tws_io_wait)",
                "serial_value": round(e2e_serial, 3),
                "serial_mode": "tws_upload, tws_step, tws_download: each bench step waits "
                               "for its own copies",
            },
            "gpu_launches": int(launches),
            "clocks": clocks,
        }
        if not args.no_renderer:
            result["renderer"] = renderer_leg(tws, torch, g, stream, size, peak)
        if ws == 1 and not args.no_cpu:
            result["cpu_baseline"] = cpu_baseline_leg(tws, g, size, args.cpu_seconds)
    g.close()
    if rank == 0 and ws == 1:
        # the metric's comparisons, measured in the same run: many grids batched
        # against the plain kernel one grid at a time, and the serving loop's
        # time-to-completion percentiles against serial plain execution
        if not args.no_batched:
            torch.cuda.empty_cache()
            result["batched_vs_plain"] = run_c3(args)
            result["batched_vs_plain_ratio"] = result["batched_vs_plain"][
                "speedup_vs_one_grid_at_a_time"]
        if not args.no_serving:
            torch.cuda.empty_cache()
            sv = serving_leg(args.serving_requests, args.max_steps, C5_ARMS_DEFAULT)
            result["serving"] = sv
            arm = sv.get("served_fp16_batched", {})
            result["serving_latency_s"] = {k: arm.get("latency_s_" + k)
                                           for k in ("p50", "p95", "p99")}
            result["serving_vs_serial_plain"] = {"at_70pct_load": sv.get("aggregate_speedup"),
                                                 "saturated": sv.get("saturated_speedup")}
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()
    return result


# Algorithmic bytes per cell of the renderer-facing calls.
#   surface: read b, d, v (16); write height, render height, flow speed, foam
#            (4 each), normal (12), dry mask (1)
#   export:  flow map (read v 8, write 2 halves 4) + TerrainData RGBA32F (read b, d 8,
#            write 16); its mip pyramid adds the write of every level l >= 1,
#            16 / 4^l bytes per cell each: 16/3 in all (the reads of the
#            intermediate levels that build the next are not counted)
SURFACE_BYTES_PER_CELL = 45.0
EXPORT_BYTES_PER_CELL = 36.0
MIPS_BYTES_PER_CELL = 16.0 / 3.0


def renderer_leg(tws, torch, g, stream, size, peak):
    """The renderer-facing outputs on the benchmark grid's state: tws_surface and
    tws_export_textures (with and without the full mip pyramid), each timed with
    CUDA events on the grid's stream over 20 calls after 3 warm-up calls.  Their
    inputs (268 MB) and outputs exceed the L2."""
    cells = size * size
    dev = torch.device("cuda")
    f32 = lambda n: torch.empty(n, dtype=torch.float32, device=dev)  # noqa: E731
    height, rheight, speed, foam = f32(cells), f32(cells), f32(cells), f32(cells)
    normal = f32(3 * cells)
    dry = torch.empty(cells, dtype=torch.uint8, device=dev)
    so = tws.SurfaceOut(height.data_ptr(), rheight.data_ptr(), normal.data_ptr(),
                        speed.data_ptr(), foam.data_ptr(), dry.data_ptr())
    rgba = f32(4 * cells)
    flowmap = torch.empty(2 * cells, dtype=torch.int16, device=dev)
    levels, texels, w = 0, 0, size
    while w >= 2:
        w //= 2
        levels += 1
        texels += w * w
    mips = f32(4 * texels)

    def timed(fn, reps=20, warm=3):
        for _ in range(warm):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 1e3 / reps

    def entry(seconds, bpc):
        gbs = bpc * cells / seconds / 1e9
        return {"us": round(seconds * 1e6, 2), "bytes_per_cell": round(bpc, 2),
                "gbs": round(gbs, 1), "frac_of_measured_hbm": round(gbs / peak, 4)}

    t_surface = timed(lambda: g.surface(so))
    t_export = timed(lambda: g.export_textures(rgba.data_ptr(), flowmap.data_ptr(), 0, None))
    t_mips = timed(lambda: g.export_textures(rgba.data_ptr(), flowmap.data_ptr(), levels,
                                             mips.data_ptr()))
    return {
        "grid": [size, size],
        "surface": entry(t_surface, SURFACE_BYTES_PER_CELL),
        "export": entry(t_export, EXPORT_BYTES_PER_CELL),
        "export_with_mips": dict(entry(t_mips, EXPORT_BYTES_PER_CELL + MIPS_BYTES_PER_CELL),
                                 mip_levels=levels),
    }


def cpu_baseline_leg(tws, g, size, budget_s):
    """The FP32 oracle on the host cores, bounded sample of the same grid; the
    GPU's state after the same steps is compared with it on the full grid."""
    from oracle import oracle as O

    p, rain = scene(tws, size)
    b, d = O.terrain(2026, size, size, 40.0, 15.0)
    f = np.zeros((size, size, 4), np.float32)
    v = np.zeros((size, size, 2), np.float32)
    src = [(s[0], s[1], s[2], s[3], s[4]) for s in rain]
    kf, ka, c = p.as_tuple()
    threads = O.max_threads()
    # one step touches the pages, four more size the sample to about budget_s,
    # timed as three runs of n steps that continue the same state (median)
    O.step_f32(b, d, f, v, kf, ka, c, O.BOUNDARY_CLOSED, src, nsteps=1, threads=threads)
    t4 = O.step_f32(b, d, f, v, kf, ka, c, O.BOUNDARY_CLOSED, src, nsteps=4, threads=threads)
    n = int(max(1, min(2000, budget_s / 3 / max(t4 / 4, 1e-6))))
    runs = [O.step_f32(b, d, f, v, kf, ka, c, O.BOUNDARY_CLOSED, src, nsteps=n, threads=threads)
            for _ in range(3)]
    tn = statistics.median(runs)
    total_steps = 3 * n + 5
    # the GPU on the same steps
    g.generate_scene(2026, 40.0, 15.0)
    g.set_sources(rain)
    g.step(total_steps)
    gd, gf, gv = g.download()
    err = float(np.abs(gd.astype(np.float64) - d).max())
    rel = err / max(1e-30, float(np.abs(d).max()))
    bitexact = bool(np.array_equal(gd.view(np.uint32), d.view(np.uint32))
                    and np.array_equal(gf.view(np.uint32), f.view(np.uint32))
                    and np.array_equal(gv.view(np.uint32), v.view(np.uint32)))
    vg, vo = float(np.sum(gd, dtype=np.float64)), O.volume(d)
    # the FP64 oracle on a few steps of the same grid (reported beside the FP32 port)
    b64, d64 = (a.astype(np.float64) for a in O.terrain(2026, size, size, 40.0, 15.0))
    f64 = np.zeros((size, size, 4), np.float64)
    k64 = O.params_physical()
    src64 = [(s[0], s[1], s[2], s[3], 0.01) for s in rain]
    O.step_f64(b64, d64, f64, None, *k64, O.BOUNDARY_CLOSED, src64, nsteps=1, threads=threads)
    n64 = max(1, min(n, 10))
    t64 = statistics.median(
        O.step_f64(b64, d64, f64, None, *k64, O.BOUNDARY_CLOSED, src64, nsteps=n64,
                   threads=threads) for _ in range(3))
    return {
        "value": round(size * size * n / tn / 1e9, 4),
        "fp64_value": round(size * size * n64 / t64 / 1e9, 4),
        "fp64_sample": f"FP64 oracle, median of 3 runs of {n64} steps of the same grid "
                       "(+1 warm-up step)",
        "unit": "Gcell-steps/s",
        "cores": threads,
        "kind": "port",
        "sample": f"{size}x{size} grid, median of 3 runs of {n} steps (+5 warm-up steps), "
                  f"FP32 oracle, OpenMP {threads} threads; GPU state after the same "
                  f"{total_steps} steps compared on the full grid",
        "seconds": round(tn, 3),
        "runs_seconds": [round(t, 3) for t in runs],
        "parity": {"steps": total_steps, "bitexact": bitexact, "max_abs_depth_err": err,
                   "rel_max_depth_err": rel,
                   "rel_volume_diff": abs(vg - vo) / max(1e-30, abs(vo))},
    }


# ------------------------------------------------------------------ reference arm

def run_reference(args):
    """The reference's path on the host cores: the CPU port of its shaders
    (the reference itself is an OpenGL/Win32 program that cannot run here).
    Each bench step advances the same 4096^2 grid by `ref_chain` steps."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return None
    from oracle import oracle as O

    size = args.size
    ref_chain = 5
    kf, ka, c = (np.float32(x) for x in O.params_physical(0.02, 9.81, 1.0, 1.0, 0.998))
    (cx, cy), = O.rain_centers(2026, size, size, 64, 1)
    src = [(O.SOURCE_DISK, cx, cy, 64, 0.01)]
    b, d = O.terrain(2026, size, size, 40.0, 15.0)
    f = np.zeros((size, size, 4), np.float32)
    v = np.zeros((size, size, 2), np.float32)
    threads = O.max_threads()
    warmup = max(3, args.warmup)
    for _ in range(warmup):
        O.step_f32(b, d, f, v, kf, ka, c, O.BOUNDARY_CLOSED, src, nsteps=ref_chain, threads=threads)
    per = []
    for _ in range(args.steps):
        per.append(O.step_f32(b, d, f, v, kf, ka, c, O.BOUNDARY_CLOSED, src, nsteps=ref_chain,
                              threads=threads))
    total = sum(per)
    value = size * size * ref_chain * args.steps / total / 1e9
    return {
        "metric": METRIC,
        "impl": "reference",
        "value": round(value, 4),
        "unit": "Gcell-steps/s",
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": warmup,
        "ms_per_step": round(total / args.steps * 1e3, 3),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic: seeded PCG32 fBm terrain 0-40 m, fill 15 m, rain disk r=64",
        "config": {
            "workload": f"{size}x{size} FP32 virtual-pipe grid, closed walls, rain r=64, "
                        f"{ref_chain} simulation steps per bench step (bounded CPU sample)",
            "grid": [size, size],
            "sim_steps_per_bench_step": ref_chain,
            "parallelism": "host cores (OpenMP)",
        },
        "cpu_baseline": {
            "value": round(value, 4), "unit": "Gcell-steps/s", "cores": threads, "kind": "port",
            "sample": f"{size}x{size} grid, {ref_chain} steps per bench step, FP32 CPU port of "
                      "flowUpdate.comp + flowApply.comp (the reference runs them through OpenGL, "
                      "which this machine does not have)",
        },
        "e2e": {"value": round(value, 4), "unit": "Gcell-steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "p50_ms": round(sorted(per)[len(per) // 2] * 1e3, 3),
        "p99_ms": round(sorted(per)[min(len(per) - 1, int(0.99 * len(per)))] * 1e3, 3),
    }


# ------------------------------------------------------------------ other configurations

def _events(torch, stream, n):
    return [torch.cuda.Event(enable_timing=True) for _ in range(n)]


def run_c1(args):
    """256^2, closed walls, rain r=16, 1000 steps: throughput, per-step latency,
    parity with the FP32 oracle and drift against the FP64 oracle."""
    import torch

    import terrainwatersim_gb300 as tws
    from oracle import oracle as O

    W = H = 256
    steps = 1000
    p = tws.params_physical(0.02, 9.81, 1.0, 1.0, 0.998, tws.BOUNDARY_CLOSED)
    rain = tws.rain_disks(2026, W, H, 16, 0.01, 1)
    stream = torch.cuda.Stream()
    g = tws.Grid(W, H, p, stream=stream.cuda_stream)
    g.set_sources(rain)
    g.generate_scene(2026, 40.0, 15.0)
    tuned = g.autotune(24)
    g.generate_scene(2026, 40.0, 15.0)
    g.step(50)  # warm-up
    g.generate_scene(2026, 40.0, 15.0)
    torch.cuda.synchronize()
    ev = _events(torch, stream, steps + 1)
    ev[0].record(stream)
    for i in range(steps):
        g.step(1)
        ev[i + 1].record(stream)
    torch.cuda.synchronize()
    per = sorted(ev[i].elapsed_time(ev[i + 1]) * 1e3 for i in range(steps))
    total = ev[0].elapsed_time(ev[steps]) / 1e3
    d, f, v = g.download()
    vol = g.volume()
    b, od = O.terrain(2026, W, H, 40.0, 15.0)
    of = np.zeros((H, W, 4), np.float32)
    ov = np.zeros((H, W, 2), np.float32)
    src = [(s[0], s[1], s[2], s[3], s[4]) for s in rain]
    kf, ka, c = p.as_tuple()
    threads = O.max_threads()
    # the oracle's own step loops are the timed CPU baseline (FP32 and FP64),
    # each the median of three runs from the initial state
    d0 = od.copy()
    t32s = []
    for _ in range(3):
        od[...], of[...], ov[...] = d0, 0.0, 0.0
        t32s.append(O.step_f32(b, od, of, ov, kf, ka, c, O.BOUNDARY_CLOSED, src, nsteps=steps,
                               threads=threads))
    t32 = statistics.median(t32s)
    k64 = O.params_physical()
    t64s = []
    for _ in range(3):
        b64, d64 = O.terrain(2026, W, H, 40.0, 15.0)
        b64, d64 = b64.astype(np.float64), d64.astype(np.float64)
        f64 = np.zeros((H, W, 4), np.float64)
        t64s.append(O.step_f64(b64, d64, f64, None, *k64, O.BOUNDARY_CLOSED,
                               [(s[0], s[1], s[2], s[3], 0.01) for s in rain], nsteps=steps,
                               threads=threads))
    t64 = statistics.median(t64s)
    v64 = O.volume(d64)
    g.close()
    resident = None
    if tws.resident_fits(W, H):
        # the same 1000 steps with the grid held in one cluster's shared memory
        g = tws.Grid(W, H, p, stream=stream.cuda_stream)
        g.set_sources(rain)
        g.set_resident(True)
        for _ in range(3):
            g.generate_scene(2026, 40.0, 15.0)
            g.step(steps)
        g.generate_scene(2026, 40.0, 15.0)
        torch.cuda.synchronize()
        n0 = tws.lib().tws_launch_count()
        ev[0].record(stream)
        g.step(steps)
        ev[1].record(stream)
        torch.cuda.synchronize()
        rt = ev[0].elapsed_time(ev[1]) / 1e3
        launches = int(tws.lib().tws_launch_count() - n0)
        rd, rf, rv = g.download()
        g.close()
        resident = {
            "kernel": "resident_kernel (one 16-CTA cluster, state in distributed shared memory)",
            "gcell_steps_per_s": round(W * H * steps / rt / 1e9, 3),
            "step_us_mean": round(rt / steps * 1e6, 3),
            "launches": launches,
            "bitexact_vs_fp32_oracle": bool(np.array_equal(rd.view(np.uint32), od.view(np.uint32))
                                            and np.array_equal(rf.view(np.uint32), of.view(np.uint32))
                                            and np.array_equal(rv.view(np.uint32), ov.view(np.uint32))),
        }
    return {
        "config": "256x256 FP32, closed walls, rain r=16 +0.01 m/step, 1000 steps, one launch per step",
        "gcell_steps_per_s": round(W * H * steps / total / 1e9, 3),
        "step_us_p50": round(per[len(per) // 2], 2),
        "step_us_p99": round(per[int(0.99 * len(per))], 2),
        "variant": tuned,
        "bitexact_vs_fp32_oracle": bool(np.array_equal(d.view(np.uint32), od.view(np.uint32))
                                        and np.array_equal(f.view(np.uint32), of.view(np.uint32))
                                        and np.array_equal(v.view(np.uint32), ov.view(np.uint32))),
        "rel_volume_diff_vs_fp32_oracle": abs(vol - O.volume(od)) / O.volume(od),
        "max_abs_depth_err_vs_fp64": float(np.abs(d - d64).max()),
        "rel_volume_drift_vs_fp64": abs(vol - v64) / v64,
        "resident": resident,
        "cpu_oracle": {"fp32_gcell_steps_per_s": round(W * H * steps / t32 / 1e9, 4),
                       "fp64_gcell_steps_per_s": round(W * H * steps / t64 / 1e9, 4),
                       "cores": threads, "kind": "port",
                       "sample": f"the same {steps} steps of the {W}x{H} grid, OpenMP, "
                                 "median of 3 runs"},
    }


def c3_workload(n=64, seed=2026):
    """64 grids: side log-uniform in [128, 2048] rounded to 32, aspect U[1, 4],
    own terrain seed, fill U[8, 20] m, rain U[0.002, 0.02] m/step on one disk of
    radius 16."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        side = int(round(np.exp(rng.uniform(np.log(128), np.log(2048))) / 32)) * 32
        aspect = rng.uniform(1.0, 4.0)
        other = max(32, int(round(side * aspect / 32)) * 32)
        W, H = (side, other) if i % 2 == 0 else (other, side)
        out.append(dict(W=W, H=H, seed=10000 + i, fill=float(rng.uniform(8, 20)),
                        rate=float(rng.uniform(0.002, 0.02)), radius=16))
    return out


def run_c3(args):
    import torch

    import terrainwatersim_gb300 as tws
    from oracle import oracle as O

    steps = 2000
    work = c3_workload()
    p = tws.params_physical(0.02, 9.81, 1.0, 1.0, 0.998, tws.BOUNDARY_CLOSED)
    grids = []
    for w in work:
        g = tws.Grid(w["W"], w["H"], p)
        g.set_sources(tws.rain_disks(w["seed"], w["W"], w["H"], w["radius"], w["rate"], 1))
        grids.append(g)
    cells = sum(w["W"] * w["H"] for w in work)

    def reset():
        for g, w in zip(grids, work):
            g.generate_scene(w["seed"], 40.0, w["fill"])
        for g in grids:
            g.sync()

    # per-grid plain launches: every grid advanced on its own, one launch per step
    reset()
    for g in grids:
        g.set_variant(0)
        g.step(16)
    torch.cuda.synchronize()
    reset()
    t0 = time.perf_counter()
    for g in grids:  # one grid at a time
        g.step(steps)
        g.sync()
    plain_s = time.perf_counter() - t0
    reset()
    t0 = time.perf_counter()
    for g in grids:  # every grid on its own stream, all in flight together
        g.step(steps)
    for g in grids:
        g.sync()
    plain_streams_s = time.perf_counter() - t0

    # batched: one persistent launch per step over all 64 grids, graph chains of 16
    reset()
    batch = tws.Batch()
    for g in grids:
        batch.add(g)
    # every batched variant on the same 192 steps (state reset before each)
    sweep = {}
    for vi, (k, tx, ty) in enumerate(tws.batch_variants()):
        reset()
        batch.set_variant(vi)
        batch.step(32)
        batch.sync()
        t0 = time.perf_counter()
        batch.step(192)
        batch.sync()
        sweep[f"{vi}_k{k}_{tx}x{ty}"] = round(cells * 192 / (time.perf_counter() - t0) / 1e9, 3)
    tuned = batch.autotune(32)
    batch.step(32)
    batch.sync()
    reset()
    ev = _events(torch, None, 2)
    t0 = time.perf_counter()
    batch.step(steps)
    batch.sync()
    batch_s = time.perf_counter() - t0
    chains, replayed = batch.stats()

    # FP64 oracle on 4 sampled grids (the smallest four, for CPU time)
    order = sorted(range(len(work)), key=lambda i: work[i]["W"] * work[i]["H"])[:4]
    checks = []
    for i in order:
        w, g = work[i], grids[i]
        d, _, _ = g.download(flux=False, velocity=False)
        vol = float(np.sum(d, dtype=np.float64))
        b64, d64 = O.terrain(w["seed"], w["W"], w["H"], 40.0, w["fill"])
        b64, d64 = b64.astype(np.float64), d64.astype(np.float64)
        f64 = np.zeros((w["H"], w["W"], 4), np.float64)
        (cx, cy), = O.rain_centers(w["seed"], w["W"], w["H"], w["radius"], 1)
        O.step_f64(b64, d64, f64, None, *O.params_physical(), O.BOUNDARY_CLOSED,
                   [(O.SOURCE_DISK, cx, cy, w["radius"], w["rate"])], nsteps=steps)
        v64 = O.volume(d64)
        checks.append({"grid": [w["W"], w["H"]],
                       "max_abs_depth_err_vs_fp64": float(np.abs(d - d64).max()),
                       "rel_volume_drift_vs_fp64": abs(vol - v64) / v64})
    batch.close()
    for g in grids:
        g.close()
    del ev
    return {
        "config": "64 uneven grids (side log-uniform 128-2048, aspect 1-4), 2000 steps, "
                  "closed walls, per-grid seed/fill/rain",
        "cells": cells,
        "batched_gcell_steps_per_s": round(cells * steps / batch_s / 1e9, 3),
        "per_grid_plain_gcell_steps_per_s": round(cells * steps / plain_s / 1e9, 3),
        "per_grid_plain_concurrent_streams_gcell_steps_per_s":
            round(cells * steps / plain_streams_s / 1e9, 3),
        "speedup_vs_one_grid_at_a_time": round(plain_s / batch_s, 3),
        "speedup_vs_concurrent_streams": round(plain_streams_s / batch_s, 3),
        "batched_variant": {"index": tuned, "k_tile": tws.batch_variants()[tuned]},
        "batched_variant_sweep_gcell_steps_per_s": sweep,
        "chains": chains, "graph_replays": replayed,
        "fp64_checks": checks,
    }


def run_c4(args):
    """16384^2, 8 rain disks r=128, FP16 flux storage vs all-FP32, 5000 steps.
    Volume drift against the exact FP64 bookkeeping (initial FP64 volume plus
    the rain added); depth error against the FP64 oracle on a 1024^2 window
    after a reduced run whose domain of dependence fits an oracle crop."""
    import torch

    import terrainwatersim_gb300 as tws
    from oracle import oracle as O

    N = args.size if args.size != W_DEFAULT else 16384
    steps = 5000
    p = tws.params_physical(0.02, 9.81, 1.0, 1.0, 0.998, tws.BOUNDARY_CLOSED)
    rain = tws.rain_disks(2026, N, N, 128, 0.01, 8)
    out = {"config": f"{N}x{N}, 8 rain disks r=128 +0.01 m/step, closed walls, {steps} steps"}
    disk_cells = 0
    for s in rain:
        r = int(s[3])
        yy, xx = np.mgrid[-r:r + 1, -r:r + 1]
        disk_cells += int(np.count_nonzero(xx * xx + yy * yy <= r * r))
    for name, fs in (("fp16_flux", tws.FLUX_F16), ("fp32", tws.FLUX_F32)):
        g = tws.Grid(N, N, p, fs)
        g.set_sources(rain)
        g.generate_scene(2026, 40.0, 15.0)
        v0 = g.volume()
        tuned = g.autotune(24)
        g.generate_scene(2026, 40.0, 15.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        g.step(steps)
        g.sync()
        secs = time.perf_counter() - t0
        vol = g.volume()
        exact = v0 + steps * 0.01 * disk_cells
        bpc = BYTES_PER_CELL_STEP_F16 if fs == tws.FLUX_F16 else BYTES_PER_CELL_STEP_F32
        out[name] = {"gcell_steps_per_s": round(N * N * steps / secs / 1e9, 3),
                     "effective_gbs": round(bpc * N * N * steps / secs / 1e9, 1),
                     "variant": tuned, "flux_scale": g.buffers().flux_scale,
                     "rel_volume_drift_vs_fp64_bookkeeping": abs(vol - exact) / exact}
        g.close()
        torch.cuda.empty_cache()
    # Depth error on a 1024^2 window centred on the first rain disk, where the
    # water moves (the initial state d = max(0, 15 - b) is a lake at rest, so a
    # window away from every disk would see no flow at all).  The FP64 oracle
    # runs on a crop that holds the window's whole domain of dependence (two
    # cells per step); where the crop reaches the grid's edge it is the grid's
    # own closed wall.
    short, win = args.c4_window_steps, 1024
    margin = 2 * short + 8
    cx, cy = int(rain[0][1]), int(rain[0][2])
    x0 = min(max(0, cx - win // 2), N - win)
    y0 = min(max(0, cy - win // 2), N - win)
    cx0, cy0 = max(0, x0 - margin), max(0, y0 - margin)
    cx1, cy1 = min(N, x0 + win + margin), min(N, y0 + win + margin)
    b, d0 = O.terrain(2026, N, N, 40.0, 15.0)
    b64 = np.ascontiguousarray(b[cy0:cy1, cx0:cx1]).astype(np.float64)
    d64 = np.ascontiguousarray(d0[cy0:cy1, cx0:cx1]).astype(np.float64)
    d0w = d0[y0:y0 + win, x0:x0 + win].astype(np.float64)
    del b, d0
    f64 = np.zeros(b64.shape + (4,), np.float64)
    srcs = [(O.SOURCE_DISK, s[1] - cx0, s[2] - cy0, s[3], 0.01) for s in rain]
    t0 = time.perf_counter()
    O.step_f64(b64, d64, f64, None, *O.params_physical(), O.BOUNDARY_CLOSED, srcs, nsteps=short)
    t64 = time.perf_counter() - t0
    ref = d64[y0 - cy0:y0 - cy0 + win, x0 - cx0:x0 - cx0 + win].copy()
    del b64, d64, f64
    moved = np.abs(ref - d0w) > 1e-3
    out["window"] = {"origin": [x0, y0], "size": win, "steps": short,
                     "centre_rain_disk": [cx, cy, int(rain[0][3])],
                     "fp64_crop": [cx1 - cx0, cy1 - cy0],
                     "fp64_seconds": round(t64, 1),
                     "cells_moved_over_1mm_frac": round(float(moved.mean()), 4),
                     "max_depth_change_m": float(np.abs(ref - d0w).max())}
    wins = {}
    for name, fs in (("fp16_flux", tws.FLUX_F16), ("fp32", tws.FLUX_F32)):
        g = tws.Grid(N, N, p, fs)
        g.set_sources(rain)
        g.generate_scene(2026, 40.0, 15.0)
        g.step(short)
        d, _, _ = g.download(flux=False, velocity=False)
        g.close()
        gw = d[y0:y0 + win, x0:x0 + win].astype(np.float64)
        del d
        wins[name] = gw
        err = np.abs(gw - ref)
        out[name]["window_steps"] = short
        out[name]["window_max_abs_depth_err_vs_fp64"] = float(err.max())
        out[name]["window_rel_max_depth_err_vs_fp64"] = float(err.max()
                                                               / max(1e-30, np.abs(ref).max()))
        out[name]["window_mean_abs_depth_err_vs_fp64"] = float(err.mean())
        out[name]["window_rel_volume_diff_vs_fp64"] = float(abs(gw.sum() - ref.sum()) / ref.sum())
    out["window"]["fp16_vs_fp32_max_abs_depth_diff"] = float(
        np.abs(wins["fp16_flux"] - wins["fp32"]).max())
    return out


def c5_workload(n, max_steps, seed=2026):
    """Requests: side log-uniform [64, 4096], aspect U[1, 2], own terrain seed,
    fill U[8, 20] m, one rain disk (radius min(W, H)/32, at least 4 cells,
    +0.01 m/step), steps log-uniform [100, max_steps]."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        side = int(round(np.exp(rng.uniform(np.log(64), np.log(4096)))))
        other = int(round(side * rng.uniform(1.0, 2.0)))
        W, H = (side, other) if i % 2 == 0 else (other, side)
        steps = int(round(np.exp(rng.uniform(np.log(100), np.log(max_steps)))))
        out.append(dict(W=W, H=H, seed=50000 + i, fill=float(rng.uniform(8, 20)),
                        radius=max(4, min(W, H) // 32), rate=0.01, steps=steps))
    return out


C5_ARMS_ALL = (("served_fp16_batched", "f16", False, True),
               ("served_fp32_batched", "f32", False, True),
               ("serial_fp32_plain", "f32", True, True),
               ("saturated_served_fp16_batched", "f16", False, False),
               ("saturated_served_fp32_batched", "f32", False, False),
               ("saturated_serial_fp32_plain", "f32", True, False))
# the default bench line's serving leg: the served FP16 path against serial
# plain-kernel execution, at 70% load (latency) and saturated (capacity)
C5_ARMS_DEFAULT = tuple(a for a in C5_ARMS_ALL if "fp32_batched" not in a[0])


def serving_leg(n, max_steps, arms=C5_ARMS_ALL):
    """Serving loop vs serial plain-kernel execution of the same request
    stream (the first n requests of the seeded stream).  Each arm reports
    time-to-completion percentiles over its requests, aggregate Gcell-steps/s
    over the makespan, and each request's final volume against exact FP64
    bookkeeping (initial FP64 volume plus the rain added)."""
    import torch

    import terrainwatersim_gb300 as tws
    from terrainwatersim_gb300 import serve

    work = c5_workload(n, max_steps)
    total_cell_steps = float(sum(w["W"] * w["H"] * w["steps"] for w in work))
    p = tws.params_physical(0.02, 9.81, 1.0, 1.0, 0.998, tws.BOUNDARY_CLOSED)

    # capacity: the batched FP16 path on a large grid (cell-steps per second)
    g = tws.Grid(4096, 4096, p, tws.FLUX_F16)
    g.generate_scene(1, 40.0, 15.0)
    g.step(32)
    g.sync()
    t0 = time.perf_counter()
    g.step(400)
    g.sync()
    capacity = 4096 * 4096 * 400 / (time.perf_counter() - t0)
    g.close()
    load = 0.7
    rate = load * capacity / (total_cell_steps / n)  # requests per second
    rng = np.random.default_rng(7)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, n))
    arrivals -= arrivals[0]

    # exact FP64 bookkeeping of the final volumes: initial volume + rain added
    expected = []
    for w in work:
        gg = tws.Grid(w["W"], w["H"], p, tws.FLUX_F32)
        gg.generate_scene(w["seed"], 40.0, w["fill"])
        v0 = gg.volume()
        gg.close()
        r = w["radius"]
        yy, xx = np.mgrid[-r:r + 1, -r:r + 1]
        ncells = int(np.count_nonzero(xx * xx + yy * yy <= r * r))
        expected.append(v0 + w["steps"] * float(np.float32(w["rate"])) * ncells)
    torch.cuda.empty_cache()

    def requests():
        for i, w in enumerate(work):
            src = tws.rain_disks(w["seed"], w["W"], w["H"], w["radius"], w["rate"], 1)
            yield serve.make_request(i, w["W"], w["H"], w["seed"], w["fill"], p, src, w["steps"],
                                     float(arrivals[i]))

    out = {"config": f"{n} Poisson requests, side log-uniform 64-4096, aspect 1-2, steps "
                     f"log-uniform 100-{max_steps}, one rain disk each, closed walls, "
                     f"arrival rate for {int(load * 100)}% load of the measured FP16 capacity",
           "requests": n, "total_cell_steps": total_cell_steps,
           "capacity_gcell_steps_per_s": round(capacity / 1e9, 3),
           "arrival_rate_per_s": round(rate, 3), "arrival_span_s": round(float(arrivals[-1]), 3)}
    for name, fs_name, serial, poisson in arms:
        fs = tws.FLUX_F16 if fs_name == "f16" else tws.FLUX_F32
        with serve.Server(memory_budget_bytes=120e9, flux_storage=fs) as srv:
            for r in requests():
                if not poisson:  # every request present at the start: capacity
                    r.arrival_s = 0.0
                srv.submit(r)
            srv.close_submissions()
            srv.run(serial=serial)
            res = sorted(srv.results(), key=lambda r: r.id)
            st = srv.stats()
        ok = [r for r in res if r.status == 0]
        lat = np.array([r.latency_s for r in ok])
        makespan = max(r.done_s for r in ok) - min(r.arrival_s for r in ok)
        drift = [abs(r.volume - expected[r.id]) / expected[r.id] for r in ok]
        out[name] = {
            "completed": len(ok),
            "aggregate_gcell_steps_per_s": round(st["cell_steps"] / makespan / 1e9, 3),
            "busy_gcell_steps_per_s": round(st["cell_steps"] / st["seconds"] / 1e9, 3),
            "makespan_s": round(makespan, 3),
            "latency_s_p50": round(float(np.percentile(lat, 50)), 4),
            "latency_s_p95": round(float(np.percentile(lat, 95)), 4),
            "latency_s_p99": round(float(np.percentile(lat, 99)), 4),
            "peak_resident_gb": round(st["peak_bytes"] / 1e9, 3),
            "chains": st["chains"],
            "max_rel_volume_drift_vs_fp64_bookkeeping": float(max(drift)),
        }

    def ratio(a, b):
        if a in out and b in out:
            return round(out[a]["aggregate_gcell_steps_per_s"]
                         / out[b]["aggregate_gcell_steps_per_s"], 3)
        return None
    out["aggregate_speedup"] = ratio("served_fp16_batched", "serial_fp32_plain")
    out["saturated_speedup"] = ratio("saturated_served_fp16_batched",
                                     "saturated_serial_fp32_plain")
    sp = ratio("saturated_served_fp32_batched", "saturated_serial_fp32_plain")
    if sp is not None:
        out["saturated_speedup_fp32_served"] = sp
    return out


def run_c5(args):
    """Serving loop vs serial plain-kernel execution of the full request stream."""
    return serving_leg(args.requests, args.max_steps, C5_ARMS_ALL)


def main():
    args = parse()
    if args.config != "c2":
        res = {"c1": run_c1, "c3": run_c3, "c4": run_c4, "c5": run_c5}[args.config](args)
        print(json.dumps(res), flush=True)
        return
    res = run_reference(args) if args.impl == "reference" else run_ours(args)
    if res is not None:
        print(json.dumps(res), flush=True)


if __name__ == "__main__":
    main()
