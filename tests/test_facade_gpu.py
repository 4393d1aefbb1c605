"""The C++ facade (include/tws_watersim.hpp) used from a C++ program the way
the reference's scene uses Terrain: frame-time driven PerformSimulationStep
with its 10-step clamp, brush strokes, parameter setters.  The program is
compiled here against libtws.so and its output compared with the oracle."""
from __future__ import annotations

import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT, assert_bitexact

pytestmark = pytest.mark.gpu


def _cuda_home():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return os.environ.get("CUDA_HOME") or os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def _build(tmp_path):
    import terrainwatersim_gb300 as tws
    lib_dir = os.path.dirname(tws.library_path())
    cuda = _cuda_home()
    exe = str(tmp_path / "facade_check")
    cxx = shutil.which("g++") or "g++"
    subprocess.run([cxx, "-std=c++17", "-O2", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"),
                    "-I", os.path.join(cuda, "include"),
                    os.path.join(ROOT, "tests", "cpp", "facade_check.cpp"), "-L", lib_dir, "-ltws",
                    f"-Wl,-rpath,{lib_dir}", "-L", os.path.join(cuda, "lib64"), "-lcudart",
                    f"-Wl,-rpath,{os.path.join(cuda, 'lib64')}", "-o", exe], check=True)
    return exe


def test_cpp_facade_matches_oracle(tmp_path, oracle):
    N = 128
    exe = _build(tmp_path)
    out = str(tmp_path / "state.bin")
    r = subprocess.run([exe, str(N), out], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    raw = np.fromfile(out, dtype=np.uint8)
    total = int(raw[:4].view(np.uint32)[0])
    body = raw[4:].view(np.float32)
    d = body[:N * N].reshape(N, N)
    f = body[N * N:5 * N * N].reshape(N, N, 4)
    v = body[5 * N * N:].reshape(N, N, 2)

    # replay: Terrain.cpp:242-247 accumulator in double, step 1/60 s as float
    step = float(np.float32(1.0) / np.float32(60.0))
    acc, steps = 0.0, []
    for fr in (0.025, 0.025, 0.4, 0.025, 0.010, 0.030):
        acc += fr
        n = int(acc / step)
        acc -= step * n
        steps.append(min(n, 10))
    assert total == sum(steps)
    kf, ka, c = oracle.params_reference(60.0, 0.97, 20.0, float(N), N)
    b, od = oracle.terrain(77, N, N, 40.0, 15.0)
    of = np.zeros((N, N, 4), np.float32)
    ov = np.zeros((N, N, 2), np.float32)
    wx = np.float32(np.float32(0.3) * np.float32(N)) + np.float32(np.float32(5.0) * np.float32(N))
    wz = np.float32(np.float32(0.6) * np.float32(N))
    px, pz = np.float32(wx / np.float32(N)), np.float32(wz / np.float32(N))
    px, pz = np.float32(px - np.trunc(px)), np.float32(pz - np.trunc(pz))
    bx, by = float(np.float32(px * np.float32(N))), float(np.float32(pz * np.float32(N)))
    for i, n in enumerate(steps):
        if i == 1:
            oracle.sources_f32(od, [(oracle.SOURCE_BRUSH, bx, by, 32.0, 4.0)])
        if n:
            oracle.step_f32(b, od, of, ov, kf, ka, c, oracle.BOUNDARY_OPEN, nsteps=n)
    assert_bitexact(d, od, "depth")
    assert_bitexact(f, of, "flux")
    assert_bitexact(v, ov, "velocity")


def test_cpp_facade_reference_reset_matches_oracle(tmp_path, oracle):
    """WaterSim::CreateHeightmapFromNoiseAndResetSim() called twice gives the
    reference's second scene after start-up (a new noise table per call)."""
    N = 160
    exe = _build(tmp_path)
    out = str(tmp_path / "scene.bin")
    r = subprocess.run([exe, str(N), out, "reference"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    body = np.fromfile(out, dtype=np.float32)
    b, d = body[:N * N].reshape(N, N), body[N * N:].reshape(N, N)
    ob, od = oracle.reference_terrain(N, N, 300.0, generation=1)
    assert_bitexact(b, ob, "terrain")
    assert_bitexact(d, od, "depth")


def test_cpp_facade_refreshes_textures_after_a_step(tmp_path, oracle):
    """With texture targets set, a PerformSimulationStep call that takes a step
    rewrites TerrainData (RGBA32F), its whole mip pyramid and the RG16F flow
    map, as the reference regenerates the mips after its steps
    (Terrain.cpp:272-276); a call that takes no step leaves them alone."""
    N = 64
    exe = _build(tmp_path)
    out = str(tmp_path / "tex.bin")
    r = subprocess.run([exe, str(N), out, "textures"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    raw = np.fromfile(out, dtype=np.uint8)
    assert int(raw[:4].view(np.uint32)[0]) == 1
    pos = 4
    d = raw[pos:pos + 4 * N * N].view(np.float32).reshape(N, N)
    pos += 4 * N * N
    kf, ka, c = oracle.params_reference(60.0, 0.98, 10.0, float(N), N)
    b, od = oracle.terrain(91, N, N, 40.0, 15.0)
    of = np.zeros((N, N, 4), np.float32)
    ov = np.zeros((N, N, 2), np.float32)
    oracle.step_f32(b, od, of, ov, kf, ka, c, oracle.BOUNDARY_OPEN, nsteps=1)
    assert_bitexact(d, od, "depth")
    levels = int(np.log2(N))
    rgba, mips = oracle.terrain_mips(b, od, levels)
    texels = sum(m.shape[0] * m.shape[1] for m in mips)
    flow = ov.astype(np.float16).view(np.uint16)
    for pass_ in range(2):
        g_rgba = raw[pos:pos + 16 * N * N].view(np.float32).reshape(N, N, 4)
        pos += 16 * N * N
        g_mips = raw[pos:pos + 16 * texels].view(np.float32)
        pos += 16 * texels
        g_flow = raw[pos:pos + 4 * N * N].view(np.uint16).reshape(N, N, 2)
        pos += 4 * N * N
        if pass_ == 0:
            assert_bitexact(g_rgba, rgba, "TerrainData")
            assert_bitexact(g_mips, np.concatenate([m.ravel() for m in mips]), "mips")
            assert np.array_equal(g_flow, flow)
        else:  # the idle frame wrote nothing
            assert not g_rgba.any() and not g_mips.any() and not g_flow.any()
