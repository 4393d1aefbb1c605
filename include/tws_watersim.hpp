// tws_watersim.hpp -- C++ facade over tws.h with the method names of the
// simulation half of terrainwatersim's Terrain class
// (terrainwatersim/source/scene/Terrain.h:15-153), for renderer-side callers.
//
// Header-only; link against libtws.so.  Errors are reported as tws::Error
// exceptions (the reference logs and asserts; a C++ caller gets the status).
// One WaterSim per thread at a time, like the reference's single GL thread.
#pragma once

#include <cmath>
#include <cstdint>
#include <stdexcept>
#include <string>

#include "tws.h"

namespace tws {

class Error : public std::runtime_error {
 public:
  Error(int code, const std::string& what) : std::runtime_error(what), code_(code) {}
  int code() const { return code_; }

 private:
  int code_;
};

inline void check(int code, tws_grid* g = nullptr) {
  if (code != TWS_OK) {
    std::string m = tws_error_string(code);
    if (g) m += std::string(": ") + tws_last_error(g);
    throw Error(code, m);
  }
}

class WaterSim {
 public:
  // Terrain::Terrain's simulation defaults (Terrain.cpp:22-30): a 1024 x 1024
  // grid over 1024 world units, 60 steps per second, flow damping 0.98,
  // flow acceleration 10.  The reference's border is the open sink.
  explicit WaterSim(unsigned gridResolution = 1024, float gridWorldSize = 1024.0f,
                    int boundary = TWS_BOUNDARY_OPEN, int fluxStorage = TWS_FLUX_F32,
                    void* cudaStream = nullptr)
      : m_gridResolution(gridResolution),
        m_gridWorldSize(gridWorldSize),
        m_boundary(boundary),
        m_stepsPerSecond(60.0f),
        m_simulationStepLength((double)(1.0f / 60.0f)),
        m_flowDamping(0.98f),
        m_flowAcceleration(10.0f),
        m_timeSinceLastSimulationStep(0.0) {
    tws_sim_params p;
    check(tws_params_reference(60.0f, m_flowDamping, m_flowAcceleration, m_gridWorldSize,
                               m_gridResolution, m_boundary, &p));
    check(tws_create((int)gridResolution, (int)gridResolution, &p, fluxStorage, cudaStream,
                     &m_grid));
  }
  ~WaterSim() {
    if (m_grid) tws_destroy(m_grid);
  }
  WaterSim(const WaterSim&) = delete;
  WaterSim& operator=(const WaterSim&) = delete;

  /// Terrain::CreateHeightmapFromNoiseAndResetSim (Terrain.cpp:200-238): the
  /// reference's own noise terrain (height scale 300, Terrain.cpp:25) and
  /// central pool, outflow and flow map zero.  Each call draws the next noise
  /// table, as the reference's application-wide generator (seeded once,
  /// Application.cpp:57) does, so the first call gives the reference's first
  /// scene.
  void CreateHeightmapFromNoiseAndResetSim() {
    check(tws_generate_reference_scene(m_grid, TWS_REFERENCE_NOISE_SEED, m_noiseScenes,
                                       m_heightScale),
          m_grid);
    ++m_noiseScenes;
    m_timeSinceLastSimulationStep = 0.0;
  }

  /// The same reset with the benchmark's seeded generator instead: terrain in
  /// [0, heightScale), depth max(0, fill - terrain), outflow and flow map zero.
  void CreateHeightmapFromNoiseAndResetSim(uint64_t seed, float heightScale, float fill) {
    check(tws_generate_scene(m_grid, seed, heightScale, fill), m_grid);
    m_timeSinceLastSimulationStep = 0.0;
  }

  /// Reset from host arrays (terrain required, depth may be null).
  void ResetFromHeightmap(const float* terrain, const float* depth) {
    check(tws_upload(m_grid, terrain, depth, nullptr), m_grid);
    m_timeSinceLastSimulationStep = 0.0;
  }

  /// Terrain::PerformSimulationStep (Terrain.cpp:240-277): a fixed-step
  /// accumulator, at most 10 steps per call.  Returns the steps taken.  When
  /// texture targets are set (SetTextureTargets), a call that took a step
  /// also rewrites them, mip pyramid included, as the reference regenerates
  /// TerrainData's mips after its steps (Terrain.cpp:272-276); without
  /// targets the renderer reads the device buffers (GetBuffers) directly.
  unsigned PerformSimulationStep(double lastFrameSeconds) {
    m_timeSinceLastSimulationStep += lastFrameSeconds;
    unsigned n = (unsigned)(m_timeSinceLastSimulationStep / m_simulationStepLength);
    m_timeSinceLastSimulationStep -= m_simulationStepLength * n;
    if (n > 10u) n = 10u;
    if (n > 0) {
      check(tws_step(m_grid, (int)n), m_grid);
      if (m_texRgba || m_texFlowmap)
        check(tws_export_textures(m_grid, m_texRgba, m_texFlowmap, m_texMipLevels, m_texMips),
              m_grid);
    }
    return n;
  }

  /// Device buffers (caller-owned, layouts of tws_export_textures) that
  /// PerformSimulationStep refreshes after every call that took a step:
  /// TerrainData as RGBA32F, the RG16F flow map, and `mipLevels` levels of
  /// TerrainData's mip pyramid in `mips`.  All null (the default) turns the
  /// refresh off.
  void SetTextureTargets(float* terrainRgba, uint16_t* flowmapRg16f, int mipLevels = 0,
                         float* mips = nullptr) {
    m_texRgba = terrainRgba;
    m_texFlowmap = flowmapRg16f;
    m_texMipLevels = mips ? mipLevels : 0;
    m_texMips = mips;
  }

  /// Advance exactly n steps.
  void Step(int n) { check(tws_step(m_grid, n), m_grid); }

  /// Terrain::ApplyRadialWaterBrush (Terrain.cpp:150-168): the world position
  /// is wrapped into the grid (fraction part of position / world size), the
  /// brush has BrushSizeSq 32 and intensity `strength`.
  void ApplyRadialWaterBrush(float worldX, float worldZ, float strength) {
    float px = worldX / m_gridWorldSize, pz = worldZ / m_gridWorldSize;
    px = px - std::trunc(px);
    pz = pz - std::trunc(pz);
    tws_source s;
    s.kind = TWS_SOURCE_BRUSH;
    s.cx = px * (float)m_gridResolution;
    s.cy = pz * (float)m_gridResolution;
    s.radius = 32.0f;
    s.rate = strength;
    check(tws_apply_source(m_grid, &s), m_grid);
  }

  /// Per-step sources (the benchmark's rain); not in the reference.
  void SetRain(const tws_source* sources, int n) { check(tws_set_sources(m_grid, sources, n), m_grid); }

  // ---- getters / setters (Terrain.h:76-83, Terrain.cpp:175-198)
  float GetTerrainWorldSize() const { return m_gridWorldSize; }
  /// As Terrain.h:76 computes it: 1/step + 0.5 as a float.
  float GetSimulationStepsPerSecond() const {
    return static_cast<float>(1.0f / m_simulationStepLength + 0.5f);
  }
  void SetSimulationStepsPerSecond(float simulationStepsPerSecond) {
    m_stepsPerSecond = simulationStepsPerSecond;
    m_simulationStepLength = (double)(1.0f / simulationStepsPerSecond);
    UpdateSimulationParameters();
  }
  float GetFlowDamping() const { return m_flowDamping; }
  void SetFlowDamping(float flowDamping) {
    m_flowDamping = flowDamping;
    UpdateSimulationParameters();
  }
  float GetFlowAcceleration() const { return m_flowAcceleration; }
  void SetFlowAcceleration(float flowAcceleration) {
    m_flowAcceleration = flowAcceleration;
    UpdateSimulationParameters();
  }

  /// Device buffers the renderer reads (Terrain.cpp:288, 323-330).
  tws_buffers GetBuffers() const {
    tws_buffers b;
    check(tws_get_buffers(m_grid, &b), m_grid);
    return b;
  }
  double TotalWaterVolume() {
    double v = 0.0;
    check(tws_volume(m_grid, &v), m_grid);
    return v;
  }
  void Download(float* depth, float* flux, float* velocity) {
    check(tws_download(m_grid, depth, flux, velocity), m_grid);
  }
  void Sync() { check(tws_sync(m_grid), m_grid); }
  tws_grid* Handle() { return m_grid; }

 private:
  // Re-derives all three per-step constants, as the reference's setters do.
  void UpdateSimulationParameters() {
    tws_sim_params p;
    check(tws_params_reference(m_stepsPerSecond, m_flowDamping, m_flowAcceleration, m_gridWorldSize,
                               m_gridResolution, m_boundary, &p));
    check(tws_set_params(m_grid, &p), m_grid);
  }

  tws_grid* m_grid = nullptr;
  unsigned m_gridResolution;
  float m_gridWorldSize;
  int m_boundary;
  float m_stepsPerSecond;
  double m_simulationStepLength;  // seconds, as ezTime holds it
  float m_flowDamping;
  float m_flowAcceleration;
  double m_timeSinceLastSimulationStep;
  float m_heightScale = 300.0f;  // Terrain.cpp:25
  int m_noiseScenes = 0;         // noise tables drawn so far
  // texture targets PerformSimulationStep refreshes (none by default)
  float* m_texRgba = nullptr;
  uint16_t* m_texFlowmap = nullptr;
  int m_texMipLevels = 0;
  float* m_texMips = nullptr;
};

}  // namespace tws
