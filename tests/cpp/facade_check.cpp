// Drives the C++ facade (include/tws_watersim.hpp) the way the reference's
// scene drives Terrain (Scene.cpp:354-364): brush strokes and frame-time
// driven PerformSimulationStep calls.  Prints the state for the Python test
// to compare with the oracle.
#include <cuda_runtime_api.h>

#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "tws_watersim.hpp"

// Mode "textures": texture targets set on the facade; one frame that takes a
// step refreshes TerrainData, its mips and the flow map, then the buffers are
// cleared and a frame that takes no step must leave them clear.  Writes the
// depth and the refreshed textures, then the textures after the idle frame.
static int texture_refresh(unsigned N, const char* out) {
  tws::WaterSim sim(N, (float)N);
  sim.CreateHeightmapFromNoiseAndResetSim(91, 40.0f, 15.0f);
  int levels = 0;
  size_t texels = 0;
  for (unsigned w = N; w >= 2; w /= 2) texels += (size_t)(w / 2) * (w / 2), ++levels;
  const size_t cells = (size_t)N * N;
  float *rgba = nullptr, *mips = nullptr;
  uint16_t* flow = nullptr;
  if (cudaMalloc(reinterpret_cast<void**>(&rgba), cells * 16) != cudaSuccess ||
      cudaMalloc(reinterpret_cast<void**>(&mips), texels * 16) != cudaSuccess ||
      cudaMalloc(reinterpret_cast<void**>(&flow), cells * 4) != cudaSuccess)
    return 4;
  sim.SetTextureTargets(rgba, flow, levels, mips);
  const unsigned n = sim.PerformSimulationStep(0.025);  // one 1/60 s step
  sim.Sync();
  std::vector<float> d(cells), h_rgba(cells * 4), h_mips(texels * 4);
  std::vector<uint16_t> h_flow(cells * 2);
  sim.Download(d.data(), nullptr, nullptr);
  FILE* fh = std::fopen(out, "wb");
  if (!fh) return 2;
  std::fwrite(&n, sizeof(n), 1, fh);
  std::fwrite(d.data(), 4, d.size(), fh);
  for (int pass = 0; pass < 2; ++pass) {
    if (cudaMemcpy(h_rgba.data(), rgba, cells * 16, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(h_mips.data(), mips, texels * 16, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(h_flow.data(), flow, cells * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
      return 5;
    std::fwrite(h_rgba.data(), 4, h_rgba.size(), fh);
    std::fwrite(h_mips.data(), 4, h_mips.size(), fh);
    std::fwrite(h_flow.data(), 2, h_flow.size(), fh);
    if (pass == 0) {  // clear, then a frame too short for a step
      cudaMemset(rgba, 0, cells * 16);
      cudaMemset(mips, 0, texels * 16);
      cudaMemset(flow, 0, cells * 4);
      cudaDeviceSynchronize();
      if (sim.PerformSimulationStep(0.001) != 0) return 6;
      sim.Sync();
    }
  }
  std::fclose(fh);
  cudaFree(rgba);
  cudaFree(mips);
  cudaFree(flow);
  return 0;
}

// Mode "reference": the reference's own reset, called twice (the second call
// draws the next noise table, as in the reference application); writes the
// terrain and depth after the second call.
static int reference_reset(unsigned N, const char* out) {
  tws::WaterSim sim(N, (float)N);
  sim.CreateHeightmapFromNoiseAndResetSim();
  sim.CreateHeightmapFromNoiseAndResetSim();
  sim.Sync();
  std::vector<float> b((size_t)N * N), d((size_t)N * N);
  if (tws_download_terrain(sim.Handle(), b.data()) != TWS_OK) return 3;
  sim.Download(d.data(), nullptr, nullptr);
  FILE* fh = std::fopen(out, "wb");
  if (!fh) return 2;
  std::fwrite(b.data(), 4, b.size(), fh);
  std::fwrite(d.data(), 4, d.size(), fh);
  std::fclose(fh);
  return 0;
}

int main(int argc, char** argv) {
  const unsigned N = argc > 1 ? (unsigned)std::atoi(argv[1]) : 128;
  const char* out = argc > 2 ? argv[2] : "facade_out.bin";
  if (argc > 3 && std::string(argv[3]) == "textures") {
    try {
      return texture_refresh(N, out);
    } catch (const tws::Error& e) {
      std::fprintf(stderr, "tws error %d: %s\n", e.code(), e.what());
      return 1;
    }
  }
  if (argc > 3 && std::string(argv[3]) == "reference") {
    try {
      return reference_reset(N, out);
    } catch (const tws::Error& e) {
      std::fprintf(stderr, "tws error %d: %s\n", e.code(), e.what());
      return 1;
    }
  }
  try {
    tws::WaterSim sim(N, (float)N);
    sim.CreateHeightmapFromNoiseAndResetSim(77, 40.0f, 15.0f);
    sim.SetFlowDamping(0.97f);
    sim.SetFlowAcceleration(20.0f);
    unsigned total = 0;
    // 1/60 s steps; frames of 25 ms and one 400 ms stall (clamped to 10 steps)
    const double frames[] = {0.025, 0.025, 0.4, 0.025, 0.010, 0.030};
    for (int i = 0; i < 6; ++i) {
      if (i == 1) sim.ApplyRadialWaterBrush(0.3f * N + 5.0f * N, 0.6f * N, 4.0f);
      total += sim.PerformSimulationStep(frames[i]);
    }
    sim.Sync();
    std::vector<float> d((size_t)N * N), f((size_t)N * N * 4), v((size_t)N * N * 2);
    sim.Download(d.data(), f.data(), v.data());
    FILE* fh = std::fopen(out, "wb");
    if (!fh) return 2;
    std::fwrite(&total, sizeof(total), 1, fh);
    std::fwrite(d.data(), 4, d.size(), fh);
    std::fwrite(f.data(), 4, f.size(), fh);
    std::fwrite(v.data(), 4, v.size(), fh);
    std::fclose(fh);
    std::printf("steps %u volume %.6f sps %.2f\n", total, sim.TotalWaterVolume(),
                sim.GetSimulationStepsPerSecond());
  } catch (const tws::Error& e) {
    std::fprintf(stderr, "tws error %d: %s\n", e.code(), e.what());
    return 1;
  }
  return 0;
}
