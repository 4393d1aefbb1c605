// Drives the C++ facade (include/tws_watersim.hpp) the way the reference's
// scene drives Terrain (Scene.cpp:354-364): brush strokes and frame-time
// driven PerformSimulationStep calls.  Prints the state for the Python test
// to compare with the oracle.
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "tws_watersim.hpp"

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
