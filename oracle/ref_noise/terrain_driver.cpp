// terrain_driver.cpp -- drives the reference's own Random and NoiseGenerator
// (compiled from their source files, see the Makefile's `ref` target) the way
// Terrain::CreateHeightmapFromNoiseAndResetSim does (Terrain.cpp:200-222), so
// the oracle's restatement of that scene can be checked against the reference
// code.  TEST INFRASTRUCTURE only.
//
// Terrain.cpp's loop needs the GL texture classes, so its per-cell formula is
// restated here (the noise itself is the reference's code):
//   b = (noise(x m, y m, 0; octaves 2..10, persistence 0.43, periodic) * 0.5 + 0.5) * hs
//   d = max(0, (0.45 - pow(|(x m - 0.5, y m - 0.5)|^2, 2) * 800) * hs - b),  m = 1 / (N - 1)
#include <cmath>
#include <vector>

#include "ez_shim.h"
#include "NoiseGenerator.h"
#include "Random.h"

extern "C" {

// The reference's white-noise table after Random::Init(seed) and `generation`
// earlier NoiseGenerator constructions (each takes 4096 numbers).
void tws_ref_noise_table(unsigned seed, int generation, float* out4096) {
  Random::Init(seed);
  for (int g = 0; g < generation; ++g)
    for (int i = 0; i < 4096; ++i) Random::NextFloat();
  for (int i = 0; i < 4096; ++i) out4096[i] = Random::NextFloat();
}

void tws_ref_reference_terrain(unsigned seed, int generation, int N, float height_scale, float* b,
                               float* d) {
  Random::Init(seed);
  for (int g = 0; g < generation; ++g) NoiseGenerator skipped;
  NoiseGenerator noiseGen;
  const float m = 1.0f / static_cast<float>(N - 1);
  for (int y = 0; y < N; ++y)
    for (int x = 0; x < N; ++x) {
      const float bb =
          (noiseGen.GetValueNoise(ezVec3(m * x, m * y, 0.0f), 2, 10, 0.43f, true, nullptr) * 0.5f +
           0.5f) *
          height_scale;
      const float ex = x * m - 0.5f, ey = y * m - 0.5f;
      const float len2 = ex * ex + ey * ey;
      b[x + y * N] = bb;
      d[x + y * N] = std::max(0.0f, (0.45f - std::pow(len2, 2.0f) * 800.0f) * height_scale - bb);
    }
}

}  // extern "C"
