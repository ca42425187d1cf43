// Drives the C++ mirror of the reference's FluidSimulation / FluidSimBase
// through libsph_gb300.so the way projects/Simulation drives FluidSimCPU:
// initialize, tweak settings, update, read particles back.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "sph_fluid_simulation.hpp"

static_assert(sizeof(sph::Vec3) == 12, "Vec3 must be three packed floats");

int main() {
  sph::FluidSimCUDA plugin(3);
  auto& sim = plugin.simulation();
  sim.setGravity(true);
  sim.setGravityScale(9.81f);
  sim.setInteractionRadius(0.35f);
  sim.setDensityTarget(55.0f);
  sim.setPressureMultiplier(500.0f);
  sim.setNearPressureMultiplier(18.0f);
  sim.setViscosityStrength(0.06f);
  sim.setBound({6.0f, 6.0f, 6.0f});
  plugin.initialize(4096);
  sim.setProfiling(true);
  for (int k = 0; k < 10; ++k) plugin.update(1.0f / 60.0f);
  double rho = 0.0;
  for (uint32_t i = 0; i < sim.numParticles(); ++i) {
    const float d = sim.getDensity(i);
    const sph::Vec3 p = sim.getPosition(i);
    if (!(d > 0.0f) || !std::isfinite(p.x) || std::fabs(p.y) > 3.0f) {
      std::printf("bad particle %u: density %g y %g\n", i, d, p.y);
      return 1;
    }
    rho += d;
  }
  if (sim.getDensity(1u << 30) != 0.0f) return 2;  // out of range -> 0
  if (plugin.render() == nullptr) return 3;
  if (sim.OutPositions.size() != sim.numParticles() || sim.OutPositions[7].w != 0.34f)
    return 4;
  // snapshot: save, move on, load back -> the saved state again
  const sph::Vec3 p7 = sim.getPosition(7);
  const char* snap = std::getenv("SPH_SNAPSHOT_PATH");
  const std::string path = snap ? snap : "fluid_sim_host.sph";
  sim.Save(path);
  for (int k = 0; k < 3; ++k) plugin.update(1.0f / 60.0f);
  sim.Load(path);
  const sph::Vec3 q7 = sim.getPosition(7);
  if (q7.x != p7.x || q7.y != p7.y || q7.z != p7.z) return 5;
  // a frame from a camera on the +z axis looking at the origin (perspective,
  // 90 degrees, as the app's Camera)
  const float P[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, -1.0002f, -1, 0, 0, -0.020002f, 0};
  float V[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, -8, 1};  // eye at z = 8
  float VP[16];
  for (int c = 0; c < 4; ++c)
    for (int r = 0; r < 4; ++r) {
      float acc = 0;
      for (int k = 0; k < 4; ++k) acc += P[k * 4 + r] * V[c * 4 + k];
      VP[c * 4 + r] = acc;
    }
  std::vector<uint8_t> rgba;
  std::vector<float> depth;
  plugin.render(VP, P, 256, 256, rgba, &depth);
  size_t drawn = 0;
  for (float d : depth) drawn += d < 1.0f;
  if (drawn == 0 || rgba.size() != 4u * 256 * 256) return 6;
  std::printf("ok n=%u mean density %.3f density phase %.4f ms, %zu pixels drawn\n",
              sim.numParticles(), rho / sim.numParticles(), sim.getElapsedTimeDensity(),
              drawn);
  return 0;
}
