// Drives the C++ mirror of the reference's FluidSimulation / FluidSimBase
// through libsph_gb300.so the way projects/Simulation drives FluidSimCPU:
// initialize, tweak settings, update, read particles back.
#include <cmath>
#include <cstdio>

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
  std::printf("ok n=%u mean density %.3f density phase %.4f ms\n", sim.numParticles(),
              rho / sim.numParticles(), sim.getElapsedTimeDensity());
  return 0;
}
