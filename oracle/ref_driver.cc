// Stepwise driver over the reference's own FluidSimulation class -- test
// infrastructure only (builds into oracle/_ref/, never shipped).
//
// Compiled by oracle/Makefile together with the UNMODIFIED reference sources
// engine/physics/physicsWorld.cc and engine/core/random.cc of
// Allkams/Fluid-Simulation-3D. Private members are reached by compiling this
// translation unit with `private` defined as `public` around the reference
// header; the reference translation unit itself is compiled as is.
//
// Usage:  ref_driver <mode> <in.bin> <out.bin>
//   mode "substep": one substep decomposed into the reference's own phases:
//       prediction (physicsWorld.cc:42-48), UpdateSpatialLookup (:466-498),
//       updateDensities (:304-311), exact pressure acceleration through
//       CalculatePressureForce (:367-422) with the velocity zeroed and dt=1,
//       the real pressure pass, Jacobi viscosity through
//       CalculateViscosityForce (:424-464) with save/restore, and the
//       integrate/collision block of Update (:81-108) restated.
//       With flag bit 0 set the lookup is re-sorted stably by (key, index)
//       before the density pass, giving the canonical bucket order.
//   mode "update": `steps` calls of the reference's Update(dt) (Gauss-Seidel
//       viscosity, the reference's own sort), timing each call.
//   mode "init": the reference's own InitializeData(n) (physicsWorld.cc:
//       112-147 with GridArrangement :518-557), nothing loaded over it.
//   mode "speed": getSpeed(i) and getSpeedNormalzied(i) (physicsWorld.cc:
//       172-182) of the loaded velocities for i = 0..n (i = n is out of range).
//
// in.bin : u32 magic 'SPHI', u32 n, u32 steps, u32 flags,
//          f32 radius, rho0, k, kn, mu, gscale, gravity_on, bx, by, bz, dt,
//          f32 pos[3n], f32 vel[3n]
// out.bin (substep): u32 hash[n], key[n], start[n], lookup_id[n];
//          f32 lookup_raw[3n] (spatialLookup after std::sort),
//          f32 pred[3n], dens[2n], acc_p[3n], vel_p[3n], vel_v[3n],
//          pos[3n], vel[3n]
// out.bin (update):  f32 pos[3n], vel[3n], dens[2n], f64 ms[steps],
//          f64 phase_ms[6] (last step's reference timers)
// out.bin (init):    f32 pos[3n], f32 out_w[n] (OutPositions.w)
// out.bin (speed):   f32 speed[n+1], f32 speed_normalized[n+1]
#include <algorithm>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "config.h"
#define private public
#include "physics/physicsWorld.h"
#undef private

using Physics::Fluid::FluidSimulation;

namespace {

struct Header {
  uint32_t magic, n, steps, flags;
  float radius, rho0, k, kn, mu, gscale, gravity_on, bx, by, bz, dt;
};

template <typename T> void Put(FILE* f, const std::vector<T>& v) {
  if (!v.empty()) fwrite(v.data(), sizeof(T), v.size(), f);
}

void Configure(FluidSimulation& S, const Header& h) {
  S.setInteractionRadius(h.radius);
  S.setDensityTarget(h.rho0);
  S.setPressureMultiplier(h.k);
  S.setNearPressureMultiplier(h.kn);
  S.setViscosityStrength(h.mu);
  S.setGravityScale(h.gscale);
  S.setGravity(h.gravity_on != 0.0f);
  S.setBound(glm::vec3(h.bx, h.by, h.bz));
}

// Replaces InitializeData's lattice with the given state (the public
// `positions` buffer, physicsWorld.h:79, and the zeroed velocity, :133).
void Load(FluidSimulation& S, const Header& h, const std::vector<float>& pos,
          const std::vector<float>& vel) {
  S.InitializeData(static_cast<int>(h.n));
  for (uint32_t i = 0; i < h.n; ++i) {
    S.positions[i] = glm::vec3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
    S.velocity[i] = glm::vec3(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]);
  }
}

int Substep(FluidSimulation& S, const Header& h, FILE* out) {
  const uint32_t n = h.n;
  const float dt = h.dt;
  // Prediction, physicsWorld.cc:42-48 (same statements, serial).
  for (uint32_t i = 0; i < n; ++i) {
    S.velocity[i] += S.CalculateExternalFoce(S.positions[i], S.velocity[i]) * dt;
    S.predictedPositions[i] = S.positions[i] + S.velocity[i] * (1.0f / 120.0f);
  }
  S.UpdateSpatialLookup();
  std::vector<float> lookupRaw(3 * n);
  for (uint32_t s = 0; s < n; ++s) {
    lookupRaw[3 * s] = S.spatialLookup[s].x;
    lookupRaw[3 * s + 1] = S.spatialLookup[s].y;
    lookupRaw[3 * s + 2] = S.spatialLookup[s].z;
  }
  if (h.flags & 1u) {
    std::stable_sort(S.spatialLookup.begin(), S.spatialLookup.end(),
                     [](const glm::vec3& a, const glm::vec3& b) {
                       return a.z < b.z || (a.z == b.z && a.x < b.x);
                     });
  }
  std::vector<uint32_t> hash(n), key(n), start(n), lid(n);
  for (uint32_t i = 0; i < n; ++i) {
    hash[i] = S.HashCell(S.PositionToCellCoord(S.predictedPositions[i]));
    key[i] = S.GetKeyFromHash(hash[i], n);
    start[i] = S.startIndices[i];
  }
  for (uint32_t s = 0; s < n; ++s) lid[s] = static_cast<uint32_t>(S.spatialLookup[s].x);
  std::vector<float> pred(3 * n);
  for (uint32_t i = 0; i < n; ++i)
    for (int c = 0; c < 3; ++c) pred[3 * i + c] = S.predictedPositions[i][c];

  S.updateDensities();
  std::vector<float> dens(2 * n);
  for (uint32_t i = 0; i < n; ++i) {
    dens[2 * i] = S.densities[i].x;
    dens[2 * i + 1] = S.densities[i].y;
  }
  // Exact pressure acceleration: zero the velocity, dt = 1, restore.
  std::vector<float> accP(3 * n);
  for (uint32_t i = 0; i < n; ++i) {
    glm::vec3 keep = S.velocity[i];
    S.velocity[i] = glm::vec3(0.0f);
    S.CalculatePressureForce(i, 1.0f);
    for (int c = 0; c < 3; ++c) accP[3 * i + c] = S.velocity[i][c];
    S.velocity[i] = keep;
  }
  // The real pressure pass (order-independent: pressure reads no velocity).
  for (uint32_t i = 0; i < n; ++i) S.CalculatePressureForce(i, dt);
  std::vector<float> velP(3 * n);
  for (uint32_t i = 0; i < n; ++i)
    for (int c = 0; c < 3; ++c) velP[3 * i + c] = S.velocity[i][c];
  // Jacobi viscosity through the reference function: every call sees the
  // post-pressure snapshot; results are committed after the loop.
  std::vector<glm::vec3> snap(S.velocity.begin(), S.velocity.begin() + n);
  std::vector<glm::vec3> jac(n);
  for (uint32_t i = 0; i < n; ++i) {
    S.CalculateViscosityForce(i, dt);
    jac[i] = S.velocity[i];
    S.velocity[i] = snap[i];
  }
  for (uint32_t i = 0; i < n; ++i) S.velocity[i] = jac[i];
  std::vector<float> velV(3 * n);
  for (uint32_t i = 0; i < n; ++i)
    for (int c = 0; c < 3; ++c) velV[3 * i + c] = S.velocity[i][c];
  // Integrate and collide, restated from physicsWorld.cc:84-107.
  for (uint32_t i = 0; i < n; ++i) {
    S.positions[i] += S.velocity[i] * dt;
    const float dampFactor = 0.95f;
    const glm::vec3 halfSize = S.BoundScale * 0.5f;
    glm::vec3 edgeDst = halfSize - abs(S.positions[i]);
    if (edgeDst.x <= 0) {
      S.positions[i].x = halfSize.x * glm::sign(S.positions[i].x);
      S.velocity[i].x *= -1 * dampFactor;
    }
    if (edgeDst.y <= 0) {
      S.positions[i].y = halfSize.y * glm::sign(S.positions[i].y);
      S.velocity[i].y *= -1 * dampFactor;
    }
    if (edgeDst.z <= 0) {
      S.positions[i].z = halfSize.z * glm::sign(S.positions[i].z);
      S.velocity[i].z *= -1 * dampFactor;
    }
  }
  std::vector<float> posF(3 * n), velF(3 * n);
  for (uint32_t i = 0; i < n; ++i)
    for (int c = 0; c < 3; ++c) {
      posF[3 * i + c] = S.positions[i][c];
      velF[3 * i + c] = S.velocity[i][c];
    }
  Put(out, hash); Put(out, key); Put(out, start); Put(out, lid);
  Put(out, lookupRaw); Put(out, pred); Put(out, dens); Put(out, accP);
  Put(out, velP); Put(out, velV); Put(out, posF); Put(out, velF);
  return 0;
}

int Update(FluidSimulation& S, const Header& h, FILE* out) {
  const uint32_t n = h.n;
  std::vector<double> ms(h.steps);
  for (uint32_t s = 0; s < h.steps; ++s) {
    auto t0 = std::chrono::steady_clock::now();
    S.Update(h.dt);
    auto t1 = std::chrono::steady_clock::now();
    ms[s] = std::chrono::duration<double, std::milli>(t1 - t0).count();
  }
  std::vector<float> pos(3 * n), vel(3 * n), dens(2 * n);
  for (uint32_t i = 0; i < n; ++i) {
    for (int c = 0; c < 3; ++c) {
      pos[3 * i + c] = S.positions[i][c];
      vel[3 * i + c] = S.velocity[i][c];
    }
    dens[2 * i] = S.densities[i].x;
    dens[2 * i + 1] = S.densities[i].y;
  }
  std::vector<double> phase = {S.getElapsedTimeGravity(),  S.getElapsedTimeSpatial(),
                               S.getElapsedTimeDensity(),  S.getElapsedTimePressure(),
                               S.getElapsedTimeViscosity(), S.getElapsedTimePosNColl()};
  Put(out, pos); Put(out, vel); Put(out, dens); Put(out, ms); Put(out, phase);
  return 0;
}

int Init(FluidSimulation& S, const Header& h, FILE* out) {
  const uint32_t n = h.n;
  S.InitializeData(static_cast<int>(n));
  std::vector<float> pos(3 * n), w(n);
  for (uint32_t i = 0; i < n; ++i) {
    for (int c = 0; c < 3; ++c) pos[3 * i + c] = S.positions[i][c];
    w[i] = S.OutPositions[i].w;
  }
  Put(out, pos); Put(out, w);
  return 0;
}

int Speed(FluidSimulation& S, const Header& h, FILE* out) {
  std::vector<float> sp(h.n + 1), nrm(h.n + 1);
  for (uint32_t i = 0; i <= h.n; ++i) {
    sp[i] = S.getSpeed(i);
    nrm[i] = S.getSpeedNormalzied(i);
  }
  Put(out, sp); Put(out, nrm);
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc != 4) {
    fprintf(stderr, "usage: %s substep|update|init|speed in.bin out.bin\n", argv[0]);
    return 2;
  }
  const std::string mode = argv[1];
  FILE* in = fopen(argv[2], "rb");
  if (!in) { perror("in"); return 2; }
  Header h{};
  if (fread(&h, sizeof(h), 1, in) != 1 || h.magic != 0x49485053u || h.n == 0) {
    fprintf(stderr, "bad header\n");
    return 2;
  }
  std::vector<float> pos(3 * h.n), vel(3 * h.n);
  if (fread(pos.data(), sizeof(float), pos.size(), in) != pos.size() ||
      fread(vel.data(), sizeof(float), vel.size(), in) != vel.size()) {
    fprintf(stderr, "short input\n");
    return 2;
  }
  fclose(in);
  FluidSimulation& S = FluidSimulation::getInstance();
  Configure(S, h);
  if (mode != "init") Load(S, h, pos, vel);
  FILE* out = fopen(argv[3], "wb");
  if (!out) { perror("out"); return 2; }
  int rc = 2;
  if (mode == "substep") rc = Substep(S, h, out);
  else if (mode == "update") rc = Update(S, h, out);
  else if (mode == "init") rc = Init(S, h, out);
  else if (mode == "speed") rc = Speed(S, h, out);
  else fprintf(stderr, "unknown mode %s\n", mode.c_str());
  fclose(out);
  return rc;
}
