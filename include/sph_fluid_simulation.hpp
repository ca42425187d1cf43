// Header-only C++ mirror of the reference's simulation class and plug-in,
// built on the C ABI of sph_gb300.h.
//
//  * sph::FluidSimulation keeps the method names, defaults and argument
//    meaning of Physics::Fluid::FluidSimulation
//    (engine/physics/physicsWorld.h:28-155): Update, InitializeData, the
//    per-particle getters (0 for an out-of-range index, physicsWorld.cc:149-
//    182), the elapsed-time getters, and every setter/getter pair of the
//    settings surface (physicsWorld.cc:214-302). The public `positions` and
//    `OutPositions` vectors are host mirrors refreshed after each Update.
//  * sph::FluidSimCUDA has the shape of FluidSimBase
//    (projects/Simulation/code/simulations/fluidSimBase.h:5-14); render()
//    hands out the headless device buffer of (position, 0.34) per particle.
//
// Differences from the reference, by design: no singleton (construct as many
// as needed), Jacobi viscosity, Update(dt, substeps) = `substeps` reference
// Updates of dt/substeps, and failures throw std::runtime_error carrying the
// library's message instead of being silent.
#pragma once

#include <array>
#include <cmath>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "sph_gb300.h"

namespace sph {

struct Vec3 {
  float x = 0, y = 0, z = 0;
};
struct Vec4 {
  float x = 0, y = 0, z = 0, w = 0;
};

// The default lattice of InitializeData (physicsWorld.cc:139-142) with
// GridArrangement (physicsWorld.cc:518-557): ceil(n^(1/3)) particles a side
// at `gap`, centred on the origin, y layers from the top, then x, then z;
// the first n points.
inline std::vector<Vec3> GridArrangement(uint32_t n, float gap = 0.215f) {
  const int per_axis =
      static_cast<int>(std::ceil(std::pow(static_cast<float>(n), 1.0f / 3.0f)));
  std::vector<Vec3> out(n);
  uint32_t i = 0;
  const float total = per_axis * gap;
  const float ox = 0 - ((total - gap) / 2.0f);
  const float oy = 0 + (total - gap) / 2.0f;
  const float oz = 0 - (total - gap) / 2.0f;
  for (int ly = 0; ly < per_axis; ++ly)
    for (int lx = 0; lx < per_axis; ++lx)
      for (int lz = 0; lz < per_axis; ++lz) {
        if (i >= n) return out;
        out[i++] = Vec3{ox + lx * gap, oy - ly * gap, oz + lz * gap};
      }
  return out;
}

// getSpeed / getSpeedNormalzied (physicsWorld.cc:172-182): glm::length, i.e.
// sqrt((x*x + y*y) + z*z), and clamp(|v|, 0, 1.5) / 1.5.
inline float SpeedOf(const Vec3& v) { return std::sqrt((v.x * v.x + v.y * v.y) + v.z * v.z); }
inline float SpeedNormalized(const Vec3& v) {
  const float s = SpeedOf(v);
  return (s < 0.0f ? 0.0f : (s > 1.5f ? 1.5f : s)) / 1.5f;
}

class FluidSimulation {
 public:
  FluidSimulation() { sph_default_params(&prm_); }
  ~FluidSimulation() { Close(); }
  FluidSimulation(const FluidSimulation&) = delete;
  FluidSimulation& operator=(const FluidSimulation&) = delete;

  // physicsWorld.cc:112-147: size the buffers, zero the velocities and lay
  // out the default cube lattice (RowSize = ceil(N^(1/3)), gap 0.215,
  // GridArrangement :518-557) unless positions are given.
  void InitializeData(int particleAmmount, const std::vector<Vec3>* init = nullptr) {
    Close();
    if (particleAmmount <= 0) throw std::invalid_argument("particle count must be positive");
    n_ = static_cast<uint32_t>(particleAmmount);
    Check(sph_create(&prm_, n_, &h_), nullptr);
    positions.assign(n_, Vec3{});
    velocity_.assign(n_, Vec3{});
    densities_.assign(2 * static_cast<size_t>(n_), 0.0f);
    if (init) {
      if (init->size() != n_) throw std::invalid_argument("position count mismatch");
      positions = *init;
    } else {
      positions = sph::GridArrangement(n_);
    }
    Upload();
  }

  // physicsWorld.cc:39-111 run `substeps` times with deltatime/substeps.
  void Update(float deltatime, int substeps = 1) {
    Require();
    Check(sph_step(h_, deltatime, substeps, stream_), h_);
    Download();
  }

  // Write `positions` / velocities back to the device (after editing them).
  void Upload() {
    Require();
    Check(sph_upload(h_, &positions[0].x, &velocity_[0].x, stream_), h_);
  }

  Vec3 getPosition(uint32_t i) const { return i < n_ ? positions[i] : Vec3{}; }
  Vec3 getVelocity(uint32_t i) const { return i < n_ ? velocity_[i] : Vec3{}; }
  float getDensity(uint32_t i) const { return i < n_ ? densities_[2 * i] : 0.0f; }
  float getNearDensity(uint32_t i) const { return i < n_ ? densities_[2 * i + 1] : 0.0f; }
  float getSpeed(uint32_t i) const { return i < n_ ? SpeedOf(velocity_[i]) : 0.0f; }
  float getSpeedNormalzied(uint32_t i) const {
    return i < n_ ? SpeedNormalized(velocity_[i]) : 0.0f;
  }

  // Device time per phase of the last Update in ms (CUDA events) when
  // profiling is on: setProfiling(true).
  void setProfiling(bool on) {
    Require();
    Check(sph_profile_enable(h_, on ? 1 : 0), h_);
    profiling_ = on;
  }
  double getElapsedTimeGravity() { return Phase(0); }
  double getElapsedTimeSpatial() { return Phase(1); }
  double getElapsedTimeDensity() { return Phase(2); }
  double getElapsedTimePressure() { return Phase(3); }
  double getElapsedTimeViscosity() { return Phase(4); }
  double getElapsedTimePosNColl() { return Phase(5); }

  void setSimulationTime(float t) { simTime_ = t; }
  float getSimulationTime() const { return simTime_; }
  void setGravity(bool on) { prm_.gravity_on = on ? 1 : 0; Push(); }
  bool getGravityStatus() const { return prm_.gravity_on != 0; }
  void setInteractionRadius(float v) { prm_.radius = v; Push(); }
  float getInteractionRadius() const { return prm_.radius; }
  void setDensityTarget(float v) { prm_.target_density = v; Push(); }
  float getDensityTarget() const { return prm_.target_density; }
  void setPressureMultiplier(float v) { prm_.pressure_mult = v; Push(); }
  float getPressureMultiplier() const { return prm_.pressure_mult; }
  void setNearPressureMultiplier(float v) { prm_.near_pressure_mult = v; Push(); }
  float getNearPressureMultiplier() const { return prm_.near_pressure_mult; }
  void setViscosityStrength(float v) { prm_.viscosity = v; Push(); }
  float getViscosityStrength() const { return prm_.viscosity; }
  void setGravityScale(float v) { prm_.gravity_scale = v; Push(); }
  float getGravityScale() const { return prm_.gravity_scale; }
  void setBound(const Vec3& b) {
    prm_.bound[0] = b.x; prm_.bound[1] = b.y; prm_.bound[2] = b.z;
    Push();
  }
  Vec3 getBounds() const { return Vec3{prm_.bound[0], prm_.bound[1], prm_.bound[2]}; }
  // Constants the reference hard-codes (physicsWorld.cc:47,87).
  void setCollisionDamping(float v) { prm_.damping = v; Push(); }
  void setPredictionDt(float v) { prm_.predict_dt = v; Push(); }

  // Snapshot of the state and settings (sph_save / sph_load); Load needs a
  // file of this simulation's particle count and refreshes the host mirrors.
  void Save(const std::string& path) {
    Require();
    Check(sph_save(h_, path.c_str(), stream_), h_);
  }
  void Load(const std::string& path) {
    Require();
    Check(sph_load(h_, path.c_str(), stream_), h_);
    Check(sph_get_params(h_, &prm_), h_);
    Download();
  }

  // Headless frame (sph_render): rgba gets 4 * width * height bytes, depth
  // (optional) width * height floats, rows bottom to top.
  void Render(const sph_view& view, std::vector<uint8_t>& rgba,
              std::vector<float>* depth = nullptr) {
    Require();
    rgba.resize(4ull * view.width * view.height);
    if (depth) depth->resize(static_cast<size_t>(view.width) * view.height);
    Check(sph_render(h_, &view, rgba.data(), depth ? depth->data() : nullptr, stream_), h_);
  }

  uint32_t numParticles() const { return n_; }
  sph_sim* handle() const { return h_; }
  void setStream(void* s) { stream_ = s; }

  // Host mirrors of the reference's public buffers (physicsWorld.h:79-80).
  std::vector<Vec3> positions;
  std::vector<Vec4> OutPositions;

 private:
  void Close() {
    if (h_) sph_destroy(h_);
    h_ = nullptr;
  }
  void Require() const {
    if (!h_) throw std::logic_error("InitializeData has not been called");
  }
  static void Check(int rc, const sph_sim* h) {
    if (rc != SPH_OK)
      throw std::runtime_error(std::string("sph_gb300: ") +
                               (h ? sph_last_error(h) : sph_global_error()));
  }
  void Push() {
    if (h_) Check(sph_set_params(h_, &prm_), h_);
  }
  void Download() {
    Check(sph_download(h_, &positions[0].x, &velocity_[0].x, densities_.data(), stream_), h_);
    OutPositions.resize(n_);
    for (uint32_t i = 0; i < n_; ++i)
      OutPositions[i] = Vec4{positions[i].x, positions[i].y, positions[i].z, 0.34f};
  }
  double Phase(int k) {
    if (!h_ || !profiling_) return 0.0;
    std::array<double, 6> ms{};
    if (sph_phase_times(h_, ms.data()) != SPH_OK) return 0.0;
    return ms[k];
  }
  sph_params prm_{};
  sph_sim* h_ = nullptr;
  uint32_t n_ = 0;
  void* stream_ = nullptr;
  bool profiling_ = false;
  float simTime_ = 0.0f;
  std::vector<Vec3> velocity_;
  std::vector<float> densities_;
};

// FluidSimBase-shaped plug-in: the app calls initialize / update / reset /
// cleanup / render exactly as it drives FluidSimCPU
// (projects/Simulation/code/simulations/fluidSimCPU.cc:9-93).
class FluidSimCUDA {
 public:
  explicit FluidSimCUDA(int substeps = 1) : substeps_(substeps) {}
  FluidSimulation& simulation() { return sim_; }
  void initialize(int particleAmount) {
    nrParticles_ = particleAmount;
    sim_.InitializeData(particleAmount);
  }
  void update(float dt) { sim_.Update(dt, substeps_); }
  void reset() { sim_.InitializeData(nrParticles_); }
  void cleanup() {}
  // Headless render: device address of float4[n] = (position, 0.34), the
  // buffer FluidSimCPU uploads to its GL SSBO each frame.
  const void* render() {
    void* p = nullptr;
    if (sph_out_positions(sim_.handle(), &p) != SPH_OK) return nullptr;
    return p;
  }
  // The frame FluidSimCPU::render draws (fluidSimCPU.cc:53-93) for a camera:
  // view_proj = cam.GetViewProjection(), proj = cam.GetProjection()
  // (column-major, glm::value_ptr), cleared to black as the app does.
  void render(const float* view_proj, const float* proj, uint32_t width, uint32_t height,
              std::vector<uint8_t>& rgba, std::vector<float>* depth = nullptr) {
    sph_view v{};
    for (int k = 0; k < 16; ++k) {
      v.view_proj[k] = view_proj[k];
      v.proj[k] = proj[k];
    }
    v.width = width;
    v.height = height;
    v.scale = 0.34f;
    v.clear[3] = 1.0f;
    sim_.Render(v, rgba, depth);
  }

 private:
  FluidSimulation sim_;
  int substeps_;
  int nrParticles_ = 0;
};

}  // namespace sph
