// Host-side engine: owns the device buffers of one or more scenes, keeps the
// layout bookkeeping (which slots each scene occupies), builds the tile tables
// of the segmented launches and runs the substep pipeline, optionally from a
// captured CUDA graph.
#pragma once

#include <cstdint>
#include <map>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/sph_gb300.h"
#include "sph_kernels.h"

namespace sph {

// A scene's state and settings as a snapshot file holds them (caller order).
struct SceneSnapshot {
  sph_params prm{};
  float dt = 0.0f;
  std::vector<float> pos, vel, dens;  // [3n], [3n], [2n]
};

class Engine {
 public:
  Engine(uint64_t capacity, uint32_t max_scenes);
  ~Engine();
  Engine(const Engine&) = delete;
  Engine& operator=(const Engine&) = delete;

  int Init();  // allocate device memory; SPH_OK or an error code

  int AddScene(const sph_params& p, uint32_t n, const float* pos3,
               const float* vel3, bool device_ptrs, float dt, uint32_t* id,
               cudaStream_t st);
  int RemoveScene(uint32_t id);
  int SetParams(uint32_t id, const sph_params& p);
  int GetParams(uint32_t id, sph_params* p) const;
  int SetDt(uint32_t id, float dt);
  int Load(uint32_t id, const float* pos3, const float* vel3, bool device_ptrs,
           cudaStream_t st);
  int Step(int substeps, cudaStream_t st);
  int Download(uint32_t id, float* pos3, float* vel3, float* dens2,
               bool device_ptrs, cudaStream_t st);
  int OutPositions(uint32_t id, void** dev_float4);
  // Snapshots (sph_snapshot.cu): write scene `id` to a file, read a file,
  // put a snapshot into an existing scene of the same size, or add it as a
  // new scene.
  int SaveSnapshot(uint32_t id, const char* path, cudaStream_t st);
  int ReadSnapshot(const char* path, SceneSnapshot* s);
  int RestoreSnapshot(uint32_t id, const SceneSnapshot& s, cudaStream_t st);
  int AddSnapshot(const SceneSnapshot& s, uint32_t* id, cudaStream_t st);
  // Headless render of scene `id`'s current state (sph_render); host outputs.
  int Render(uint32_t id, const sph_view& view, uint8_t* rgba, float* depth,
             cudaStream_t st);
  int DebugEnable(bool on);
  int DebugExport(uint32_t id, uint32_t* hash, uint32_t* key,
                  uint32_t* sorted_ids, uint32_t* start, float* dens2,
                  float* accp, float* velp, float* velv, cudaStream_t st);
  // The timed sort's own layout of the captured substep (the internal cell
  // index and key-table entry per particle, the particle at each slot, and
  // the scene's key table as slot offsets, table_len + 1 entries); the
  // table is copied only when start_cap holds it.
  int DebugExportLayout(uint32_t id, uint32_t* cell, uint32_t* key, uint32_t* slot_ids,
                        uint32_t* start, uint64_t start_cap, uint32_t* table_len,
                        int* direct, cudaStream_t st);
  int Status(uint32_t* flags, cudaStream_t st);

  int SetTuning(const sph_tuning& t);
  sph_tuning Tuning() const { return tuning_; }
  int Autotune(int substeps, int steps_per_trial, sph_tuning* best,
               float* best_ms, cudaStream_t st);

  // Per-phase device timing of each step (CUDA events on the launching
  // stream, also inside captured graphs).
  int ProfileEnable(bool on);
  int PhaseTimes(double out_ms[6]);
  uint64_t KernelLaunches() const { return launches_; }
  // Device bytes allocated per particle of capacity (Init's per-C arrays).
  static uint64_t BytesPerParticle();

  void UseGraphs(bool on) { use_graphs_ = on; }
  uint32_t NumScenes() const;
  uint64_t NumParticles() const;
  uint64_t Capacity() const { return capacity_; }
  uint32_t SceneSize(uint32_t id) const;
  const char* LastError() const { return err_.c_str(); }
  int Fail(int code, const std::string& msg);
  int CudaFail(cudaError_t e, const char* what);

 private:
  struct Scene {
    bool used = false;
    bool live = false;
    sph_params prm{};
    uint32_t n = 0;
    uint32_t base = 0;      // slots in the current layout
    float dt = 1.0f / 60.0f;
  };
  int BuildLayout(cudaStream_t st);
  int UploadScenes(int substeps, cudaStream_t st);
  int RunSubsteps(int substeps, cudaStream_t st, bool carry);
  void BuildTiles(std::vector<uint2>& out, bool old_layout) const;
  void ReleaseGraphs();

  uint64_t capacity_;
  uint32_t max_scenes_;
  std::vector<Scene> scenes_;
  std::vector<uint32_t> old_base_;  // per scene: base in the layout a step reads
  uint64_t layout_total_ = 0;       // slots occupied in the current layout
  // Free extents (base, length) of the current layout: the regions of scenes
  // removed since the last step compacted it. AddScene loads a new scene into
  // the first one that fits before it appends past the layout's end, so the
  // room a removed scene leaves is usable before the next step.
  std::vector<std::pair<uint64_t, uint64_t>> free_;
  uint32_t total_ = 0;              // live particles
  uint32_t table_total_ = 0;        // key-table entries of the live scenes
  std::vector<SceneDev> scene_dev_;  // host copy of the uploaded scene table
  int tables_ = kTablesMixed;       // their forms (TableForms)
  bool layout_dirty_ = true;
  bool scenes_dirty_ = true;
  int uploaded_substeps_ = -1;
  // The last substep of a step also predicts the next step's first substep
  // (key, rank and histogram, fused in its viscosity pass). carry_valid_:
  // nothing has changed since (state, settings, dt, layout), so the next
  // step skips k_predict_hash. count_extent_: keys whose histogram entries
  // that prediction wrote (cleared if it goes unused).
  bool carry_valid_ = false;
  uint32_t count_extent_ = 0;

  // device memory
  SceneDev* d_scenes_ = nullptr;
  uint2* d_tiles_old_ = nullptr;
  uint2* d_tiles_new_ = nullptr;
  uint32_t n_tiles_old_ = 0, n_tiles_new_ = 0;
  float4 *d_pos_[2] = {nullptr, nullptr}, *d_vel_[2] = {nullptr, nullptr};
  int cur_ = 0;  // index of the state buffers holding the current layout
  LaunchCtx ctx_{};
  float4* d_out4_ = nullptr;
  uint32_t* d_status_ = nullptr;

  // debug capture
  bool debug_ = false;
  bool debug_valid_ = false;
  uint32_t* d_dbg_hash_ = nullptr;
  uint32_t* d_dbg_key_ = nullptr;
  float4* d_dbg_accp_ = nullptr;
  float4* d_dbg_velv_ = nullptr;
  float4* d_dbg_velp_ = nullptr;
  uint32_t* d_dbg_start_ = nullptr;
  uint32_t* d_dbg_count_ = nullptr;
  uint32_t* d_dbg_partial_ = nullptr;
  uint2* d_dbg_keyrank_ = nullptr;
  uint32_t* d_dbg_tmp_ = nullptr;
  uint32_t* d_dbg_sorted_ = nullptr;
  void* d_dbg_scratch_ = nullptr;

  // render buffers, grown on demand: (depth, index) keys, RGBA8 and depth per
  // pixel, colour per particle
  unsigned long long* d_rkeys_ = nullptr;
  uint32_t* d_rrgba_ = nullptr;
  float* d_rdepth_ = nullptr;
  uint32_t* d_rcolour_ = nullptr;
  uint64_t render_pixels_ = 0;

  // Neighbour-list capacity per particle (pairs with dist <= r); a particle
  // with more neighbours is handled by the bucket walk in the force passes.
  static constexpr uint32_t kNbrCap = 64;
  sph_tuning tuning_{128, 1, 32, 2, 0, 0};
  int sm_count_ = 0;

  // The substep pipeline runs on an engine-owned non-blocking stream (stream
  // capture is not allowed on the legacy default stream), joined to the
  // caller's stream by events before and after each step.
  cudaStream_t work_ = nullptr;
  cudaEvent_t join_in_ = nullptr, join_out_ = nullptr;

  // CUDA graphs, keyed by (substeps, state parity + 2 * carried prediction)
  bool use_graphs_ = true;
  std::map<std::pair<int, int>, cudaGraphExec_t> graphs_;

  // profiling: kPhaseEvents events per substep, kMaxSubsteps substeps
  static constexpr int kPhaseEvents = 6;
  static constexpr int kMaxSubsteps = 64;
  bool profile_ = false;
  int profiled_substeps_ = 0;
  std::vector<cudaEvent_t> prof_ev_;
  uint64_t launches_ = 0;

  std::string err_;
};

}  // namespace sph
