// extern "C" boundary of libsph_gb300.so (declared in include/sph_gb300.h).
//
// The single-scene handle is an engine holding one scene; the batch handle
// exposes the engine's scene table directly.
#include <new>
#include <string>

#include "../../include/sph_gb300.h"
#include "sph_engine.h"

struct sph_sim {
  sph::Engine eng;
  uint32_t scene = 0;
  uint32_t n = 0;
  sph_params prm{};
  explicit sph_sim(uint32_t count) : eng(count, 1), n(count) {}
};

struct sph_batch {
  sph::Engine eng;
  sph_batch(uint64_t cap, uint32_t ms) : eng(cap, ms) {}
};

namespace {

thread_local std::string g_error;

cudaStream_t S(void* s) { return static_cast<cudaStream_t>(s); }

int GlobalFail(int code, const std::string& msg) {
  g_error = msg;
  return code;
}

}  // namespace

extern "C" {

void sph_default_params(sph_params* o) {
  if (!o) return;
  o->radius = 0.35f;
  o->cutoff_sq = 0.35f * 0.35f;
  o->target_density = 99.7f;
  o->pressure_mult = 300.0f;
  o->near_pressure_mult = 20.0f;
  o->viscosity = 0.5f;
  o->gravity_scale = 10.0f;
  o->gravity_on = 0;
  o->bound[0] = o->bound[1] = o->bound[2] = 20.0f;
  o->damping = 0.95f;
  o->predict_dt = 1.0f / 120.0f;
}

const char* sph_global_error(void) { return g_error.c_str(); }

int sph_create(const sph_params* params, uint32_t n, sph_sim** out) {
  if (!params || !out) return GlobalFail(SPH_ERR_INVALID, "null argument");
  *out = nullptr;
  if (n == 0 || n >= (1u << 24))
    return GlobalFail(SPH_ERR_INVALID, "n must be in [1, 2^24)");
  sph_sim* h = new (std::nothrow) sph_sim(n);
  if (!h) return GlobalFail(SPH_ERR_NOMEM, "host allocation failed");
  int rc = h->eng.Init();
  if (rc != SPH_OK) {
    g_error = h->eng.LastError();
    delete h;
    return rc;
  }
  // The scene starts at rest at the origin until sph_upload (the reference
  // zeroes every buffer in InitializeData, physicsWorld.cc:129-137).
  h->prm = *params;
  rc = h->eng.AddScene(*params, n, nullptr, nullptr, true, 1.0f / 60.0f,
                       &h->scene, nullptr);
  if (rc != SPH_OK) {
    g_error = h->eng.LastError();
    delete h;
    return rc;
  }
  *out = h;
  return SPH_OK;
}

int sph_destroy(sph_sim* sim) {
  delete sim;
  return SPH_OK;
}

int sph_set_params(sph_sim* sim, const sph_params* p) {
  if (!sim || !p) return SPH_ERR_INVALID;
  int rc = sim->eng.SetParams(sim->scene, *p);
  if (rc == SPH_OK) sim->prm = *p;
  return rc;
}

int sph_get_params(const sph_sim* sim, sph_params* out) {
  if (!sim || !out) return SPH_ERR_INVALID;
  *out = sim->prm;
  return SPH_OK;
}

uint32_t sph_num_particles(const sph_sim* sim) { return sim ? sim->n : 0; }

int sph_upload(sph_sim* sim, const float* pos3, const float* vel3, void* stream) {
  if (!sim || !pos3) return SPH_ERR_INVALID;
  return sim->eng.Load(sim->scene, pos3, vel3, false, S(stream));
}

int sph_upload_device(sph_sim* sim, const float* dpos3, const float* dvel3,
                      void* stream) {
  if (!sim || !dpos3) return SPH_ERR_INVALID;
  return sim->eng.Load(sim->scene, dpos3, dvel3, true, S(stream));
}

int sph_step(sph_sim* sim, float dt, int substeps, void* stream) {
  if (!sim) return SPH_ERR_INVALID;
  if (substeps < 1) return sim->eng.Fail(SPH_ERR_INVALID, "substeps must be >= 1");
  int rc = sim->eng.SetDt(sim->scene, dt);
  if (rc != SPH_OK) return rc;
  return sim->eng.Step(substeps, S(stream));
}

int sph_download(sph_sim* sim, float* pos3, float* vel3, float* dens2,
                 void* stream) {
  if (!sim) return SPH_ERR_INVALID;
  return sim->eng.Download(sim->scene, pos3, vel3, dens2, false, S(stream));
}

int sph_download_device(sph_sim* sim, float* dpos3, float* dvel3, float* ddens2,
                        void* stream) {
  if (!sim) return SPH_ERR_INVALID;
  return sim->eng.Download(sim->scene, dpos3, dvel3, ddens2, true, S(stream));
}

int sph_save(sph_sim* sim, const char* path, void* stream) {
  if (!sim || !path) return SPH_ERR_INVALID;
  return sim->eng.SaveSnapshot(sim->scene, path, S(stream));
}

int sph_load(sph_sim* sim, const char* path, void* stream) {
  if (!sim || !path) return SPH_ERR_INVALID;
  sph::SceneSnapshot snap;
  int rc = sim->eng.ReadSnapshot(path, &snap);
  if (rc == SPH_OK) rc = sim->eng.RestoreSnapshot(sim->scene, snap, S(stream));
  if (rc == SPH_OK) sim->prm = snap.prm;
  return rc;
}

int sph_render(sph_sim* sim, const sph_view* view, uint8_t* rgba, float* depth,
               void* stream) {
  if (!sim || !view) return SPH_ERR_INVALID;
  return sim->eng.Render(sim->scene, *view, rgba, depth, S(stream));
}

int sph_out_positions(sph_sim* sim, void** dev_float4) {
  if (!sim) return SPH_ERR_INVALID;
  return sim->eng.OutPositions(sim->scene, dev_float4);
}

int sph_debug_enable(sph_sim* sim, int enable) {
  if (!sim) return SPH_ERR_INVALID;
  return sim->eng.DebugEnable(enable != 0);
}

int sph_debug_export(sph_sim* sim, uint32_t* hash, uint32_t* key,
                     uint32_t* sorted_ids, uint32_t* start, float* dens2,
                     float* acc_p3, float* vel_p3, float* vel_v3, void* stream) {
  if (!sim) return SPH_ERR_INVALID;
  return sim->eng.DebugExport(sim->scene, hash, key, sorted_ids, start, dens2,
                              acc_p3, vel_p3, vel_v3, S(stream));
}

int sph_debug_export_layout(sph_sim* sim, uint32_t* cell, uint32_t* key,
                            uint32_t* slot_ids, uint32_t* start, uint64_t start_cap,
                            uint32_t* table_len, int* direct, void* stream) {
  if (!sim) return SPH_ERR_INVALID;
  return sim->eng.DebugExportLayout(sim->scene, cell, key, slot_ids, start, start_cap,
                                    table_len, direct, S(stream));
}

int sph_status(sph_sim* sim, uint32_t* flags, void* stream) {
  if (!sim) return SPH_ERR_INVALID;
  return sim->eng.Status(flags, S(stream));
}

int sph_profile_enable(sph_sim* sim, int enable) {
  if (!sim) return SPH_ERR_INVALID;
  return sim->eng.ProfileEnable(enable != 0);
}

int sph_phase_times(sph_sim* sim, double out_ms[6]) {
  if (!sim || !out_ms) return SPH_ERR_INVALID;
  return sim->eng.PhaseTimes(out_ms);
}

int sph_set_tuning(sph_sim* sim, const sph_tuning* t) {
  if (!sim || !t) return SPH_ERR_INVALID;
  return sim->eng.SetTuning(*t);
}

int sph_get_tuning(const sph_sim* sim, sph_tuning* t) {
  if (!sim || !t) return SPH_ERR_INVALID;
  *t = sim->eng.Tuning();
  return SPH_OK;
}

int sph_autotune(sph_sim* sim, float dt, int substeps, int steps_per_trial,
                 sph_tuning* best, float* best_ms, void* stream) {
  if (!sim) return SPH_ERR_INVALID;
  const int rc = sim->eng.SetDt(sim->scene, dt);
  if (rc != SPH_OK) return rc;
  return sim->eng.Autotune(substeps, steps_per_trial, best, best_ms, S(stream));
}

uint64_t sph_kernel_launches(const sph_sim* sim) {
  return sim ? sim->eng.KernelLaunches() : 0;
}

const char* sph_last_error(const sph_sim* sim) {
  return sim ? sim->eng.LastError() : "null handle";
}

// ------------------------------------------------------------------ batch
int sph_batch_create(uint64_t capacity, uint32_t max_scenes, sph_batch** out) {
  if (!out) return GlobalFail(SPH_ERR_INVALID, "null argument");
  *out = nullptr;
  sph_batch* b = new (std::nothrow) sph_batch(capacity, max_scenes);
  if (!b) return GlobalFail(SPH_ERR_NOMEM, "host allocation failed");
  const int rc = b->eng.Init();
  if (rc != SPH_OK) {
    g_error = b->eng.LastError();
    delete b;
    return rc;
  }
  *out = b;
  return SPH_OK;
}

int sph_batch_destroy(sph_batch* b) {
  delete b;
  return SPH_OK;
}

int sph_batch_add(sph_batch* b, const sph_params* params, uint32_t n,
                  const float* pos3, const float* vel3, float dt,
                  uint32_t* scene_id, void* stream) {
  if (!b || !params || !pos3) return SPH_ERR_INVALID;
  return b->eng.AddScene(*params, n, pos3, vel3, false, dt, scene_id, S(stream));
}

int sph_batch_remove(sph_batch* b, uint32_t scene_id) {
  if (!b) return SPH_ERR_INVALID;
  return b->eng.RemoveScene(scene_id);
}

int sph_batch_sync(sph_batch* b, void* stream) {
  if (!b) return SPH_ERR_INVALID;
  const cudaError_t e = cudaStreamSynchronize(S(stream));
  return e == cudaSuccess ? SPH_OK : b->eng.CudaFail(e, "cudaStreamSynchronize");
}

int sph_batch_status(sph_batch* b, uint32_t* flags, void* stream) {
  if (!b || !flags) return SPH_ERR_INVALID;
  return b->eng.Status(flags, S(stream));
}

int sph_batch_step(sph_batch* b, int substeps, void* stream) {
  if (!b) return SPH_ERR_INVALID;
  return b->eng.Step(substeps, S(stream));
}

int sph_batch_download(sph_batch* b, uint32_t scene_id, float* pos3,
                       float* vel3, float* dens2, void* stream) {
  if (!b) return SPH_ERR_INVALID;
  return b->eng.Download(scene_id, pos3, vel3, dens2, false, S(stream));
}

int sph_batch_save(sph_batch* b, uint32_t scene_id, const char* path, void* stream) {
  if (!b || !path) return SPH_ERR_INVALID;
  return b->eng.SaveSnapshot(scene_id, path, S(stream));
}

int sph_batch_add_snapshot(sph_batch* b, const char* path, uint32_t* scene_id,
                           void* stream) {
  if (!b || !path) return SPH_ERR_INVALID;
  sph::SceneSnapshot snap;
  const int rc = b->eng.ReadSnapshot(path, &snap);
  return rc == SPH_OK ? b->eng.AddSnapshot(snap, scene_id, S(stream)) : rc;
}

int sph_batch_render(sph_batch* b, uint32_t scene_id, const sph_view* view,
                     uint8_t* rgba, float* depth, void* stream) {
  if (!b || !view) return SPH_ERR_INVALID;
  return b->eng.Render(scene_id, *view, rgba, depth, S(stream));
}

int sph_batch_set_tuning(sph_batch* b, const sph_tuning* t) {
  if (!b || !t) return SPH_ERR_INVALID;
  return b->eng.SetTuning(*t);
}

int sph_batch_get_tuning(const sph_batch* b, sph_tuning* t) {
  if (!b || !t) return SPH_ERR_INVALID;
  *t = b->eng.Tuning();
  return SPH_OK;
}

int sph_batch_autotune(sph_batch* b, int substeps, int steps_per_trial,
                       sph_tuning* best, float* best_ms, void* stream) {
  if (!b) return SPH_ERR_INVALID;
  return b->eng.Autotune(substeps, steps_per_trial, best, best_ms, S(stream));
}

uint64_t sph_bytes_per_particle(void) { return sph::Engine::BytesPerParticle(); }

uint32_t sph_batch_num_scenes(const sph_batch* b) {
  return b ? b->eng.NumScenes() : 0;
}

uint64_t sph_batch_num_particles(const sph_batch* b) {
  return b ? b->eng.NumParticles() : 0;
}

uint64_t sph_batch_kernel_launches(const sph_batch* b) {
  return b ? b->eng.KernelLaunches() : 0;
}

int sph_batch_profile_enable(sph_batch* b, int enable) {
  if (!b) return SPH_ERR_INVALID;
  return b->eng.ProfileEnable(enable != 0);
}

int sph_batch_phase_times(sph_batch* b, double out_ms[6]) {
  if (!b || !out_ms) return SPH_ERR_INVALID;
  return b->eng.PhaseTimes(out_ms);
}

const char* sph_batch_last_error(const sph_batch* b) {
  return b ? b->eng.LastError() : "null handle";
}

}  // extern "C"
