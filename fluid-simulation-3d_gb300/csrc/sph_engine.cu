// Host engine of the SPH substep pipeline (see sph_engine.h).
#include "sph_engine.h"
#include "sph_render.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>

namespace sph {

namespace {

// The device address of a host array the device can reach directly (pinned
// memory mapped into its address space) when 16-byte aligned; nullptr for
// pageable memory, other alignments and nullptr.
template <class T> T* DeviceAlias(T* p) {
  if (!p) return nullptr;
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();  // not an error for the caller: use the staged copy
    return nullptr;
  }
  if (a.type != cudaMemoryTypeHost || !a.devicePointer) return nullptr;
  if (reinterpret_cast<std::uintptr_t>(a.devicePointer) & 15u) return nullptr;
  return static_cast<T*>(a.devicePointer);
}

constexpr float kPiF = 3.14159265358979323846f;  // glm::pi<float>()

template <class Pred> float LargestWith(float r, Pred ok) {
  // Largest float x >= 0 with ok(sqrtf(x)), for a monotone predicate on
  // the correctly rounded square root.
  float x = r * r;
  if (!std::isfinite(x)) return std::numeric_limits<float>::max();
  while (x > 0.0f && !ok(std::sqrt(x))) x = std::nextafter(x, 0.0f);
  for (;;) {
    const float y = std::nextafter(x, std::numeric_limits<float>::infinity());
    if (!ok(std::sqrt(y))) break;
    x = y;
  }
  return x;
}

// Internal cell grid along one axis: the cells of [-h, h] (the box) plus a
// margin of 2 cells each side; returns the cell count, origin = first cell.
// Any origin and size give the same physics (they shape the layout only),
// but the count is kept in [5, 2^15] so that the y and z strides stay below
// 2^30 and the 27 offsets dx + dy*wy + dz*wz of a cell are distinct modulo
// 2^32; a larger box wraps onto the grid: cells that are not neighbours may
// then share an index and a run, and the cutoff test drops their pairs, as
// the reference's does for the cells its HashCell collides.
uint32_t GridAxis(float h, float r, uint32_t* origin) {
  const double a = std::floor(static_cast<double>(-h) / r);
  const double b = std::floor(static_cast<double>(h) / r);
  double lo = std::min(a, b) - 2.0, hi = std::max(a, b) + 2.0;
  if (!std::isfinite(lo) || !std::isfinite(hi) || lo < -1e9 || hi > 1e9) {
    lo = 0.0;
    hi = 1023.0;
  }
  *origin = static_cast<uint32_t>(static_cast<int32_t>(lo));
  return static_cast<uint32_t>(std::min(hi - lo + 1.0, 32768.0));
}

// The key table of a scene: one entry per grid cell (a direct table, where a
// cell's run needs no bucket search) when the grid has at most four cells per
// particle, else n entries holding cell index mod n. The choice depends on
// the scene alone, so a scene steps bit for bit alike in any batch. The
// table buffers hold kTablePerParticle entries per particle of capacity plus
// an allowance that tuning.table = 2 spends on direct tables for scenes with
// larger grids.
constexpr uint64_t kDirectCellsPerParticle = 4;
constexpr uint64_t kTablePerParticle = kDirectCellsPerParticle;
constexpr uint64_t kTableAllowance = 65536;

// The scene's constants with a bucket table at `tbase`; the caller switches
// to a direct table (direct = 1) where it has room for one.
SceneDev MakeSceneDev(const sph_params& p, uint32_t n, uint32_t base, uint32_t tbase,
                      float sub_dt) {
  SceneDev d{};
  d.n = n;
  d.base = base;
  d.tbase = tbase;
  d.fm = (~static_cast<uint64_t>(0)) / n + 1;
  const float r = p.radius;
  d.r = r;
  d.gnx = GridAxis(p.bound[0] * 0.5f, r, &d.gx0);
  d.gny = GridAxis(p.bound[1] * 0.5f, r, &d.gy0);
  d.gnz = GridAxis(p.bound[2] * 0.5f, r, &d.gz0);
  d.gwy = d.gnx;
  d.gwz = d.gnx * d.gny;  // modulo 2^32
  const float t_lt = LargestWith(r, [r](float s) { return s < r; });
  const float t_le = LargestWith(r, [r](float s) { return s <= r; });
  d.cut_lt = std::min(p.cutoff_sq, t_lt);
  d.cut_le = std::min(p.cutoff_sq, t_le);
  d.cut_hi = d.cut_le * 1.000002f;
  d.cut_lo = d.cut_lt * 0.999998f;  d.r2 = r * r;
  // kernels.h:28,40,52,64,76 -- same float expressions.
  d.vol2 = 15.0f / (2.0f * kPiF * powf(r, 5.0f));
  d.vol3 = 15.0f / (kPiF * powf(r, 6.0f));
  d.ds2h = 0.5f * (15.0f / (powf(r, 5.0f) * kPiF));
  d.ds3h = 0.5f * (45.0f / (powf(r, 6.0f) * kPiF));
  d.vscale = 315.0f / (64.0f * kPiF * powf(std::fabs(r), 9.0f));
  d.rho0 = p.target_density;
  d.k = p.pressure_mult;
  d.kn = p.near_pressure_mult;
  d.mu = p.viscosity;
  d.gy = p.gravity_on ? -p.gravity_scale : 0.0f;
  d.hx = p.bound[0] * 0.5f;
  d.hy = p.bound[1] * 0.5f;
  d.hz = p.bound[2] * 0.5f;
  d.ndamp = -1.0f * p.damping;
  d.pdt = p.predict_dt;
  d.dt = sub_dt;
  return d;
}

uint64_t GridCells(const SceneDev& d) {
  return static_cast<uint64_t>(d.gnx) * d.gny * d.gnz;
}

template <class T> cudaError_t Alloc(T** p, uint64_t count) {
  return cudaMalloc(reinterpret_cast<void**>(p),
                    std::max<uint64_t>(count, 1) * sizeof(T));
}

}  // namespace

Engine::Engine(uint64_t capacity, uint32_t max_scenes)
    : capacity_(capacity), max_scenes_(max_scenes) {
  scenes_.resize(max_scenes);
  old_base_.assign(max_scenes, 0);
}

Engine::~Engine() {
  ReleaseGraphs();
  for (auto& e : prof_ev_)
    if (e) cudaEventDestroy(e);
  if (join_in_) cudaEventDestroy(join_in_);
  if (join_out_) cudaEventDestroy(join_out_);
  if (work_) cudaStreamDestroy(work_);
  void* ptrs[] = {d_scenes_, d_tiles_old_, d_tiles_new_, d_pos_[0], d_pos_[1],
                  d_vel_[0], d_vel_[1], ctx_.pred, ctx_.rec_v, ctx_.dens_a,
                  ctx_.dens_b, ctx_.keyrank, ctx_.tmp_hi, ctx_.tmp_src, ctx_.hash_s,
                  ctx_.nbr, ctx_.ncount, ctx_.cell_first, ctx_.cell_tab,
                  ctx_.count, ctx_.start,
                  ctx_.partial, d_out4_, d_status_, d_dbg_hash_, d_dbg_key_,
                  d_dbg_accp_, d_dbg_velv_, d_dbg_velp_, d_dbg_start_,
                  d_dbg_count_, d_dbg_partial_, d_dbg_keyrank_, d_dbg_tmp_,
                  d_dbg_sorted_, d_dbg_scratch_, d_rkeys_, d_rrgba_, d_rdepth_,
                  d_rcolour_};
  for (void* p : ptrs)
    if (p) cudaFree(p);
}

int Engine::Fail(int code, const std::string& msg) {
  err_ = msg;
  return code;
}

int Engine::CudaFail(cudaError_t e, const char* what) {
  err_ = std::string(what) + ": " + cudaGetErrorString(e);
  return SPH_ERR_CUDA;
}

#define SPH_CUDA(call, what)                       \
  do {                                             \
    cudaError_t e_ = (call);                       \
    if (e_ != cudaSuccess) return CudaFail(e_, what); \
  } while (0)

int Engine::Init() {
  // (the key table, kTablePerParticle entries a particle plus the allowance,
  // is indexed by 32-bit keys)
  if (capacity_ == 0 || capacity_ > (0xffffffffull - kTableAllowance) / kTablePerParticle ||
      max_scenes_ == 0 || max_scenes_ >= (1u << kTileSceneBits))
    return Fail(SPH_ERR_INVALID,
                "capacity must be in [1, 2^30 - 2^14) and scenes in [1, 2^27)");
  int dev = 0;
  SPH_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
  SPH_CUDA(cudaDeviceGetAttribute(&sm_count_, cudaDevAttrMultiProcessorCount, dev),
           "cudaDeviceGetAttribute");
  SPH_CUDA(cudaStreamCreateWithFlags(&work_, cudaStreamNonBlocking),
           "cudaStreamCreateWithFlags");
  SPH_CUDA(cudaEventCreateWithFlags(&join_in_, cudaEventDisableTiming),
           "cudaEventCreate");
  SPH_CUDA(cudaEventCreateWithFlags(&join_out_, cudaEventDisableTiming),
           "cudaEventCreate");
  const uint64_t C = capacity_;
  const uint64_t max_tiles = C / kTile + max_scenes_ + 1;
  cudaError_t e = cudaSuccess;
  auto chk = [&](cudaError_t x) { if (e == cudaSuccess) e = x; };
  chk(Alloc(&d_scenes_, max_scenes_));
  chk(Alloc(&d_tiles_old_, max_tiles));
  chk(Alloc(&d_tiles_new_, max_tiles));
  for (int b = 0; b < 2; ++b) {
    chk(Alloc(&d_pos_[b], C));
    chk(Alloc(&d_vel_[b], C));
  }
  chk(Alloc(&ctx_.pred, C));
  chk(Alloc(&ctx_.rec_v, 2 * C));
  chk(Alloc(&ctx_.dens_a, C));
  chk(Alloc(&ctx_.dens_b, C));
  chk(Alloc(&ctx_.keyrank, C));
  chk(Alloc(&ctx_.tmp_hi, C));
  chk(Alloc(&ctx_.tmp_src, C));
  chk(Alloc(&ctx_.hash_s, C));
  chk(Alloc(&ctx_.ncount, C));
  chk(Alloc(&ctx_.cell_first, C));
  chk(Alloc(&ctx_.cell_tab, C * 27ull));
  chk(Alloc(&ctx_.nbr, C * static_cast<uint64_t>(kNbrCap)));
  const uint64_t T = kTablePerParticle * C + kTableAllowance;  // key-table entries
  chk(Alloc(&ctx_.count, T));
  chk(Alloc(&ctx_.start, T + 1));
  chk(Alloc(&ctx_.partial, scan_partials_needed(T)));
  chk(Alloc(&d_out4_, C));
  chk(Alloc(&d_status_, 1));
  if (e != cudaSuccess) {
    cudaGetLastError();
    return e == cudaErrorMemoryAllocation
               ? Fail(SPH_ERR_NOMEM, "device allocation failed")
               : CudaFail(e, "cudaMalloc");
  }
  SPH_CUDA(cudaMemset(ctx_.count, 0, T * sizeof(uint32_t)), "cudaMemset");
  SPH_CUDA(cudaMemset(ctx_.dens_a, 0, C * sizeof(float2)), "cudaMemset");
  SPH_CUDA(cudaMemset(d_status_, 0, sizeof(uint32_t)), "cudaMemset");
  SPH_CUDA(cudaMemset(d_out4_, 0, C * sizeof(float4)), "cudaMemset");
  ctx_.scenes = d_scenes_;
  ctx_.out4 = d_out4_;
  ctx_.status = d_status_;
  ctx_.nbr_stride = static_cast<uint32_t>(C);
  ctx_.nbr_cap = kNbrCap;
  return SPH_OK;
}

uint64_t Engine::BytesPerParticle() {
  return 2 * 2 * sizeof(float4)                // pos, vel (double-buffered)
         + sizeof(float4) + 2 * sizeof(float4)  // pred, rec_v
         + sizeof(float2) + sizeof(float4)     // dens_a, dens_b
         + sizeof(uint4)                       // keyrank
         + sizeof(uint2) + 4 * sizeof(uint32_t)  // tmp_hi, tmp_src, hash_s,
                                                 // cell_first, ncount
         + 27 * sizeof(uint2)                  // cell_tab
         + kNbrCap * sizeof(uint32_t)          // nbr
         + kTablePerParticle * 2 * sizeof(uint32_t)  // count, start
         + sizeof(float4)                      // out4
         + sizeof(uint2);                      // tiles (old + new, per 32)
}

uint32_t Engine::NumScenes() const {
  uint32_t c = 0;
  for (const auto& s : scenes_) c += s.live ? 1 : 0;
  return c;
}

uint64_t Engine::NumParticles() const {
  uint64_t c = 0;
  for (const auto& s : scenes_) c += s.live ? s.n : 0;
  return c;
}

uint32_t Engine::SceneSize(uint32_t id) const {
  return (id < max_scenes_ && scenes_[id].live) ? scenes_[id].n : 0;
}

int Engine::AddScene(const sph_params& p, uint32_t n, const float* pos3,
                     const float* vel3, bool device_ptrs, float dt,
                     uint32_t* id, cudaStream_t st) {
  if (n == 0 || n >= (1u << 24))
    return Fail(SPH_ERR_INVALID, "scene size must be in [1, 2^24)");
  if (!(p.radius > 0.0f) || !std::isfinite(p.radius))
    return Fail(SPH_ERR_INVALID, "radius must be positive and finite");
  // where the scene goes in the current layout: the first free extent that
  // holds it, else past the end
  size_t fi = 0;
  while (fi < free_.size() && free_[fi].second < n) ++fi;
  const bool in_gap = fi < free_.size();
  if (!in_gap && layout_total_ + n > capacity_)
    return Fail(SPH_ERR_NOMEM, "scene does not fit the engine capacity");
  uint32_t s = 0;
  while (s < max_scenes_ && scenes_[s].used) ++s;
  if (s == max_scenes_) return Fail(SPH_ERR_NOMEM, "no free scene slot");
  const uint64_t base = in_gap ? free_[fi].first : layout_total_;
  if (in_gap) {
    free_[fi].first += n;
    free_[fi].second -= n;
    if (free_[fi].second == 0) free_.erase(free_.begin() + static_cast<std::ptrdiff_t>(fi));
  } else {
    layout_total_ += n;
  }
  Scene& sc = scenes_[s];
  sc = Scene{};
  sc.used = sc.live = true;
  sc.prm = p;
  sc.n = n;
  sc.dt = dt;
  old_base_[s] = static_cast<uint32_t>(base);
  layout_dirty_ = scenes_dirty_ = true;
  carry_valid_ = false;
  const int rc = Load(s, pos3, vel3, device_ptrs, st);
  if (rc != SPH_OK) {
    sc = Scene{};
    if (base + n == layout_total_)
      layout_total_ -= n;
    else
      free_.emplace_back(base, n);
    return rc;
  }
  if (id) *id = s;
  return SPH_OK;
}

int Engine::RemoveScene(uint32_t id) {
  if (id >= max_scenes_ || !scenes_[id].live)
    return Fail(SPH_ERR_INVALID, "no such scene");
  scenes_[id].live = false;  // its slots vanish at the next step's sort
  layout_dirty_ = scenes_dirty_ = true;
  carry_valid_ = false;
  bool any_live = false;
  for (uint32_t s = 0; s < max_scenes_ && !any_live; ++s) any_live = scenes_[s].live;
  if (any_live) {
    free_.emplace_back(old_base_[id], scenes_[id].n);  // reusable before then
  } else {
    free_.clear();  // nothing left to keep: the layout starts over
    layout_total_ = 0;
  }
  return SPH_OK;
}

int Engine::SetParams(uint32_t id, const sph_params& p) {
  if (id >= max_scenes_ || !scenes_[id].live)
    return Fail(SPH_ERR_INVALID, "no such scene");
  if (!(p.radius > 0.0f) || !std::isfinite(p.radius))
    return Fail(SPH_ERR_INVALID, "radius must be positive and finite");
  scenes_[id].prm = p;
  scenes_dirty_ = true;
  carry_valid_ = false;
  return SPH_OK;
}

int Engine::GetParams(uint32_t id, sph_params* p) const {
  if (id >= max_scenes_ || !scenes_[id].live || !p) return SPH_ERR_INVALID;
  *p = scenes_[id].prm;
  return SPH_OK;
}

int Engine::SetDt(uint32_t id, float dt) {
  if (id >= max_scenes_ || !scenes_[id].live)
    return Fail(SPH_ERR_INVALID, "no such scene");
  if (scenes_[id].dt != dt) {
    scenes_[id].dt = dt;
    scenes_dirty_ = true;
    carry_valid_ = false;
  }
  return SPH_OK;
}

int Engine::Load(uint32_t id, const float* pos3, const float* vel3,
                 bool device_ptrs, cudaStream_t st) {
  if (id >= max_scenes_ || !scenes_[id].live)
    return Fail(SPH_ERR_INVALID, "no such scene");
  // pos3 == nullptr loads the zero state (InitializeData, physicsWorld.cc:129-137).
  const uint32_t n = scenes_[id].n;
  carry_valid_ = false;  // a new state needs its own prediction
  const float* dp = pos3;
  const float* dv = vel3;
  const float* hp = device_ptrs ? nullptr : DeviceAlias(pos3);
  const float* hv = device_ptrs ? nullptr : DeviceAlias(vel3);
  // A single scene whose device constants and layout are current (a step
  // has run since the last change): the import also predicts the next
  // step's first substep with those constants, and that step uses it if its
  // dt and substeps are unchanged (the carry test in Step).
  const bool predict = hp && (!vel3 || hv) && max_scenes_ == 1 && !scenes_dirty_ &&
                       uploaded_substeps_ > 0 && !layout_dirty_ &&
                       n_tiles_old_ == n_tiles_new_ && total_ == n;
  if (hp && (!vel3 || hv)) {
    // pinned host rows: the import kernel reads them over the link itself
    if (predict && count_extent_)
      SPH_CUDA(cudaMemsetAsync(ctx_.count, 0, sizeof(uint32_t) * count_extent_, st),
               "histogram reset");
    SPH_CUDA(launch_import_rows(old_base_[id], n, hp, hv, d_pos_[cur_], d_vel_[cur_],
                                predict ? ctx_.scenes + id : nullptr, ctx_.count,
                                ctx_.keyrank, st),
             "import kernel");
    if (predict) {
      carry_valid_ = true;
      count_extent_ = table_total_;
    }
  } else if (!device_ptrs && pos3) {
    // Stage through the prediction / post-pressure buffers (rewritten by
    // every substep before use).
    float* sp = reinterpret_cast<float*>(ctx_.pred);
    float* sv = reinterpret_cast<float*>(ctx_.rec_v);
    SPH_CUDA(cudaMemcpyAsync(sp, pos3, sizeof(float) * 3 * n,
                             cudaMemcpyHostToDevice, st), "upload positions");
    if (vel3)
      SPH_CUDA(cudaMemcpyAsync(sv, vel3, sizeof(float) * 3 * n,
                               cudaMemcpyHostToDevice, st), "upload velocities");
    dp = sp;
    dv = vel3 ? sv : nullptr;
  } else if (!pos3) {
    dv = nullptr;
  }
  if (!(hp && (!vel3 || hv)))
    SPH_CUDA(launch_import(old_base_[id], n, dp, dv, d_pos_[cur_], d_vel_[cur_], st),
             "import kernel");
  // Densities are unknown until the next step.
  SPH_CUDA(cudaMemsetAsync(ctx_.dens_a + old_base_[id], 0, sizeof(float2) * n, st),
           "cudaMemsetAsync");
  debug_valid_ = false;
  return SPH_OK;
}

void Engine::BuildTiles(std::vector<uint2>& out, bool old_layout) const {
  out.clear();
  for (uint32_t s = 0; s < max_scenes_; ++s) {
    const Scene& sc = scenes_[s];
    if (!sc.live) continue;
    const uint32_t b = old_layout ? old_base_[s] : sc.base;
    for (uint32_t f = 0; f < sc.n; f += kTile)
      out.push_back(make_tile(s, b + f, std::min<uint32_t>(kTile, sc.n - f)));
  }
}

int Engine::BuildLayout(cudaStream_t st) {
  if (!layout_dirty_) return SPH_OK;
  uint32_t b = 0;
  for (uint32_t s = 0; s < max_scenes_; ++s) {
    Scene& sc = scenes_[s];
    if (!sc.live) continue;
    sc.base = b;
    b += sc.n;
  }
  total_ = b;
  std::vector<uint2> t_old, t_new;
  BuildTiles(t_old, true);
  BuildTiles(t_new, false);
  n_tiles_old_ = static_cast<uint32_t>(t_old.size());
  n_tiles_new_ = static_cast<uint32_t>(t_new.size());
  if (n_tiles_old_)
    SPH_CUDA(cudaMemcpyAsync(d_tiles_old_, t_old.data(), sizeof(uint2) * n_tiles_old_,
                             cudaMemcpyHostToDevice, st), "upload tiles");
  if (n_tiles_new_)
    SPH_CUDA(cudaMemcpyAsync(d_tiles_new_, t_new.data(), sizeof(uint2) * n_tiles_new_,
                             cudaMemcpyHostToDevice, st), "upload tiles");
  // The host vectors die at return: make the copies complete first.
  SPH_CUDA(cudaStreamSynchronize(st), "cudaStreamSynchronize");
  ReleaseGraphs();
  scenes_dirty_ = true;
  return SPH_OK;
}

int Engine::UploadScenes(int substeps, cudaStream_t st) {
  if (!scenes_dirty_ && uploaded_substeps_ == substeps) return SPH_OK;
  std::vector<SceneDev> h(max_scenes_);
  uint32_t hi = 0;
  uint64_t tb = 0;  // key tables in layout order, like the slots
  uint64_t allowance = kTableAllowance;
  uint32_t n_direct = 0, n_live = 0;
  for (uint32_t s = 0; s < max_scenes_; ++s) {
    const Scene& sc = scenes_[s];
    if (!sc.live) continue;
    SceneDev& d = h[s];
    d = MakeSceneDev(sc.prm, sc.n, sc.base, static_cast<uint32_t>(tb),
                     sc.dt / static_cast<float>(substeps));
    const uint64_t cells = GridCells(d);
    if (tuning_.table != 1 && cells <= kDirectCellsPerParticle * sc.n) {
      d.direct = 1;
    } else if (tuning_.table == 2 && cells - sc.n <= allowance) {
      d.direct = 1;
      allowance -= cells - sc.n;
    }
    tb += d.direct ? cells : sc.n;
    n_direct += d.direct;
    ++n_live;
    hi = s + 1;
  }
  const int tables = n_direct == n_live ? kTablesDirect
                     : n_direct == 0    ? kTablesBuckets
                                        : kTablesMixed;
  if (tb != table_total_ || tables != tables_) {
    // the scan's length and the kernels' table forms are part of the
    // captured graphs
    table_total_ = static_cast<uint32_t>(tb);
    tables_ = tables;
    ReleaseGraphs();
  }
  if (hi)
    SPH_CUDA(cudaMemcpyAsync(d_scenes_, h.data(), sizeof(SceneDev) * hi,
                             cudaMemcpyHostToDevice, st), "upload scenes");
  SPH_CUDA(cudaStreamSynchronize(st), "cudaStreamSynchronize");
  scene_dev_ = std::move(h);
  scenes_dirty_ = false;
  uploaded_substeps_ = substeps;
  return SPH_OK;
}

// Launches `substeps` substeps starting from state buffers cur_. Does not
// change engine state, so it can run under stream capture.
int Engine::RunSubsteps(int substeps, cudaStream_t st, bool carry) {
  LaunchCtx c = ctx_;
  c.block_nbr = tuning_.block;
  c.block_force = tuning_.force_block ? tuning_.force_block : tuning_.block;
  c.cell_tile = tuning_.cell_tile;
  c.gather = tuning_.gather;
  c.lanes = 32 / tuning_.particles_per_warp;
  c.tables = tables_;
  c.pdl = !profile_;  // phase events between kernels need plain launches
  c.max_blocks = 0;
  c.src_limit = static_cast<uint32_t>(capacity_);
  int cur = cur_;
  const Tiles told{d_tiles_old_, n_tiles_old_};
  const Tiles tnew{d_tiles_new_, n_tiles_new_};
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  SPH_CUDA(cudaStreamIsCapturing(st, &cap), "cudaStreamIsCapturing");
  const bool capturing = cap == cudaStreamCaptureStatusActive;
  for (int ss = 0; ss < substeps; ++ss) {
    c.pos = d_pos_[cur];
    c.vel = d_vel_[cur];
    c.pos2 = d_pos_[1 - cur];
    c.vel2 = d_vel_[1 - cur];
    const bool dbg = debug_ && ss == 0;
    c.dbg_accp = dbg ? d_dbg_accp_ : nullptr;
    c.dbg_velv = dbg ? d_dbg_velv_ : nullptr;
    const Tiles& first = ss == 0 ? told : tnew;
    cudaEvent_t* ev = profile_ ? &prof_ev_[ss * kPhaseEvents] : nullptr;
    cudaError_t e = cudaSuccess;
    // External records become event nodes when the stream is being captured
    // (a plain record would only express a dependency).
    auto mark = [&](int k) {
      if (!ev || e != cudaSuccess) return;
      e = capturing ? cudaEventRecordWithFlags(ev[k], st, cudaEventRecordExternal)
                    : cudaEventRecord(ev[k], st);
    };
    mark(0);
    if (ss == 0 && !carry) e = launch_predict_hash(c, first, st);
    mark(1);
    if (e == cudaSuccess) e = launch_scan(c, table_total_, st);
    if (e == cudaSuccess) e = launch_sort_reorder(c, first, tnew, total_, st);
    mark(2);
    if (e == cudaSuccess && dbg) e = launch_ref_lookup(c, tnew, total_, st);
    if (e == cudaSuccess) e = launch_density(c, tnew, st);
    mark(3);
    if (e == cudaSuccess) e = launch_pressure(c, tnew, st);
    mark(4);
    // every viscosity pass predicts the following substep, the last one
    // the next step's first (used when nothing changes in between)
    if (e == cudaSuccess)
      e = launch_visc_integrate(c, tnew, 1, ss + 1 == substeps ? 1 : 0, st);
    mark(5);
    if (e == cudaSuccess && dbg)
      e = cudaMemcpy2DAsync(d_dbg_velp_, sizeof(float4), c.rec_v + 1,
                            2 * sizeof(float4), sizeof(float4), total_,
                            cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) return CudaFail(e, "substep launch");
    cur = 1 - cur;
  }
  return SPH_OK;
}

int Engine::ProfileEnable(bool on) {
  if (on && prof_ev_.empty()) {
    prof_ev_.resize(kPhaseEvents * kMaxSubsteps);
    for (auto& e : prof_ev_) SPH_CUDA(cudaEventCreate(&e), "cudaEventCreate");
  }
  if (on != profile_) ReleaseGraphs();
  profile_ = on;
  profiled_substeps_ = 0;
  return SPH_OK;
}

// ms per phase of the last step, summed over its substeps, in the order of
// the reference's timers (Gravity, Spatial, Density, Pressure, Viscosity,
// PosNColl; physicsWorld.h:45-50). Integration and collision run inside the
// viscosity kernel, so PosNColl is reported as 0.
int Engine::PhaseTimes(double out[6]) {
  for (int k = 0; k < 6; ++k) out[k] = 0.0;
  if (!profile_ || profiled_substeps_ == 0)
    return Fail(SPH_ERR_STATE, "profiling not enabled or no step run");
  for (int ss = 0; ss < profiled_substeps_; ++ss) {
    cudaEvent_t* ev = &prof_ev_[ss * kPhaseEvents];
    SPH_CUDA(cudaEventSynchronize(ev[kPhaseEvents - 1]), "cudaEventSynchronize");
    for (int k = 0; k < 5; ++k) {
      float ms = 0.0f;
      SPH_CUDA(cudaEventElapsedTime(&ms, ev[k], ev[k + 1]), "cudaEventElapsedTime");
      out[k] += ms;
    }
  }
  return SPH_OK;
}

void Engine::ReleaseGraphs() {
  for (auto& kv : graphs_) cudaGraphExecDestroy(kv.second);
  graphs_.clear();
}

int Engine::Step(int substeps, cudaStream_t st) {
  if (substeps < 1 || substeps > kMaxSubsteps)
    return Fail(SPH_ERR_INVALID, "substeps must be in [1, 64]");
  if (debug_ && substeps != 1)
    return Fail(SPH_ERR_STATE, "debug capture needs substeps == 1");
  // the previous step already predicted this step's first substep unless
  // something changed since (checked before the layout and scene tables
  // are refreshed)
  const bool carry = carry_valid_ && !layout_dirty_ && !scenes_dirty_ &&
                     uploaded_substeps_ == substeps && n_tiles_old_ == n_tiles_new_;
  int rc = BuildLayout(st);
  if (rc != SPH_OK) return rc;
  rc = UploadScenes(substeps, st);
  if (rc != SPH_OK) return rc;
  if (!carry && count_extent_) {
    // an unused carried prediction left its histogram behind
    SPH_CUDA(cudaMemsetAsync(ctx_.count, 0, sizeof(uint32_t) * count_extent_, st),
             "histogram reset");
    count_extent_ = 0;
  }
  if (total_ > 0) {
    // join: the work stream starts after everything queued on `st`
    SPH_CUDA(cudaEventRecord(join_in_, st), "cudaEventRecord");
    SPH_CUDA(cudaStreamWaitEvent(work_, join_in_, 0), "cudaStreamWaitEvent");
    const bool steady = n_tiles_old_ == n_tiles_new_ && !layout_dirty_;
    if (use_graphs_ && steady && !debug_) {
      const auto key = std::make_pair(substeps, cur_ + (carry ? 2 : 0));
      auto it = graphs_.find(key);
      if (it == graphs_.end()) {
        cudaGraph_t g = nullptr;
        SPH_CUDA(cudaStreamBeginCapture(work_, cudaStreamCaptureModeThreadLocal),
                 "cudaStreamBeginCapture");
        rc = RunSubsteps(substeps, work_, carry);
        const cudaError_t e = cudaStreamEndCapture(work_, &g);
        if (rc != SPH_OK) {
          if (g) cudaGraphDestroy(g);
          return rc;
        }
        SPH_CUDA(e, "cudaStreamEndCapture");
        cudaGraphExec_t ex = nullptr;
        const cudaError_t ei = cudaGraphInstantiate(&ex, g, 0);
        cudaGraphDestroy(g);
        SPH_CUDA(ei, "cudaGraphInstantiate");
        it = graphs_.emplace(key, ex).first;
      }
      SPH_CUDA(cudaGraphLaunch(it->second, work_), "cudaGraphLaunch");
    } else {
      rc = RunSubsteps(substeps, work_, carry);
      if (rc != SPH_OK) return rc;
    }
    // join back: later work on `st` sees the step's results
    SPH_CUDA(cudaEventRecord(join_out_, work_), "cudaEventRecord");
    SPH_CUDA(cudaStreamWaitEvent(st, join_out_, 0), "cudaStreamWaitEvent");
    launches_ += static_cast<uint64_t>(carry ? 0 : kKernelsPredict) +
                 static_cast<uint64_t>(kernels_per_substep(table_total_, tables_)) * substeps;
    carry_valid_ = true;
    count_extent_ = table_total_;
    profiled_substeps_ = profile_ ? substeps : 0;
    if (substeps & 1) cur_ = 1 - cur_;
  }
  if (layout_dirty_ || n_tiles_old_ != n_tiles_new_) {
    // The data now sits in the compacted layout.
    if (n_tiles_new_)
      SPH_CUDA(cudaMemcpyAsync(d_tiles_old_, d_tiles_new_, sizeof(uint2) * n_tiles_new_,
                               cudaMemcpyDeviceToDevice, st), "tile copy");
    n_tiles_old_ = n_tiles_new_;
    for (uint32_t s = 0; s < max_scenes_; ++s)
      if (scenes_[s].live) old_base_[s] = scenes_[s].base;
    layout_total_ = total_;
    layout_dirty_ = false;
    free_.clear();
    for (auto& sc : scenes_)
      if (sc.used && !sc.live) sc.used = false;
  }
  debug_valid_ = debug_;
  return SPH_OK;
}

int Engine::Download(uint32_t id, float* pos3, float* vel3, float* dens2,
                     bool device_ptrs, cudaStream_t st) {
  if (id >= max_scenes_ || !scenes_[id].live)
    return Fail(SPH_ERR_INVALID, "no such scene");
  const uint32_t n = scenes_[id].n;
  const uint32_t b = old_base_[id];
  if (!device_ptrs && (pos3 || vel3 || dens2)) {
    // Pinned, 16-byte aligned outputs: one kernel gathers the rows in caller
    // order and stores them over the host link itself, 16-byte words per
    // 32 rows (the slot map goes to the sort's source-slot scratch, which
    // every substep rewrites before use).
    float* hp = DeviceAlias(pos3);
    float* hv = DeviceAlias(vel3);
    float* hd = DeviceAlias(dens2);
    if ((!pos3 || hp) && (!vel3 || hv) && (!dens2 || hd)) {
      SPH_CUDA(launch_export_rows(b, n, d_pos_[cur_], d_vel_[cur_], ctx_.dens_a,
                                  ctx_.tmp_src + b, hp, hv, hd, st),
               "export kernel");
      SPH_CUDA(cudaStreamSynchronize(st), "cudaStreamSynchronize");
      return SPH_OK;
    }
  }
  float *op = pos3, *ov = vel3, *od = dens2;
  // Other host memory stages through the prediction / post-pressure /
  // density buffers (16-32 B per slot, rewritten by every substep before
  // use) and the copy engine.
  float* scratch = reinterpret_cast<float*>(ctx_.pred);
  float* scratch_v = reinterpret_cast<float*>(ctx_.rec_v);
  float* scratch_d = reinterpret_cast<float*>(ctx_.dens_b);
  if (!device_ptrs) {
    op = pos3 ? scratch : nullptr;
    ov = vel3 ? scratch_v : nullptr;
    od = dens2 ? scratch_d : nullptr;
  }
  SPH_CUDA(launch_export(b, n, d_pos_[cur_], d_vel_[cur_], ctx_.dens_a, op, ov,
                         od, nullptr, st), "export kernel");
  if (!device_ptrs) {
    if (pos3)
      SPH_CUDA(cudaMemcpyAsync(pos3, scratch, sizeof(float) * 3 * n,
                               cudaMemcpyDeviceToHost, st), "download positions");
    if (vel3)
      SPH_CUDA(cudaMemcpyAsync(vel3, scratch_v, sizeof(float) * 3 * n,
                               cudaMemcpyDeviceToHost, st), "download velocities");
    if (dens2)
      SPH_CUDA(cudaMemcpyAsync(dens2, scratch_d, sizeof(float) * 2 * n,
                               cudaMemcpyDeviceToHost, st), "download densities");
  }
  SPH_CUDA(cudaStreamSynchronize(st), "cudaStreamSynchronize");
  return SPH_OK;
}

int Engine::Render(uint32_t id, const sph_view& v, uint8_t* rgba, float* depth,
                   cudaStream_t st) {
  if (id >= max_scenes_ || !scenes_[id].live)
    return Fail(SPH_ERR_INVALID, "no such scene");
  const uint64_t pixels = static_cast<uint64_t>(v.width) * v.height;
  if (v.width == 0 || v.height == 0 || pixels > (1ull << 28))
    return Fail(SPH_ERR_INVALID, "image size must be in [1, 2^28] pixels");
  const float* P = v.proj;
  if (!(P[0] > 0.0f) || !(P[5] > 0.0f) || P[1] != 0.0f || P[2] != 0.0f || P[3] != 0.0f ||
      P[4] != 0.0f || P[6] != 0.0f || P[7] != 0.0f)
    return Fail(SPH_ERR_INVALID,
                "projection columns 0 and 1 must be (a,0,0,0) and (0,b,0,0), a, b > 0");
  if (!(v.scale > 0.0f) || !std::isfinite(v.scale))
    return Fail(SPH_ERR_INVALID, "scale must be positive and finite");
  for (float x : v.view_proj)
    if (!std::isfinite(x)) return Fail(SPH_ERR_INVALID, "view_proj must be finite");
  if (pixels > render_pixels_) {
    cudaFree(d_rkeys_);
    cudaFree(d_rrgba_);
    cudaFree(d_rdepth_);
    d_rkeys_ = nullptr;
    d_rrgba_ = nullptr;
    d_rdepth_ = nullptr;
    render_pixels_ = 0;
    cudaError_t e = Alloc(&d_rkeys_, pixels);
    if (e == cudaSuccess) e = Alloc(&d_rrgba_, pixels);
    if (e == cudaSuccess) e = Alloc(&d_rdepth_, pixels);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return Fail(SPH_ERR_NOMEM, "render buffers do not fit the device");
    }
    render_pixels_ = pixels;
  }
  if (!d_rcolour_) SPH_CUDA(Alloc(&d_rcolour_, capacity_), "cudaMalloc");
  RenderView rv{};
  for (int k = 0; k < 16; ++k) rv.vp[k] = v.view_proj[k];
  const float hs = 0.5f * v.scale;
  rv.ox = P[0] * hs;
  rv.oy = P[5] * hs;
  rv.hw = 0.5f * static_cast<float>(v.width);
  rv.hh = 0.5f * static_cast<float>(v.height);
  rv.q = v.scale * 0.25f;
  rv.width = v.width;
  rv.height = v.height;
  rv.clear = 0;
  for (int k = 0; k < 4; ++k) {
    const float c = std::fmin(std::fmax(v.clear[k], 0.0f), 1.0f) * 255.0f;
    rv.clear |= static_cast<uint32_t>(std::lrint(c)) << (8 * k);
  }
  SPH_CUDA(launch_render(old_base_[id], scenes_[id].n, d_pos_[cur_], d_vel_[cur_], rv,
                         d_rkeys_, d_rcolour_, d_rrgba_, d_rdepth_, st),
           "render kernels");
  if (rgba)
    SPH_CUDA(cudaMemcpyAsync(rgba, d_rrgba_, 4 * pixels, cudaMemcpyDeviceToHost, st),
             "download image");
  if (depth)
    SPH_CUDA(cudaMemcpyAsync(depth, d_rdepth_, 4 * pixels, cudaMemcpyDeviceToHost, st),
             "download depth");
  SPH_CUDA(cudaStreamSynchronize(st), "cudaStreamSynchronize");
  return SPH_OK;
}

int Engine::OutPositions(uint32_t id, void** dev_float4) {
  if (id >= max_scenes_ || !scenes_[id].live || !dev_float4)
    return Fail(SPH_ERR_INVALID, "no such scene");
  *dev_float4 = d_out4_ + old_base_[id];
  return SPH_OK;
}

int Engine::DebugEnable(bool on) {
  if (on && !d_dbg_hash_) {
    const uint64_t C = capacity_;
    cudaError_t e = cudaSuccess;
    auto chk = [&](cudaError_t x) { if (e == cudaSuccess) e = x; };
    chk(Alloc(&d_dbg_hash_, C));
    chk(Alloc(&d_dbg_key_, C));
    chk(Alloc(&d_dbg_accp_, C));
    chk(Alloc(&d_dbg_velv_, C));
    chk(Alloc(&d_dbg_velp_, C));
    chk(Alloc(&d_dbg_start_, C + 1));
    chk(Alloc(&d_dbg_count_, C));
    chk(Alloc(&d_dbg_partial_, scan_partials_needed(C)));
    chk(Alloc(&d_dbg_keyrank_, C));
    chk(Alloc(&d_dbg_tmp_, C));
    chk(Alloc(&d_dbg_sorted_, C));
    // three float3 (36) per particle
    chk(cudaMalloc(&d_dbg_scratch_, C * 36 + 64));
    if (e == cudaSuccess) e = cudaMemset(d_dbg_count_, 0, C * sizeof(uint32_t));
    if (e != cudaSuccess) return CudaFail(e, "debug buffers");
    ctx_.dbg_hash = d_dbg_hash_;
    ctx_.dbg_key = d_dbg_key_;
    ctx_.dbg_count = d_dbg_count_;
    ctx_.dbg_start = d_dbg_start_;
    ctx_.dbg_partial = d_dbg_partial_;
    ctx_.dbg_keyrank = d_dbg_keyrank_;
    ctx_.dbg_tmp = d_dbg_tmp_;
    ctx_.dbg_sorted = d_dbg_sorted_;
  }
  if (debug_ != on) ReleaseGraphs();
  debug_ = on;
  debug_valid_ = false;
  return SPH_OK;
}

int Engine::DebugExport(uint32_t id, uint32_t* hash, uint32_t* key,
                        uint32_t* sorted_ids, uint32_t* start, float* dens2,
                        float* accp, float* velp, float* velv,
                        cudaStream_t st) {
  if (id >= max_scenes_ || !scenes_[id].live)
    return Fail(SPH_ERR_INVALID, "no such scene");
  if (!debug_valid_) return Fail(SPH_ERR_STATE, "no captured substep");
  const uint32_t n = scenes_[id].n;
  const uint32_t b = old_base_[id];
  float* sa = static_cast<float*>(d_dbg_scratch_);
  float* sp = sa + 3 * static_cast<uint64_t>(n);
  float* sv = sp + 3 * static_cast<uint64_t>(n);
  SPH_CUDA(launch_export_debug(b, n, d_pos_[cur_], d_dbg_accp_, d_dbg_velp_,
                               d_dbg_velv_, sa, sp, sv, st), "debug export kernel");
  auto d2h = [&](void* dst, const void* src, size_t bytes) -> cudaError_t {
    if (!dst) return cudaSuccess;
    return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, st);
  };
  // The reference lookup (launch_ref_lookup) is indexed by particle (hash,
  // key) and by lookup slot (sorted ids, start) within the scene's range.
  SPH_CUDA(d2h(hash, d_dbg_hash_ + b, 4ull * n), "download");
  SPH_CUDA(d2h(key, d_dbg_key_ + b, 4ull * n), "download");
  SPH_CUDA(d2h(sorted_ids, d_dbg_sorted_ + b, 4ull * n), "download");
  SPH_CUDA(d2h(accp, sa, 12ull * n), "download");
  SPH_CUDA(d2h(velp, sp, 12ull * n), "download");
  SPH_CUDA(d2h(velv, sv, 12ull * n), "download");
  std::vector<uint32_t> st_raw(n + 1);
  SPH_CUDA(cudaMemcpyAsync(st_raw.data(), d_dbg_start_ + b, 4ull * (n + 1),
                           cudaMemcpyDeviceToHost, st), "download start");
  SPH_CUDA(cudaStreamSynchronize(st), "cudaStreamSynchronize");
  if (start) {
    for (uint32_t k = 0; k < n; ++k)
      start[k] = st_raw[k + 1] > st_raw[k] ? st_raw[k] - b : 0x7fffffffu;
  }
  if (dens2) {
    float* od = reinterpret_cast<float*>(d_dbg_scratch_);
    SPH_CUDA(launch_export(b, n, d_pos_[cur_], d_vel_[cur_], ctx_.dens_a, nullptr,
                           nullptr, od, nullptr, st), "export kernel");
    SPH_CUDA(cudaMemcpyAsync(dens2, od, 8ull * n, cudaMemcpyDeviceToHost, st),
             "download densities");
    SPH_CUDA(cudaStreamSynchronize(st), "cudaStreamSynchronize");
  }
  return SPH_OK;
}

int Engine::DebugExportLayout(uint32_t id, uint32_t* cell, uint32_t* key,
                              uint32_t* slot_ids, uint32_t* start, uint64_t start_cap,
                              uint32_t* table_len, int* direct, cudaStream_t st) {
  if (id >= max_scenes_ || !scenes_[id].live)
    return Fail(SPH_ERR_INVALID, "no such scene");
  if (!debug_valid_ || id >= scene_dev_.size()) return Fail(SPH_ERR_STATE, "no captured substep");
  const SceneDev& d = scene_dev_[id];
  const uint32_t n = scenes_[id].n;
  const uint32_t b = old_base_[id];  // the captured substep's sorted slots
  const uint64_t T = d.direct ? GridCells(d) : n;
  if (table_len) *table_len = static_cast<uint32_t>(T);
  if (direct) *direct = d.direct ? 1 : 0;
  uint32_t* sc = static_cast<uint32_t*>(d_dbg_scratch_);  // 36 B per particle
  SPH_CUDA(launch_export_layout(b, n, d_scenes_ + id, d_pos_[cur_], ctx_.pred, sc, sc + n,
                                sc + 2ull * n, st), "layout export kernel");
  auto d2h = [&](void* dst, const void* src, size_t bytes) -> cudaError_t {
    if (!dst) return cudaSuccess;
    return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, st);
  };
  SPH_CUDA(d2h(cell, sc, 4ull * n), "download");
  SPH_CUDA(d2h(key, sc + n, 4ull * n), "download");
  SPH_CUDA(d2h(slot_ids, sc + 2ull * n, 4ull * n), "download");
  if (start && start_cap >= T + 1) {
    SPH_CUDA(cudaMemcpyAsync(start, ctx_.start + d.tbase, 4ull * (T + 1),
                             cudaMemcpyDeviceToHost, st), "download start");
  }
  SPH_CUDA(cudaStreamSynchronize(st), "cudaStreamSynchronize");
  if (start && start_cap >= T + 1)
    for (uint64_t k = 0; k <= T; ++k) start[k] -= b;  // slot offsets in the scene
  return SPH_OK;
}

int Engine::Status(uint32_t* flags, cudaStream_t st) {
  uint32_t v = 0;
  SPH_CUDA(cudaMemcpyAsync(&v, d_status_, 4, cudaMemcpyDeviceToHost, st), "status");
  SPH_CUDA(cudaMemsetAsync(d_status_, 0, 4, st), "status reset");
  SPH_CUDA(cudaStreamSynchronize(st), "cudaStreamSynchronize");
  if (flags) *flags = v;
  return SPH_OK;
}

int Engine::SetTuning(const sph_tuning& t) {
  if (t.block < 32 || t.block > 1024 || (t.block & 31))
    return Fail(SPH_ERR_INVALID, "block must be a multiple of 32 in [32, 1024]");
  if (t.particles_per_warp != 32 && t.particles_per_warp != 16)
    return Fail(SPH_ERR_INVALID, "particles_per_warp must be 32 or 16");
  if (t.cell_tile != 1 && t.cell_tile != 64 && t.cell_tile != 128 &&
      t.cell_tile != 192 && t.cell_tile != 256)
    return Fail(SPH_ERR_INVALID, "cell_tile must be 1, 64, 128, 192 or 256");
  if (t.gather != 2 && t.gather != 3 && t.gather != 4 && t.gather != 8)
    return Fail(SPH_ERR_INVALID, "gather must be 2, 3, 4 or 8");
  if (t.force_block != 0 &&
      (t.force_block < 32 || t.force_block > 1024 || (t.force_block & 31)))
    return Fail(SPH_ERR_INVALID, "force_block must be 0 or a multiple of 32 in [32, 1024]");
  if (t.table < 0 || t.table > 2)
    return Fail(SPH_ERR_INVALID, "table must be 0 (automatic), 1 (buckets) or 2 (grid)");
  if (t.block != tuning_.block || t.particles_per_warp != tuning_.particles_per_warp ||
      t.cell_tile != tuning_.cell_tile || t.gather != tuning_.gather ||
      t.force_block != tuning_.force_block)
    ReleaseGraphs();
  if (t.table != tuning_.table) scenes_dirty_ = true;  // new keys and tables
  tuning_ = t;
  return SPH_OK;
}

// Coordinate search: block size x cell tile (all neighbour kernels), then
// the block size of the force kernels alone, then their particles per warp x
// gather batch.
int Engine::Autotune(int substeps, int steps_per_trial, sph_tuning* best,
                     float* best_ms, cudaStream_t st) {
  if (steps_per_trial < 1) return Fail(SPH_ERR_INVALID, "steps_per_trial >= 1");
  // The sweep times real steps. Every live scene's state (positions,
  // velocities, densities and OutPositions, in caller order) is kept on the
  // host meanwhile and loaded back afterwards, so tuning leaves the
  // simulation where it was.
  struct Saved {
    uint32_t id;
    std::vector<float> pos, vel, dens;
    std::vector<float4> out;
  };
  std::vector<Saved> saved;
  for (uint32_t s = 0; s < max_scenes_; ++s) {
    if (!scenes_[s].live) continue;
    const uint32_t n = scenes_[s].n;
    Saved v{s, std::vector<float>(3 * size_t{n}), std::vector<float>(3 * size_t{n}),
            std::vector<float>(2 * size_t{n}), std::vector<float4>(n)};
    const int r = Download(s, v.pos.data(), v.vel.data(), v.dens.data(), false, st);
    if (r != SPH_OK) return r;
    SPH_CUDA(cudaMemcpyAsync(v.out.data(), d_out4_ + old_base_[s], sizeof(float4) * n,
                             cudaMemcpyDeviceToHost, st), "save OutPositions");
    saved.push_back(std::move(v));
  }
  SPH_CUDA(cudaStreamSynchronize(st), "cudaStreamSynchronize");
  // On any failure the caller's tuning comes back (the guard), and the
  // events are released whichever way the sweep ends.
  struct TuningGuard {
    Engine* eng;
    sph_tuning orig;
    bool armed = true;
    ~TuningGuard() {
      if (armed) eng->SetTuning(orig);
    }
  } guard{this, tuning_};
  struct Events {
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    ~Events() {
      if (e0) cudaEventDestroy(e0);
      if (e1) cudaEventDestroy(e1);
    }
  } ev;
  sph_tuning win = tuning_;
  float win_ms = std::numeric_limits<float>::infinity();
  SPH_CUDA(cudaEventCreate(&ev.e0), "cudaEventCreate");
  SPH_CUDA(cudaEventCreate(&ev.e1), "cudaEventCreate");
  cudaEvent_t e0 = ev.e0, e1 = ev.e1;
  const int ppw0 = tuning_.particles_per_warp;
  int rc = SPH_OK;
  for (int round = 0; round < 3 && rc == SPH_OK; ++round) {
    std::vector<sph_tuning> space;
    if (round == 0) {
      for (int b : {64, 128, 256, 512})
        for (int tile : {1, 64, 128, 256})
          space.push_back(sph_tuning{b, tile, ppw0, tuning_.gather, 0, tuning_.table});
    } else if (round == 1) {
      for (int fb : {64, 128, 256, 512})
        space.push_back(sph_tuning{win.block, win.cell_tile, win.particles_per_warp,
                                   win.gather, fb, win.table});
    } else {
      // the force kernels' mapping: particles per warp (one or two lanes a
      // particle) x gather batch
      for (int ppw : {32, 16})
        for (int g : {2, 3, 4, 8})
          space.push_back(sph_tuning{win.block, win.cell_tile, ppw, g, win.force_block,
                                     win.table});
    }
    for (const sph_tuning& t : space) {
      if ((rc = SetTuning(t)) != SPH_OK) break;
      if ((rc = Step(substeps, st)) != SPH_OK) break;  // warm-up + capture
      cudaEventRecord(e0, st);
      for (int k = 0; k < steps_per_trial && rc == SPH_OK; ++k) rc = Step(substeps, st);
      cudaEventRecord(e1, st);
      if (rc != SPH_OK) break;
      cudaEventSynchronize(e1);
      float ms = 0.0f;
      cudaEventElapsedTime(&ms, e0, e1);
      ms /= static_cast<float>(steps_per_trial);
      if (ms < win_ms) { win_ms = ms; win = t; }
    }
  }
  for (const Saved& v : saved) {
    // Load puts the scene back in caller order at its current base, where
    // the saved densities and OutPositions line up slot for slot.
    const int r = Load(v.id, v.pos.data(), v.vel.data(), false, st);
    if (r == SPH_OK) {
      const uint32_t n = scenes_[v.id].n, b = old_base_[v.id];
      SPH_CUDA(cudaMemcpyAsync(ctx_.dens_a + b, v.dens.data(), sizeof(float2) * n,
                               cudaMemcpyHostToDevice, st), "restore densities");
      SPH_CUDA(cudaMemcpyAsync(d_out4_ + b, v.out.data(), sizeof(float4) * n,
                               cudaMemcpyHostToDevice, st), "restore OutPositions");
    }
    if (rc == SPH_OK) rc = r;
  }
  SPH_CUDA(cudaStreamSynchronize(st), "cudaStreamSynchronize");  // host copies die here
  if (rc != SPH_OK) return rc;
  guard.armed = false;
  rc = SetTuning(win);
  if (best) *best = win;
  if (best_ms) *best_ms = win_ms;
  return rc;
}

}  // namespace sph
