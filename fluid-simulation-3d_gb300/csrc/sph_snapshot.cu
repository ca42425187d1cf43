// Scene snapshots: a scene's state and settings in a binary file, for
// checkpoint / resume. The reference has no state I/O (its README lists
// export as future work); this is the engine's own format.
//
// Layout, little-endian (the byte order of every host this builds for):
//   0   8  magic "SPHSNAP1"
//   8   4  version (2)
//  12   4  n, particles
//  16  52  sph_params field by field: radius, cutoff_sq, target_density,
//          pressure_mult, near_pressure_mult, viscosity, gravity_scale
//          (float), gravity_on (int32), bound[3], damping, predict_dt (float)
//  68   4  dt of the scene's steps (float)
//  72   8  FNV-1a 64 of header bytes 0-71 followed by the payload, so a
//          damaged setting is refused like damaged state (version 1 files,
//          whose checksum covers the payload alone, still load)
//  80      payload: positions float[3n], velocities float[3n], densities
//          float[2n] (density, near density), all in the caller's order
// A loaded scene continues bit for bit as if it had never been saved: the
// physics does not depend on the slot layout, and every step recomputes its
// prediction from the stored state.
#include <cstdio>
#include <cstring>
#include <memory>
#include <vector>

#include "sph_engine.h"

namespace sph {
namespace {

constexpr char kMagic[8] = {'S', 'P', 'H', 'S', 'N', 'A', 'P', '1'};
constexpr uint32_t kVersion = 2;
constexpr size_t kHeader = 80;
constexpr size_t kDigestAt = 72;  // header bytes before the digest

uint64_t Fnv1a(const unsigned char* p, size_t bytes, uint64_t h) {
  for (size_t i = 0; i < bytes; ++i) {
    h ^= p[i];
    h *= 1099511628211ull;
  }
  return h;
}

uint64_t Fnv1a(const std::vector<float>& a, uint64_t h) {
  return Fnv1a(reinterpret_cast<const unsigned char*>(a.data()), a.size() * sizeof(float), h);
}

// The checksum of a version-2 file: header bytes 0-71, then the payload
// (head == nullptr: the payload alone, as version 1 wrote it).
uint64_t Digest(const unsigned char* head, const SceneSnapshot& s) {
  uint64_t h = 14695981039346656037ull;
  if (head) h = Fnv1a(head, kDigestAt, h);
  h = Fnv1a(s.pos, h);
  h = Fnv1a(s.vel, h);
  return Fnv1a(s.dens, h);
}

#define SPH_CUDA_RC(call, what)                     \
  do {                                              \
    const cudaError_t e_ = (call);                  \
    if (e_ != cudaSuccess) return CudaFail(e_, what); \
  } while (0)

struct FileCloser {
  void operator()(std::FILE* f) const {
    if (f) std::fclose(f);
  }
};

void Put(std::vector<unsigned char>& out, const void* p, size_t n) {
  const unsigned char* b = static_cast<const unsigned char*>(p);
  out.insert(out.end(), b, b + n);
}

}  // namespace

int Engine::SaveSnapshot(uint32_t id, const char* path, cudaStream_t st) {
  if (!path) return Fail(SPH_ERR_INVALID, "no path");
  if (id >= max_scenes_ || !scenes_[id].live)
    return Fail(SPH_ERR_INVALID, "no such scene");
  SceneSnapshot s;
  const uint32_t n = scenes_[id].n;
  s.prm = scenes_[id].prm;
  s.dt = scenes_[id].dt;
  s.pos.resize(3ull * n);
  s.vel.resize(3ull * n);
  s.dens.resize(2ull * n);
  const int rc = Download(id, s.pos.data(), s.vel.data(), s.dens.data(), false, st);
  if (rc != SPH_OK) return rc;
  std::vector<unsigned char> head;
  head.reserve(kHeader);
  Put(head, kMagic, 8);
  Put(head, &kVersion, 4);
  Put(head, &n, 4);
  const sph_params& p = s.prm;
  const float f7[7] = {p.radius, p.cutoff_sq, p.target_density, p.pressure_mult,
                       p.near_pressure_mult, p.viscosity, p.gravity_scale};
  Put(head, f7, sizeof f7);
  Put(head, &p.gravity_on, 4);
  const float f5[5] = {p.bound[0], p.bound[1], p.bound[2], p.damping, p.predict_dt};
  Put(head, f5, sizeof f5);
  Put(head, &s.dt, 4);
  const uint64_t h = Digest(head.data(), s);
  Put(head, &h, 8);
  if (head.size() != kHeader) return Fail(SPH_ERR_INVALID, "snapshot header layout");
  std::unique_ptr<std::FILE, FileCloser> f(std::fopen(path, "wb"));
  if (!f) return Fail(SPH_ERR_INVALID, std::string("cannot write ") + path);
  bool ok = std::fwrite(head.data(), 1, head.size(), f.get()) == head.size();
  for (const std::vector<float>* a : {&s.pos, &s.vel, &s.dens})
    ok = ok && std::fwrite(a->data(), sizeof(float), a->size(), f.get()) == a->size();
  ok = ok && std::fflush(f.get()) == 0;
  if (!ok) return Fail(SPH_ERR_INVALID, std::string("write failed: ") + path);
  return SPH_OK;
}

int Engine::ReadSnapshot(const char* path, SceneSnapshot* s) {
  if (!path || !s) return Fail(SPH_ERR_INVALID, "no path");
  std::unique_ptr<std::FILE, FileCloser> f(std::fopen(path, "rb"));
  if (!f) return Fail(SPH_ERR_INVALID, std::string("cannot read ") + path);
  unsigned char head[kHeader];
  if (std::fread(head, 1, kHeader, f.get()) != kHeader)
    return Fail(SPH_ERR_INVALID, "snapshot truncated (header)");
  if (std::memcmp(head, kMagic, 8) != 0) return Fail(SPH_ERR_INVALID, "not a snapshot");
  uint32_t version, n;
  std::memcpy(&version, head + 8, 4);
  std::memcpy(&n, head + 12, 4);
  if (version != 1 && version != kVersion)
    return Fail(SPH_ERR_INVALID, "unknown snapshot version");
  if (n == 0 || n >= (1u << 24)) return Fail(SPH_ERR_INVALID, "snapshot size out of range");
  float f7[7], f5[5];
  sph_params& p = s->prm;
  std::memcpy(f7, head + 16, sizeof f7);
  std::memcpy(&p.gravity_on, head + 44, 4);
  std::memcpy(f5, head + 48, sizeof f5);
  std::memcpy(&s->dt, head + 68, 4);
  p.radius = f7[0];
  p.cutoff_sq = f7[1];
  p.target_density = f7[2];
  p.pressure_mult = f7[3];
  p.near_pressure_mult = f7[4];
  p.viscosity = f7[5];
  p.gravity_scale = f7[6];
  p.bound[0] = f5[0];
  p.bound[1] = f5[1];
  p.bound[2] = f5[2];
  p.damping = f5[3];
  p.predict_dt = f5[4];
  uint64_t h;
  std::memcpy(&h, head + 72, 8);
  s->pos.resize(3ull * n);
  s->vel.resize(3ull * n);
  s->dens.resize(2ull * n);
  for (std::vector<float>* a : {&s->pos, &s->vel, &s->dens})
    if (std::fread(a->data(), sizeof(float), a->size(), f.get()) != a->size())
      return Fail(SPH_ERR_INVALID, "snapshot truncated (payload)");
  if (std::fgetc(f.get()) != EOF) return Fail(SPH_ERR_INVALID, "snapshot has trailing bytes");
  if (Digest(version == 1 ? nullptr : head, *s) != h)
    return Fail(SPH_ERR_INVALID, "snapshot checksum mismatch");
  return SPH_OK;
}

int Engine::RestoreSnapshot(uint32_t id, const SceneSnapshot& s, cudaStream_t st) {
  if (id >= max_scenes_ || !scenes_[id].live)
    return Fail(SPH_ERR_INVALID, "no such scene");
  const uint32_t n = static_cast<uint32_t>(s.pos.size() / 3);
  if (n != scenes_[id].n) return Fail(SPH_ERR_INVALID, "snapshot size differs from the scene");
  int rc = SetParams(id, s.prm);
  if (rc == SPH_OK) rc = SetDt(id, s.dt);
  if (rc == SPH_OK) rc = Load(id, s.pos.data(), s.vel.data(), false, st);
  if (rc != SPH_OK) return rc;
  SPH_CUDA_RC(cudaMemcpyAsync(ctx_.dens_a + old_base_[id], s.dens.data(), sizeof(float) * s.dens.size(),
                              cudaMemcpyHostToDevice, st), "restore densities");
  SPH_CUDA_RC(cudaStreamSynchronize(st), "cudaStreamSynchronize");  // host data dies after
  return SPH_OK;
}

int Engine::AddSnapshot(const SceneSnapshot& s, uint32_t* id, cudaStream_t st) {
  const uint32_t n = static_cast<uint32_t>(s.pos.size() / 3);
  uint32_t sid = 0;
  int rc = AddScene(s.prm, n, s.pos.data(), s.vel.data(), false, s.dt, &sid, st);
  if (rc != SPH_OK) return rc;
  SPH_CUDA_RC(cudaMemcpyAsync(ctx_.dens_a + old_base_[sid], s.dens.data(), sizeof(float) * s.dens.size(),
                              cudaMemcpyHostToDevice, st), "restore densities");
  SPH_CUDA_RC(cudaStreamSynchronize(st), "cudaStreamSynchronize");
  if (id) *id = sid;
  return SPH_OK;
}

}  // namespace sph
