// Host-visible declarations of the SPH kernels' launchers.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "sph_device.cuh"

namespace sph {

constexpr uint32_t kStatusNonFinite = 0x1u;
constexpr uint32_t kStatusRange = 0x2u;

// A tile is (scene | (len-1) << 27, first slot): up to 32 consecutive slots
// of one scene.
constexpr uint32_t kTileSceneBits = 27;
__host__ __device__ __forceinline__ uint32_t tile_scene(uint2 t) {
  return t.x & ((1u << kTileSceneBits) - 1u);
}
__host__ __device__ __forceinline__ uint32_t tile_len(uint2 t) {
  return (t.x >> kTileSceneBits) + 1u;
}
__host__ __device__ __forceinline__ uint2 make_tile(uint32_t scene,
                                                    uint32_t first,
                                                    uint32_t len) {
  return make_uint2(scene | ((len - 1u) << kTileSceneBits), first);
}

// glm::sign for floats: 1, -1, or 0 for +-0 and NaN.
__device__ __forceinline__ float copysign_or_zero(float x) {
  return static_cast<float>(0.0f < x) - static_cast<float>(x < 0.0f);
}

struct Tiles {
  const uint2* d = nullptr;  // device tile table
  uint32_t n = 0;
};

// Device buffers and launch shape used by one engine.
// Key-table forms present in a launch: the neighbour kernels are compiled
// for direct tables only, bucket tables only, or both (chosen per scene).
enum TableForms : int { kTablesMixed = 0, kTablesDirect = 1, kTablesBuckets = 2 };

struct LaunchCtx {
  const SceneDev* scenes = nullptr;
  float4* pos = nullptr;   // state A (read at substep start)
  float4* vel = nullptr;
  float4* pos2 = nullptr;  // state B (written by the reorder)
  float4* vel2 = nullptr;
  float4* pred = nullptr;
  float4* rec_v = nullptr;  // 2 per slot: (pred, post-pressure velocity)
  float2* dens_a = nullptr;
  float4* dens_b = nullptr;  // (1/rho, P/rho, 1/rho_n, Pn/rho_n) per slot
  uint4* keyrank = nullptr;   // (key, arrival rank, cell, id) per old slot
  uint2* tmp_hi = nullptr;    // (cell, id) per bucketed slot
  uint32_t* tmp_src = nullptr;  // source slot per bucketed slot
  uint32_t* hash_s = nullptr;   // internal cell index per sorted slot
  uint32_t* cell_first = nullptr;  // first slot of the particle's cell
  uint2* cell_tab = nullptr;    // per cell (first slot): 9 rows x 3 runs
  uint32_t* count = nullptr;
  uint32_t* start = nullptr;
  uint32_t* partial = nullptr;
  uint32_t* nbr = nullptr;      // neighbour lists, nbr[k * nbr_stride + slot]
  uint32_t* ncount = nullptr;   // neighbours per slot (> nbr_cap: overflow)
  uint32_t nbr_stride = 0;
  uint32_t nbr_cap = 0;
  int gather = 2;               // neighbour entries gathered per batch (2, 3, 4, 8)
  int lanes = 1;                // lanes per particle in the force kernels (1 or 2:
                                // 32 or 16 particles per warp)
  int cell_tile = 1;            // density-pass candidates held per cell tile
                                // (1: thread-per-particle walk)
  int tables = kTablesMixed;    // key-table forms of the live scenes
  float4* out4 = nullptr;
  uint32_t* status = nullptr;
  float4* dbg_accp = nullptr;   // captured substep: per-slot intermediates
  float4* dbg_velv = nullptr;
  // captured substep: the reference's spatial lookup (launch_ref_lookup)
  uint32_t* dbg_hash = nullptr;     // HashCell per particle (base + index)
  uint32_t* dbg_key = nullptr;      // hash % n per particle (base + index)
  uint32_t* dbg_count = nullptr;    // key histogram (zero between uses)
  uint32_t* dbg_start = nullptr;    // startIndices as slot offsets
  uint32_t* dbg_partial = nullptr;  // scan partials
  uint2* dbg_keyrank = nullptr;     // (key, arrival rank) per slot
  uint32_t* dbg_tmp = nullptr;      // bucketed particle indices
  uint32_t* dbg_sorted = nullptr;   // (key, index)-ordered particle indices
  uint32_t src_limit = 0;  // slots of the layout a substep reads
  bool pdl = true;        // programmatic dependent launch (off while the
                          // engine records phase events between kernels)
  int block_misc = 256;   // predict/scatter/reorder
  int block_nbr = 128;    // neighbour kernels (density)
  int block_force = 128;  // pressure and viscosity
  uint32_t max_blocks = 0;  // persistent grid cap (0 = no cap)
};

inline uint32_t grid_for(uint32_t ntiles, int block, uint32_t max_blocks) {
  const uint32_t wpb = static_cast<uint32_t>(block) / 32u;
  uint32_t g = (ntiles + wpb - 1) / wpb;
  if (max_blocks && g > max_blocks) g = max_blocks;
  return g == 0 ? 1 : g;
}

uint32_t scan_partials_needed(uint64_t len);

cudaError_t launch_predict_hash(const LaunchCtx& c, const Tiles& old_tiles,
                                cudaStream_t st);
cudaError_t launch_scan(const LaunchCtx& c, uint32_t len, cudaStream_t st);
cudaError_t launch_sort_reorder(const LaunchCtx& c, const Tiles& old_tiles,
                                const Tiles& new_tiles, uint32_t total,
                                cudaStream_t st);
cudaError_t launch_density(const LaunchCtx& c, const Tiles& tiles,
                           cudaStream_t st);
cudaError_t launch_pressure(const LaunchCtx& c, const Tiles& tiles,
                            cudaStream_t st);
cudaError_t launch_visc_integrate(const LaunchCtx& c, const Tiles& tiles,
                                  int fuse_next, int write_out,
                                  cudaStream_t st);

// Kernels launched by one substep over a key table of `keys` entries (scan 2
// or 3, scatter, reorder, cell table unless every table is direct, density,
// pressure, viscosity), and by the standalone prediction of a step's first
// substep.
int kernels_per_substep(uint32_t keys, int tables);
constexpr int kKernelsPredict = 1;
cudaError_t launch_export(uint32_t first, uint32_t n, const float4* pos,
                          const float4* vel, const float2* dens, float* opos,
                          float* ovel, float* odens, uint32_t* oids,
                          cudaStream_t st);
// The same rows written into host memory the device maps (pinned, every
// output 16-byte aligned; nullptr outputs are skipped), in caller order,
// through slot_of[n] (device scratch, overwritten).
cudaError_t launch_export_rows(uint32_t first, uint32_t n, const float4* pos,
                              const float4* vel, const float2* dens, uint32_t* slot_of,
                              float* opos, float* ovel, float* odens, cudaStream_t st);
cudaError_t launch_export_debug(uint32_t first, uint32_t n, const float4* pos,
                                const float4* accp, const float4* velp,
                                const float4* velv, float* oaccp, float* ovelp,
                                float* ovelv, cudaStream_t st);
// The timed sort's layout of scene slots [first, first + n) after a
// captured substep: caller index per slot (oslot[n]), and per caller index
// the internal cell index (ocell[n]) and key-table entry relative to the
// scene's table (okey[n]). All device pointers.
cudaError_t launch_export_layout(uint32_t first, uint32_t n, const SceneDev* scene,
                                 const float4* pos, const float4* pred, uint32_t* ocell,
                                 uint32_t* okey, uint32_t* oslot, cudaStream_t st);
// The reference's spatial lookup of the substep being launched (after its
// sort): k_ref_hash, the scan, k_ref_scatter, k_ref_order into the dbg_*
// buffers of `c`.
cudaError_t launch_ref_lookup(const LaunchCtx& c, const Tiles& new_tiles,
                              uint32_t total, cudaStream_t st);
cudaError_t launch_import(uint32_t first, uint32_t n, const float* ipos,
                          const float* ivel, float4* pos, float4* vel,
                          cudaStream_t st);
// The same import reading host memory the device addresses directly (pinned
// buffers, 16-byte aligned): rows move as aligned float4 per warp. With
// `scene` (the scene's device constants) it also writes the next step's
// first prediction (keyrank, histogram in count) as k_predict_hash does.
cudaError_t launch_import_rows(uint32_t first, uint32_t n, const float* ipos,
                               const float* ivel, float4* pos, float4* vel,
                               const SceneDev* scene, uint32_t* count, uint4* keyrank,
                               cudaStream_t st);

}  // namespace sph
