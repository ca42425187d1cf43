// Device-side definitions shared by the SPH kernels (sm_103a).
//
// Layout in HBM (one engine, S scenes concatenated, capacity P particles):
//   pos[P], vel[P]      float4 state in the current sorted layout; pos.w holds
//                       the particle's index in its scene as raw bits
//   pred[P]             float4 (predicted position, cell index as raw bits)
//   dens_a[P]           float2 (density, near density)
//   dens_b[P]           float4 (1/rho, P/rho, 1/rho_n, Pn/rho_n)
//   rec_v[2P]           32-byte records (pred, post-pressure velocity): the
//                       Jacobi snapshot the viscosity pass reads
//   keyrank[P]          uint4 (global key, arrival rank in the key bucket,
//                       cell index, particle index)
//   tmp_hi[P], tmp_src[P] bucketed (cell index, particle index) and source
//                       slot, before the order inside each bucket is fixed
//   count[4P+2^16], start[4P+2^16+1] uint32 counting-sort key tables; the
//                       scenes' tables follow one another in layout order
//                       (scene s owns [tbase, tbase + its table size)), so the
//                       prefix at a scene's first key is its first slot. A
//                       table is the scene's grid (one key per cell) or n
//                       buckets (cell index mod n)
//   cell_tab[27P]       bucket tables only: per cell (at its first slot) its
//                       neighbour runs as 9 rows (dy, dz) of 3 runs
//                       (dx = -1, 0, +1); a grid table's rows are read from
//                       start[] directly
//
// The layout is sorted by an internal cell index, not by the reference's
// HashCell key: the index is linear in the cell coordinates with x fastest
// over a grid anchored at the box, so the three x-neighbour cells of a row
// are consecutive keys and, with a grid table or when their buckets hold only
// those cells, one contiguous run of slots. Consecutive slots are then spatial neighbours,
// which the neighbour walks and the force gathers turn into cache hits. The
// set of pairs within the cutoff does not depend on the key function (every
// such pair lies in adjacent cells, and a run holds only its own cell), so
// the physics is the reference's; the reference's own key order
// (spatialLookup / startIndices) is rebuilt on demand by the debug pass.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace sph {

// Hash multipliers of HashCell (engine/physics/physicsWorld.cc:507-509).
constexpr uint32_t kHashX = 15823u;
constexpr uint32_t kHashY = 9737333u;
constexpr uint32_t kHashZ = 440817757u;

// Particles per tile: one warp. Tiles never straddle scenes.
constexpr int kTile = 32;

// Per-scene descriptor, built on the host from sph_params.
struct SceneDev {
  uint32_t n;         // particles
  uint32_t base;      // first slot of the scene's current layout
  uint64_t fm;        // Lemire magic for x % n
  uint32_t tbase;     // first entry of the scene's key table
  uint32_t direct;    // 1: one key per grid cell (key = cell index, the grid
                      //    clamped); 0: n keys, key = cell index % n
  uint32_t gx0, gy0, gz0;  // origin cell of the internal grid (int32 bits)
  uint32_t gnx, gny, gnz;  // grid cells per axis
  uint32_t gwy, gwz;  // y and z strides of the internal cell index
  float r;            // interaction radius
  float cut_lt;       // d2 <= cut_lt  <=>  d2 <= sqrRadius && sqrtf(d2) < r
  float cut_le;       // d2 <= cut_le  <=>  d2 <= sqrRadius && sqrtf(d2) <= r
  float cut_hi;       // cut_le widened by 2e-6 relative: bounds the FMA
                      // estimate of d2 for every pair with d2 <= cut_le
  float cut_lo;       // cut_lt narrowed by 2e-6: an FMA estimate below it
                      // certifies d2 <= cut_lt without the exact recompute
  float r2;           // r*r
  float vol2, vol3;   // density kernel scales   (kernels.h:28,40)
  float ds2h, ds3h;   // 0.5 * derivative scales (kernels.h:52,64)
  float vscale;       // poly6 scale             (kernels.h:76)
  float rho0, k, kn, mu;
  float gy;           // -gravityScale if gravity else 0   (:313-323)
  float hx, hy, hz;   // BoundScale * 0.5                   (:88)
  float ndamp;        // -1 * dampFactor                    (:94)
  float pdt;          // prediction look-ahead 1/120        (:47)
  float dt;           // substep dt
};

// x % d for 32-bit x, d >= 1, with M = floor((2^64-1)/d) + 1 (Lemire et al.,
// "Faster Remainder by Direct Computation", 2019).
__device__ __forceinline__ uint32_t fastmod(uint32_t x, uint64_t M,
                                            uint32_t d) {
  const uint64_t low = M * static_cast<uint64_t>(x);
  return static_cast<uint32_t>(__umul64hi(low, static_cast<uint64_t>(d)));
}

// Gravity + prediction of physicsWorld.cc:45-47 with the reference's
// rounding (separate multiply and add, no FMA contraction).
__device__ __forceinline__ void predict(const SceneDev& S, float4 p, float4 v,
                                        float3& vn, float3& pr) {
  vn.x = __fadd_rn(v.x, __fmul_rn(0.0f, S.dt));
  vn.y = __fadd_rn(v.y, __fmul_rn(S.gy, S.dt));
  vn.z = __fadd_rn(v.z, __fmul_rn(0.0f, S.dt));
  pr.x = __fadd_rn(p.x, __fmul_rn(vn.x, S.pdt));
  pr.y = __fadd_rn(p.y, __fmul_rn(vn.y, S.pdt));
  pr.z = __fadd_rn(p.z, __fmul_rn(vn.z, S.pdt));
}

// PositionToCellCoord (physicsWorld.cc:499-503): floor of the IEEE quotient.
__device__ __forceinline__ int cell_of(float p, float r) {
  return static_cast<int>(floorf(__fdiv_rn(p, r)));
}

// HashCell (physicsWorld.cc:505-511); the float->uint32 cast wraps modulo
// 2^32 as on x86-64.
__device__ __forceinline__ uint32_t hash_cell(int cx, int cy, int cz) {
  return static_cast<uint32_t>(cx) * kHashX + static_cast<uint32_t>(cy) * kHashY +
         static_cast<uint32_t>(cz) * kHashZ;
}

__device__ __forceinline__ uint32_t hash_of(const SceneDev& S, float3 pr) {
  return hash_cell(cell_of(pr.x, S.r), cell_of(pr.y, S.r), cell_of(pr.z, S.r));
}

// Grid coordinate of cell c along one axis, clamped to [1, count - 2]: the
// grid's first and last cells stay empty, so the three x-neighbours of any
// occupied cell are consecutive indices of one row. Clamping is monotone, so
// cells that are neighbours stay neighbours (a cell beyond the grid shares
// the edge cell with the cells between, and the cutoff test drops the extra
// candidates this brings).
// (The origin lies in [-1e9, 1e9] and count in [5, 2^15], so the bounds fit
// an int.)
__device__ __forceinline__ uint32_t grid_coord(int c, uint32_t origin, uint32_t count) {
  const int lo = static_cast<int>(origin) + 1;
  const int hi = lo + static_cast<int>(count) - 3;
  return static_cast<uint32_t>(min(max(c, lo), hi) - lo) + 1u;
}

// Internal cell index of the sort (the reference's cells, another key):
// (cx - x0) + (cy - y0) * wy + (cz - z0) * wz, with the coordinates clamped
// to the grid for a direct table, else modulo 2^32. Linear in the cell
// coordinates like HashCell, so index(c + d) = index(c) + dx + dy*wy + dz*wz
// for every occupied cell, and distinct neighbour offsets never share an
// index (|dx + dy*wy + dz*wz| < 2^32).
__device__ __forceinline__ uint32_t cell_index(const SceneDev& S, float3 pr) {
  const int x = cell_of(pr.x, S.r), y = cell_of(pr.y, S.r), z = cell_of(pr.z, S.r);
  if (S.direct)
    return grid_coord(x, S.gx0, S.gnx) + grid_coord(y, S.gy0, S.gny) * S.gwy +
           grid_coord(z, S.gz0, S.gnz) * S.gwz;
  return (static_cast<uint32_t>(x) - S.gx0) + (static_cast<uint32_t>(y) - S.gy0) * S.gwy +
         (static_cast<uint32_t>(z) - S.gz0) * S.gwz;
}

// Key-table entry of a cell: its own entry in a direct table, else its
// bucket, cell index mod n (a bucket may then hold several cells).
__device__ __forceinline__ uint32_t table_key(const SceneDev& S, uint32_t cell) {
  return S.tbase + (S.direct ? cell : fastmod(cell, S.fm, S.n));
}

// Run-length flag of a cell-table row whose three x-runs are one contiguous
// run (stored in the row's first entry; the other two entries of such a row
// are not written and must not be read).
constexpr uint32_t kRunMerged = 0x80000000u;

}  // namespace sph
