// SPH substep kernels for GB300 (sm_103a).
//
// One substep (engine/physics/physicsWorld.cc:39-111) is:
//   k_predict_hash   gravity + prediction + cell hash + key, counting-sort
//                    histogram (atomic arrival rank)        :42-48, :473-482
//   k_scan_*         exclusive prefix of the key histogram = start table
//   k_scatter        bucket each particle at start[key] + rank
//   k_reorder        canonical (key, index) order inside each bucket and
//                    gather of the state into SoA float4      :484-496
//   k_density        density / near density                  :304-365
//   k_pressure       pressure + near pressure -> velocity     :367-422
//   k_visc_integrate Jacobi viscosity, integrate, box collision, and the
//                    next substep's k_predict_hash fused in  :424-464, :81-108
// Every kernel is a persistent, segmented launch: warps stride over a tile
// table whose entries are (scene, first slot) runs of 32 particles, so one
// launch serves any number of scenes of uneven sizes.
#include "sph_kernels.h"

#include <cstdio>

namespace sph {

namespace {

constexpr uint32_t Delta(int o) {
  return static_cast<uint32_t>(o / 9 - 1) * kHashX +
         static_cast<uint32_t>((o / 3) % 3 - 1) * kHashY +
         static_cast<uint32_t>(o % 3 - 1) * kHashZ;
}

__constant__ uint32_t c_delta[27] = {
    Delta(0),  Delta(1),  Delta(2),  Delta(3),  Delta(4),  Delta(5),  Delta(6),
    Delta(7),  Delta(8),  Delta(9),  Delta(10), Delta(11), Delta(12), Delta(13),
    Delta(14), Delta(15), Delta(16), Delta(17), Delta(18), Delta(19), Delta(20),
    Delta(21), Delta(22), Delta(23), Delta(24), Delta(25), Delta(26)};

__device__ __forceinline__ uint32_t warp_id_global() {
  return blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
}
__device__ __forceinline__ uint32_t warps_total() {
  return gridDim.x * (blockDim.x >> 5);
}

// glm dot(v, v) of physicsWorld.cc:355: three rounded products summed left to
// right (no FMA contraction), so boundary pairs classify as in the reference.
__device__ __forceinline__ float dist2(float dx, float dy, float dz) {
  return __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)),
                   __fmul_rn(dz, dz));
}

__device__ __forceinline__ void flag(uint32_t* status, uint32_t f) {
  atomicOr(status, f);
}

// Walk of the 27 neighbour buckets in the reference's order
// (CalculateDensity :331-363 and the force loops): for each offset cell,
// scan [start[key], start[key+1]) and keep entries whose float(hash) equals
// the cell's (the reference stores the hash as a float, :480, :346).
template <class F>
__device__ __forceinline__ void walk27(const SceneDev& S,
                                       const uint32_t* __restrict__ start,
                                       const float4* __restrict__ pred,
                                       float3 p, F&& visit) {
  const uint32_t hc = hash_cell(cell_of(p.x, S.r), cell_of(p.y, S.r),
                                cell_of(p.z, S.r));
#pragma unroll 1
  for (int o = 0; o < 27; ++o) {
    const uint32_t h = hc + c_delta[o];
    const uint32_t key = S.base + fastmod(h, S.fm, S.n);
    const float hf = __uint2float_rn(h);
    const uint32_t b0 = __ldg(start + key);
    const uint32_t b1 = __ldg(start + key + 1);
#pragma unroll 1
    for (uint32_t j = b0; j < b1; ++j) {
      const float4 q = __ldg(pred + j);
      if (q.w != hf) continue;
      visit(j, q);
    }
  }
}

// ----------------------------------------------------------------- predict
__device__ __forceinline__ void predict_key(const SceneDev& S, float4 p,
                                            float4 v, uint32_t& key,
                                            uint32_t& hash) {
  float3 vn, pr;
  predict(S, p, v, vn, pr);
  hash = hash_of(S, pr);
  key = S.base + fastmod(hash, S.fm, S.n);
}

__global__ void k_predict_hash(const uint2* __restrict__ tiles, uint32_t ntiles,
                               const SceneDev* __restrict__ scenes,
                               const float4* __restrict__ pos,
                               const float4* __restrict__ vel,
                               uint32_t* __restrict__ count,
                               uint2* __restrict__ keyrank) {
  const int lane = threadIdx.x & 31;
  for (uint32_t t = warp_id_global(); t < ntiles; t += warps_total()) {
    const uint2 tile = tiles[t];
    const SceneDev S = scenes[tile_scene(tile)];
    const uint32_t s = tile.y + lane;
    if (static_cast<uint32_t>(lane) >= tile_len(tile)) continue;
    uint32_t key, hash;
    predict_key(S, pos[s], vel[s], key, hash);
    const uint32_t r = atomicAdd(count + key, 1u);
    keyrank[s] = make_uint2(key, r);
  }
}

// -------------------------------------------------------------------- scan
constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanBlock = kScanThreads * kScanItems;

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t x) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, d);
    if (lane >= d) x += y;
  }
  return x;
}

// Block-wide exclusive scan of one value per thread; returns the block total
// through *total.
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t x,
                                                    uint32_t* total) {
  __shared__ uint32_t warp_sums[32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const uint32_t incl = warp_incl_scan(x);
  if (lane == 31) warp_sums[w] = incl;
  __syncthreads();
  if (w == 0) {
    const int nw = blockDim.x >> 5;
    uint32_t v = lane < nw ? warp_sums[lane] : 0u;
    v = warp_incl_scan(v);
    warp_sums[lane] = v;
  }
  __syncthreads();
  const uint32_t before = w > 0 ? warp_sums[w - 1] : 0u;
  *total = warp_sums[(blockDim.x >> 5) - 1];
  __syncthreads();
  return before + incl - x;
}

__global__ void __launch_bounds__(kScanThreads)
k_scan_reduce(const uint32_t* __restrict__ count, uint32_t len,
              uint32_t* __restrict__ partial) {
  const uint32_t b0 = blockIdx.x * kScanBlock + threadIdx.x * kScanItems;
  uint32_t s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k)
    if (b0 + k < len) s += count[b0 + k];
  uint32_t total;
  block_excl_scan(s, &total);
  if (threadIdx.x == 0) partial[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kScanThreads)
k_scan_partials(uint32_t* __restrict__ partial, uint32_t nb,
                uint32_t* __restrict__ start, uint32_t len) {
  uint32_t carry = 0;
  for (uint32_t c = 0; c < nb; c += kScanThreads) {
    const uint32_t i = c + threadIdx.x;
    const uint32_t v = i < nb ? partial[i] : 0u;
    uint32_t total;
    const uint32_t ex = block_excl_scan(v, &total);
    if (i < nb) partial[i] = carry + ex;
    carry += total;
  }
  if (threadIdx.x == 0) start[len] = carry;
}

__global__ void __launch_bounds__(kScanThreads)
k_scan_down(uint32_t* __restrict__ count, uint32_t len,
            const uint32_t* __restrict__ partial,
            uint32_t* __restrict__ start) {
  const uint32_t b0 = blockIdx.x * kScanBlock + threadIdx.x * kScanItems;
  uint32_t v[kScanItems];
  uint32_t s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    v[k] = (b0 + k < len) ? count[b0 + k] : 0u;
    s += v[k];
  }
  uint32_t total;
  uint32_t run = block_excl_scan(s, &total) + partial[blockIdx.x];
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    if (b0 + k < len) {
      start[b0 + k] = run;
      count[b0 + k] = 0u;  // ready for the next substep's histogram
    }
    run += v[k];
  }
}

// ----------------------------------------------------------------- scatter
__global__ void k_scatter(const uint2* __restrict__ tiles, uint32_t ntiles,
                          const SceneDev* __restrict__ scenes,
                          const uint2* __restrict__ keyrank,
                          const uint32_t* __restrict__ start,
                          const float4* __restrict__ pos, uint32_t total,
                          uint2* __restrict__ tmp, uint32_t* status) {
  const int lane = threadIdx.x & 31;
  for (uint32_t t = warp_id_global(); t < ntiles; t += warps_total()) {
    const uint2 tile = tiles[t];
    const SceneDev S = scenes[tile_scene(tile)];
    const uint32_t s = tile.y + lane;
    if (static_cast<uint32_t>(lane) >= tile_len(tile)) continue;
    const uint2 kr = keyrank[s];
    const uint32_t dst = start[kr.x] + kr.y;
    if (dst >= total) { flag(status, kStatusRange); continue; }
    tmp[dst] = make_uint2(__float_as_uint(pos[s].w), s);
  }
}

// ----------------------------------------------------------------- reorder
// Thread per bucketed slot t: rank the particle among its bucket by index
// (canonical (key, index) order), recompute its gravity/prediction exactly
// as k_predict_hash did, and write the state to its final slot.
__global__ void k_reorder(const uint2* __restrict__ tiles, uint32_t ntiles,
                          const SceneDev* __restrict__ scenes,
                          const uint2* __restrict__ tmp,
                          const uint32_t* __restrict__ start,
                          const float4* __restrict__ pos_in,
                          const float4* __restrict__ vel_in,
                          float4* __restrict__ pos_out,
                          float4* __restrict__ vel_out,
                          float4* __restrict__ pred,
                          uint32_t* __restrict__ dbg_hash,
                          uint32_t* __restrict__ dbg_key, uint32_t src_limit,
                          uint32_t* status) {
  const int lane = threadIdx.x & 31;
  for (uint32_t t = warp_id_global(); t < ntiles; t += warps_total()) {
    const uint2 tile = tiles[t];
    const SceneDev S = scenes[tile_scene(tile)];
    const uint32_t slot = tile.y + lane;
    if (static_cast<uint32_t>(lane) >= tile_len(tile)) continue;
    const uint2 me = tmp[slot];
    if (me.y >= src_limit) { flag(status, kStatusRange); continue; }
    const float4 p = pos_in[me.y];
    const float4 v = vel_in[me.y];
    float3 vn, pr;
    predict(S, p, v, vn, pr);
    const uint32_t hash = hash_of(S, pr);
    const uint32_t key = S.base + fastmod(hash, S.fm, S.n);
    const uint32_t b0 = start[key], b1 = start[key + 1];
    if (slot < b0 || slot >= b1) { flag(status, kStatusRange); continue; }
    uint32_t rank = 0;
    for (uint32_t u = b0; u < b1; ++u) rank += (tmp[u].x < me.x) ? 1u : 0u;
    const uint32_t f = b0 + rank;
    pos_out[f] = p;
    vel_out[f] = make_float4(vn.x, vn.y, vn.z, 0.0f);
    pred[f] = make_float4(pr.x, pr.y, pr.z, __uint2float_rn(hash));
    if (dbg_hash) {
      dbg_hash[f] = hash;
      dbg_key[f] = key - S.base;
    }
  }
}

// ----------------------------------------------------------------- density
// CalculateDensity (:325-365), self included. The kernel condition
// `sqrDist <= sqrRadius && dist < r` is the exact float test d2 <= cut_lt.
__global__ void k_density(const uint2* __restrict__ tiles, uint32_t ntiles,
                          const SceneDev* __restrict__ scenes,
                          const float4* __restrict__ pred,
                          const uint32_t* __restrict__ start,
                          float2* __restrict__ dens_a,
                          float4* __restrict__ dens_b) {
  const int lane = threadIdx.x & 31;
  for (uint32_t t = warp_id_global(); t < ntiles; t += warps_total()) {
    const uint2 tile = tiles[t];
    const SceneDev S = scenes[tile_scene(tile)];
    const uint32_t i = tile.y + lane;
    if (static_cast<uint32_t>(lane) >= tile_len(tile)) continue;
    const float4 pi = pred[i];
    const float3 p = make_float3(pi.x, pi.y, pi.z);
    float s2 = 0.0f, s3 = 0.0f;
    walk27(S, start, pred, p, [&](uint32_t, float4 q) {
      const float dx = q.x - p.x, dy = q.y - p.y, dz = q.z - p.z;
      const float d2 = dist2(dx, dy, dz);
      if (d2 <= S.cut_lt) {
        const float w = S.r - __fsqrt_rn(d2);
        const float w2 = w * w;
        s2 += w2;
        s3 += w2 * w;
      }
    });
    const float rho = s2 * S.vol2, rhon = s3 * S.vol3;
    dens_a[i] = make_float2(rho, rhon);
    const float ir = 1.0f / rho, irn = 1.0f / rhon;
    const float P = (rho - S.rho0) * S.k, Pn = rhon * S.kn;
    dens_b[i] = make_float4(ir, P * ir, irn, Pn * irn);
  }
}

// ---------------------------------------------------------------- pressure
// CalculatePressureForce (:367-422), self skipped. The shared pressure over
// the neighbour's density is 0.5*(Pi + Pj)/rho_j = 0.5*(Pi*(1/rho_j) +
// Pj/rho_j); the 0.5 is folded into ds2h/ds3h.
__global__ void k_pressure(const uint2* __restrict__ tiles, uint32_t ntiles,
                           const SceneDev* __restrict__ scenes,
                           const float4* __restrict__ pred,
                           const uint32_t* __restrict__ start,
                           const float2* __restrict__ dens_a,
                           const float4* __restrict__ dens_b,
                           const float4* __restrict__ vel,
                           float4* __restrict__ velp,
                           float4* __restrict__ dbg_accp) {
  const int lane = threadIdx.x & 31;
  for (uint32_t t = warp_id_global(); t < ntiles; t += warps_total()) {
    const uint2 tile = tiles[t];
    const SceneDev S = scenes[tile_scene(tile)];
    const uint32_t i = tile.y + lane;
    if (static_cast<uint32_t>(lane) >= tile_len(tile)) continue;
    const float4 pi = pred[i];
    const float3 p = make_float3(pi.x, pi.y, pi.z);
    const float2 di = dens_a[i];
    const float Pi = (di.x - S.rho0) * S.k, Pni = di.y * S.kn;
    float fx = 0.0f, fy = 0.0f, fz = 0.0f;
    walk27(S, start, pred, p, [&](uint32_t j, float4 q) {
      if (j == i) return;
      const float dx = q.x - p.x, dy = q.y - p.y, dz = q.z - p.z;
      const float d2 = dist2(dx, dy, dz);
      if (d2 <= S.cut_le) {
        const float4 b = __ldg(dens_b + j);
        const float dist = __fsqrt_rn(d2);
        const float inv = d2 > 0.0f ? rsqrtf(d2) : 0.0f;
        const float w = S.r - dist;
        const float a2 = S.ds2h * fmaf(Pi, b.x, b.y);
        const float a3 = S.ds3h * w * fmaf(Pni, b.z, b.w);
        const float tsum = -w * (a2 + a3);
        if (d2 > 0.0f) {
          const float s = tsum * inv;
          fx += dx * s; fy += dy * s; fz += dz * s;
        } else {
          fy += tsum;  // dir = (0,1,0) for coincident particles (:414)
        }
      }
    });
    const float inv_rho = 1.0f / di.x;
    const float ax = fx * inv_rho, ay = fy * inv_rho, az = fz * inv_rho;
    const float4 v = vel[i];
    velp[i] = make_float4(v.x + ax * S.dt, v.y + ay * S.dt, v.z + az * S.dt, 0.f);
    if (dbg_accp) dbg_accp[i] = make_float4(ax, ay, az, 0.0f);
  }
}

// ------------------------------------------------ viscosity + integrate
// CalculateViscosityForce (:424-464) reading the post-pressure snapshot
// (Jacobi), then pos += v*dt and the box collision (:81-108). poly6 uses
// r^2 - d2 for r*r - dist*dist. With next_dt > 0 the next substep's
// prediction/hash/histogram (k_predict_hash) runs here on the new state.
__global__ void k_visc_integrate(
    const uint2* __restrict__ tiles, uint32_t ntiles,
    const SceneDev* __restrict__ scenes, const float4* __restrict__ pred,
    const uint32_t* __restrict__ start, const float4* __restrict__ velp,
    float4* __restrict__ pos, float4* __restrict__ vel,
    float4* __restrict__ out4, int fuse_next, uint32_t* __restrict__ count,
    uint2* __restrict__ keyrank, float4* __restrict__ dbg_velv,
    uint32_t* status) {
  const int lane = threadIdx.x & 31;
  for (uint32_t t = warp_id_global(); t < ntiles; t += warps_total()) {
    const uint2 tile = tiles[t];
    const SceneDev S = scenes[tile_scene(tile)];
    const uint32_t i = tile.y + lane;
    const bool live = static_cast<uint32_t>(lane) < tile_len(tile);
    bool bad = false;
    if (live) {
      const float4 pi = pred[i];
      const float3 p = make_float3(pi.x, pi.y, pi.z);
      const float4 vi = velp[i];
      float fx = 0.0f, fy = 0.0f, fz = 0.0f;
      walk27(S, start, pred, p, [&](uint32_t j, float4 q) {
        if (j == i) return;
        const float dx = q.x - p.x, dy = q.y - p.y, dz = q.z - p.z;
        const float d2 = dist2(dx, dy, dz);
        if (d2 <= S.cut_lt) {
          const float dist = __fsqrt_rn(d2);
          const float w = __fsub_rn(S.r2, __fmul_rn(dist, dist));
          const float w3 = w * w * w;
          const float4 vj = __ldg(velp + j);
          fx += (vj.x - vi.x) * w3;
          fy += (vj.y - vi.y) * w3;
          fz += (vj.z - vi.z) * w3;
        }
      });
      const float c = S.vscale * S.mu * S.dt;
      float3 v = make_float3(vi.x + fx * c, vi.y + fy * c, vi.z + fz * c);
      if (dbg_velv) dbg_velv[i] = make_float4(v.x, v.y, v.z, 0.0f);
      float4 x = pos[i];
      x.x = __fadd_rn(x.x, __fmul_rn(v.x, S.dt));
      x.y = __fadd_rn(x.y, __fmul_rn(v.y, S.dt));
      x.z = __fadd_rn(x.z, __fmul_rn(v.z, S.dt));
      // edgeDst = halfSize - |pos|; if <= 0 clamp to the wall and reflect.
      if (S.hx - fabsf(x.x) <= 0.0f) { x.x = S.hx * copysign_or_zero(x.x); v.x *= S.ndamp; }
      if (S.hy - fabsf(x.y) <= 0.0f) { x.y = S.hy * copysign_or_zero(x.y); v.y *= S.ndamp; }
      if (S.hz - fabsf(x.z) <= 0.0f) { x.z = S.hz * copysign_or_zero(x.z); v.z *= S.ndamp; }
      pos[i] = x;
      const float4 v4 = make_float4(v.x, v.y, v.z, 0.0f);
      vel[i] = v4;
      bad = !(isfinite(x.x) && isfinite(x.y) && isfinite(x.z) &&
              isfinite(v.x) && isfinite(v.y) && isfinite(v.z));
      if (out4) {
        const uint32_t id = __float_as_uint(x.w);
        if (id < S.n) out4[S.base + id] = make_float4(x.x, x.y, x.z, 0.34f);
        else bad = true;
      }
      if (fuse_next) {
        uint32_t key, hash;
        predict_key(S, x, v4, key, hash);
        const uint32_t r = atomicAdd(count + key, 1u);
        keyrank[i] = make_uint2(key, r);
      }
    }
    if (__any_sync(0xffffffffu, bad) && lane == 0) flag(status, kStatusNonFinite);
  }
}

// ------------------------------------------------------------ readback
// Gather a scene's slot-ordered arrays into the caller's particle order.
__global__ void k_export(uint32_t first, uint32_t n,
                         const float4* __restrict__ pos,
                         const float4* __restrict__ vel,
                         const float2* __restrict__ dens,
                         float* __restrict__ opos, float* __restrict__ ovel,
                         float* __restrict__ odens,
                         uint32_t* __restrict__ oids) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const uint32_t s = first + k;
  const float4 p = pos[s];
  const uint32_t id = __float_as_uint(p.w);
  if (id >= n) return;
  if (oids) oids[k] = id;
  if (opos) { opos[3 * id] = p.x; opos[3 * id + 1] = p.y; opos[3 * id + 2] = p.z; }
  if (ovel) {
    const float4 v = vel[s];
    ovel[3 * id] = v.x; ovel[3 * id + 1] = v.y; ovel[3 * id + 2] = v.z;
  }
  if (odens) {
    const float2 d = dens[s];
    odens[2 * id] = d.x; odens[2 * id + 1] = d.y;
  }
}

// Debug intermediates of one scene to caller order.
__global__ void k_export_debug(uint32_t first, uint32_t n,
                               const float4* __restrict__ pos,
                               const uint32_t* __restrict__ dhash,
                               const uint32_t* __restrict__ dkey,
                               const float4* __restrict__ accp,
                               const float4* __restrict__ velp,
                               const float4* __restrict__ velv,
                               uint32_t* __restrict__ ohash,
                               uint32_t* __restrict__ okey,
                               float* __restrict__ oaccp,
                               float* __restrict__ ovelp,
                               float* __restrict__ ovelv) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const uint32_t s = first + k;
  const uint32_t id = __float_as_uint(pos[s].w);
  if (id >= n) return;
  ohash[id] = dhash[s];
  okey[id] = dkey[s];
  const float4 a = accp[s], b = velp[s], c = velv[s];
  oaccp[3 * id] = a.x; oaccp[3 * id + 1] = a.y; oaccp[3 * id + 2] = a.z;
  ovelp[3 * id] = b.x; ovelp[3 * id + 1] = b.y; ovelp[3 * id + 2] = b.z;
  ovelv[3 * id] = c.x; ovelv[3 * id + 1] = c.y; ovelv[3 * id + 2] = c.z;
}

// Load caller-order AoS arrays into a scene's slots (identity layout).
__global__ void k_import(uint32_t first, uint32_t n,
                         const float* __restrict__ ipos,
                         const float* __restrict__ ivel,
                         float4* __restrict__ pos, float4* __restrict__ vel) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  pos[first + k] = ipos ? make_float4(ipos[3 * k], ipos[3 * k + 1],
                                      ipos[3 * k + 2], __uint_as_float(k))
                       : make_float4(0.0f, 0.0f, 0.0f, __uint_as_float(k));
  vel[first + k] = ivel ? make_float4(ivel[3 * k], ivel[3 * k + 1],
                                      ivel[3 * k + 2], 0.0f)
                        : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
}

}  // namespace

// ------------------------------------------------------------- launchers
cudaError_t launch_predict_hash(const LaunchCtx& c, const Tiles& old_tiles,
                                cudaStream_t st) {
  if (old_tiles.n == 0) return cudaSuccess;
  k_predict_hash<<<grid_for(old_tiles.n, c.block_misc, c.max_blocks), c.block_misc, 0, st>>>(
      old_tiles.d, old_tiles.n, c.scenes, c.pos, c.vel, c.count, c.keyrank);
  return cudaGetLastError();
}

cudaError_t launch_scan(const LaunchCtx& c, uint32_t len, cudaStream_t st) {
  const uint32_t nb = (len + kScanBlock - 1) / kScanBlock;
  if (nb == 0) return cudaSuccess;
  k_scan_reduce<<<nb, kScanThreads, 0, st>>>(c.count, len, c.partial);
  k_scan_partials<<<1, kScanThreads, 0, st>>>(c.partial, nb, c.start, len);
  k_scan_down<<<nb, kScanThreads, 0, st>>>(c.count, len, c.partial, c.start);
  return cudaGetLastError();
}

uint32_t scan_partials_needed(uint64_t len) {
  return static_cast<uint32_t>((len + kScanBlock - 1) / kScanBlock) + 1;
}

cudaError_t launch_sort_reorder(const LaunchCtx& c, const Tiles& old_tiles,
                                const Tiles& new_tiles, uint32_t total,
                                cudaStream_t st) {
  if (old_tiles.n) {
    k_scatter<<<grid_for(old_tiles.n, c.block_misc, c.max_blocks), c.block_misc, 0, st>>>(
        old_tiles.d, old_tiles.n, c.scenes, c.keyrank, c.start, c.pos, total,
        c.tmp, c.status);
  }
  if (new_tiles.n) {
    k_reorder<<<grid_for(new_tiles.n, c.block_misc, c.max_blocks), c.block_misc, 0, st>>>(
        new_tiles.d, new_tiles.n, c.scenes, c.tmp, c.start, c.pos, c.vel,
        c.pos2, c.vel2, c.pred, c.dbg_hash, c.dbg_key, c.src_limit, c.status);
  }
  return cudaGetLastError();
}

cudaError_t launch_density(const LaunchCtx& c, const Tiles& tiles,
                           cudaStream_t st) {
  if (tiles.n == 0) return cudaSuccess;
  const int b = c.block_nbr;
  k_density<<<grid_for(tiles.n, b, c.max_blocks), b, 0, st>>>(
      tiles.d, tiles.n, c.scenes, c.pred, c.start, c.dens_a, c.dens_b);
  return cudaGetLastError();
}

cudaError_t launch_pressure(const LaunchCtx& c, const Tiles& tiles,
                            cudaStream_t st) {
  if (tiles.n == 0) return cudaSuccess;
  const int b = c.block_nbr;
  k_pressure<<<grid_for(tiles.n, b, c.max_blocks), b, 0, st>>>(
      tiles.d, tiles.n, c.scenes, c.pred, c.start, c.dens_a, c.dens_b, c.vel2,
      c.velp, c.dbg_accp);
  return cudaGetLastError();
}

cudaError_t launch_visc_integrate(const LaunchCtx& c, const Tiles& tiles,
                                  int fuse_next, int write_out,
                                  cudaStream_t st) {
  if (tiles.n == 0) return cudaSuccess;
  const int b = c.block_nbr;
  k_visc_integrate<<<grid_for(tiles.n, b, c.max_blocks), b, 0, st>>>(
      tiles.d, tiles.n, c.scenes, c.pred, c.start, c.velp, c.pos2, c.vel2,
      write_out ? c.out4 : nullptr, fuse_next, c.count, c.keyrank, c.dbg_velv,
      c.status);
  return cudaGetLastError();
}

cudaError_t launch_export(uint32_t first, uint32_t n, const float4* pos,
                          const float4* vel, const float2* dens, float* opos,
                          float* ovel, float* odens, uint32_t* oids,
                          cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  k_export<<<(n + 255) / 256, 256, 0, st>>>(first, n, pos, vel, dens, opos,
                                            ovel, odens, oids);
  return cudaGetLastError();
}

cudaError_t launch_export_debug(uint32_t first, uint32_t n, const float4* pos,
                                const uint32_t* dhash, const uint32_t* dkey,
                                const float4* accp, const float4* velp,
                                const float4* velv, uint32_t* ohash,
                                uint32_t* okey, float* oaccp, float* ovelp,
                                float* ovelv, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  k_export_debug<<<(n + 255) / 256, 256, 0, st>>>(first, n, pos, dhash, dkey,
                                                  accp, velp, velv, ohash, okey,
                                                  oaccp, ovelp, ovelv);
  return cudaGetLastError();
}

cudaError_t launch_import(uint32_t first, uint32_t n, const float* ipos,
                          const float* ivel, float4* pos, float4* vel,
                          cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  k_import<<<(n + 255) / 256, 256, 0, st>>>(first, n, ipos, ivel, pos, vel);
  return cudaGetLastError();
}

}  // namespace sph
