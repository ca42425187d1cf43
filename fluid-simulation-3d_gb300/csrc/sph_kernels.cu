// SPH substep kernels for GB300 (sm_103a).
//
// One substep (engine/physics/physicsWorld.cc:39-111) is:
//   k_predict_hash   gravity + prediction + cell index + key, counting-sort
//                    histogram (warp-aggregated atomics)    :42-48, :473-482
//   k_scan_*         exclusive prefix of the key histogram = start table
//   k_scatter        bucket each particle at start[key] + arrival rank
//   k_reorder        deterministic order inside each bucket and gather of
//                    the state into SoA float4                :484-496
//   k_cell_table     per cell, its neighbour runs (the bucket walk of
//                    :331-346 resolved once per cell instead of per particle)
//   k_density        density / near density and neighbour lists :304-365
//   k_pressure       pressure + near pressure over the list   :367-422
//   k_visc_integrate Jacobi viscosity over the list, integrate, box
//                    collision, next substep's prediction    :424-464, :81-108
// and, when a substep is captured for export, k_ref_* rebuild the
// reference's own spatial lookup (HashCell keys, (key, index) order and
// startIndices, :466-496) from the same predicted positions.
//
// The sort key is the internal cell index (sph_device.cuh) modulo the scene
// size; inside a key bucket particles are ordered by (cell index, particle
// index), so every cell is a contiguous run of slots and the three cells of
// an x-row usually one run. Every kernel is a persistent, segmented launch:
// warps stride over a tile table of (scene, first slot) runs of up to 32
// particles of one scene, so one launch serves any number of scenes of
// uneven sizes.
#include "sph_kernels.h"

namespace sph {

namespace {

constexpr uint32_t kFull = 0xffffffffu;

__device__ __forceinline__ uint32_t warp_id_global() {
  return blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
}
__device__ __forceinline__ uint32_t warps_total() {
  return gridDim.x * (blockDim.x >> 5);
}
__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31; }

// glm dot(v, v) of physicsWorld.cc:355: three rounded products summed left to
// right (no FMA contraction), so boundary pairs classify as in the reference.
__device__ __forceinline__ float dist2(float dx, float dy, float dz) {
  return __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)),
                   __fmul_rn(dz, dz));
}
// Fast estimate of the same value (within a few ulp of dist2).
__device__ __forceinline__ float dist2_fast(float dx, float dy, float dz) {
  return fmaf(dz, dz, fmaf(dy, dy, dx * dx));
}
// Hardware square root estimate (sqrt.approx.f32: 0 -> 0).
__device__ __forceinline__ float sqrt_approx(float x) {
  float y;
  asm("sqrt.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__device__ __forceinline__ void flag(uint32_t* status, uint32_t f) {
  atomicOr(status, f);
}

// Programmatic dependent launch: the substep kernels are launched with
// programmatic stream serialisation (launch_pdl), so each one is scheduled
// while its predecessor's last wave runs. Every such kernel starts here: it
// lets its own successor be scheduled, then waits for its predecessor to
// complete with its memory visible (a hardware dependency, not a spin), so
// nothing is read early. Without the launch attribute both are no-ops.
__device__ __forceinline__ void pdl_enter() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
}

// Entry k of slot i's neighbour list, k-major (entry k of all slots, then
// entry k + 1), so a warp's appends and loads of one entry are contiguous.
// 64-bit: k * stride passes 2^32 for capacities above 2^26.
__device__ __forceinline__ uint64_t nbr_index(uint32_t i, uint32_t k,
                                              uint32_t stride) {
  return static_cast<uint64_t>(k) * stride + i;
}

// 32-byte particle records (rec_v): two float4 halves that a neighbour
// gather fetches with one 256-bit load from one sector.
__device__ __forceinline__ void load_rec(const float4* __restrict__ rec,
                                         uint32_t j, float4& a, float4& b) {
  asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
      : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y),
        "=f"(b.z), "=f"(b.w)
      : "l"(rec + 2ull * j));
}
__device__ __forceinline__ void store_rec(float4* __restrict__ rec, uint32_t i,
                                          float4 a, float4 b) {
  asm volatile("st.global.v8.f32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};"
               :
               : "l"(rec + 2ull * i), "f"(a.x), "f"(a.y), "f"(a.z), "f"(a.w),
                 "f"(b.x), "f"(b.y), "f"(b.z), "f"(b.w)
               : "memory");
}

// kGather consecutive entries of slot i's list from entry k0, those below
// cnt (<= the list capacity) only: a batch of 3 that starts near the end of
// a full list would otherwise read past the list rows. Each entry is read
// once per pass, so the loads carry the streaming (evict-first) hint and
// leave the cache to the neighbours' gathered state.
// With kStep = 2 (two lanes per particle) a lane reads every other entry:
// k0, k0 + 2, ...
template <int kGather, int kStep = 1>
__device__ __forceinline__ void load_nbr_batch(const uint32_t* __restrict__ nbr,
                                               uint32_t i, uint32_t k0,
                                               uint32_t stride, uint32_t cnt,
                                               uint32_t (&j)[kGather]) {
  const uint32_t* p = nbr + nbr_index(i, k0, stride);
#pragma unroll
  for (int u = 0; u < kGather; ++u)
    j[u] = k0 + kStep * u < cnt ? __ldcs(p + static_cast<uint64_t>(kStep * u) * stride) : 0u;
}

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t x) {
  const uint32_t lane = lane_id();
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t y = __shfl_up_sync(kFull, x, d);
    if (lane >= static_cast<uint32_t>(d)) x += y;
  }
  return x;
}

// Rank among the lanes of the warp that share `key`, and one atomicAdd per
// distinct key (particles stored in the previous sorted order share cells
// with their warp neighbours). All 32 lanes must call; inactive lanes pass
// active = false and get 0.
__device__ __forceinline__ uint32_t aggregated_rank(uint32_t* count,
                                                    uint32_t key,
                                                    bool active) {
  const uint32_t am = __ballot_sync(kFull, active);
  if (!active) return 0u;
  const uint32_t lane = lane_id();
  const uint32_t peers = __match_any_sync(am, key);
  const int leader = __ffs(peers) - 1;
  uint32_t base = 0;
  if (static_cast<int>(lane) == leader) base = atomicAdd(count + key, __popc(peers));
  base = __shfl_sync(peers, base, leader);
  return base + __popc(peers & ((1u << lane) - 1u));
}

// Row w (dy = w/3 - 1, dz = w%3 - 1) of a cell of a direct key table: its
// three x-neighbour cells are consecutive table entries, so the row is one
// run from two start-table reads. k0 = tbase + cell - gwy - gwz, the entry of
// row 0's middle cell.
__device__ __forceinline__ uint2 direct_row(const SceneDev& S,
                                            const uint32_t* __restrict__ start,
                                            uint32_t k0, int w) {
  const uint32_t k = k0 + static_cast<uint32_t>(w / 3) * S.gwy +
                     static_cast<uint32_t>(w % 3) * S.gwz;
  const uint32_t f = __ldg(start + k - 1);
  return make_uint2(f, (__ldg(start + k + 2) - f) | kRunMerged);
}

// Neighbour walk of a particle: the particles of its cell's 27 neighbour
// cells -- every candidate the reference's bucket loops would accept within
// the cutoff -- row by row, a merged row as one run. A direct key table
// gives each row from the start table (cell = the particle's cell index);
// otherwise the rows come from the cell's table built by k_cell_table (cf =
// the cell's first slot). Both visit the same particles in the same order.
template <int kTables, class F>
__device__ __forceinline__ void walk_runs(const SceneDev& S,
                                          const uint32_t* __restrict__ start,
                                          const uint2* __restrict__ cell_tab,
                                          uint32_t cf, uint32_t cell,
                                          const float4* __restrict__ pred,
                                          F&& visit) {
  const bool direct = kTables == kTablesDirect    ? true
                    : kTables == kTablesBuckets ? false
                                                : S.direct != 0u;
  if (direct) {
    // rows (dy, dz) in the cell table's order (dz fastest); k = the row's
    // middle cell
    uint32_t k = S.tbase + cell - S.gwy - S.gwz;
    int dz = 0;
#pragma unroll 1
    for (int w = 0; w < 9; ++w) {
      const uint32_t e = __ldg(start + k + 2);
#pragma unroll 1
      for (uint32_t j = __ldg(start + k - 1); j < e; ++j) visit(j, __ldg(pred + j));
      if (++dz == 3) { dz = 0; k += S.gwy - 2u * S.gwz; } else { k += S.gwz; }
    }
    return;
  }
  const uint2* row = cell_tab + static_cast<uint64_t>(cf) * 27u;
#pragma unroll 1
  for (int w = 0; w < 9; ++w, row += 3) {
    const uint2 m = __ldg(row);
    if (m.y & kRunMerged) {
      const uint32_t e = m.x + (m.y & ~kRunMerged);
#pragma unroll 1
      for (uint32_t j = m.x; j < e; ++j) visit(j, __ldg(pred + j));
    } else {
#pragma unroll 1
      for (int k = 0; k < 3; ++k) {
        const uint2 run = k ? __ldg(row + k) : m;
#pragma unroll 1
        for (uint32_t j = run.x; j < run.x + run.y; ++j) visit(j, __ldg(pred + j));
      }
    }
  }
}

// ----------------------------------------------------------------- predict
__device__ __forceinline__ void predict_key(const SceneDev& S, float4 p,
                                            float4 v, uint32_t& key,
                                            uint32_t& cell) {
  float3 vn, pr;
  predict(S, p, v, vn, pr);
  cell = cell_index(S, pr);
  key = table_key(S, cell);
}

__global__ void k_predict_hash(const uint2* __restrict__ tiles, uint32_t ntiles,
                               const SceneDev* __restrict__ scenes,
                               const float4* __restrict__ pos,
                               const float4* __restrict__ vel,
                               uint32_t* __restrict__ count,
                               uint4* __restrict__ keyrank) {
  pdl_enter();
  const uint32_t lane = lane_id();
  for (uint32_t t = warp_id_global(); t < ntiles; t += warps_total()) {
    const uint2 tile = tiles[t];
    const SceneDev S = scenes[tile_scene(tile)];  // registers, not reloads
    const uint32_t s = tile.y + lane;
    const bool live = lane < tile_len(tile);
    uint32_t key = 0, cell = 0, id = 0;
    if (live) {
      const float4 p = pos[s];
      predict_key(S, p, vel[s], key, cell);
      id = __float_as_uint(p.w);
    }
    const uint32_t r = aggregated_rank(count, key, live);
    if (live) keyrank[s] = make_uint4(key, r, cell, id);
  }
}

// -------------------------------------------------------------------- scan
constexpr int kScanThreads = 512;
constexpr int kScanItems = 4;
constexpr int kScanBlock = kScanThreads * kScanItems;
constexpr uint32_t kScanFoldBlocks = 4096;  // fold the partials scan up to here

// Block-wide exclusive scan of one value per thread; returns the block total
// through *total.
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t x,
                                                    uint32_t* total) {
  __shared__ uint32_t warp_sums[32];
  const uint32_t lane = lane_id(), w = threadIdx.x >> 5;
  const uint32_t incl = warp_incl_scan(x);
  if (lane == 31) warp_sums[w] = incl;
  __syncthreads();
  if (w == 0) {
    const uint32_t nw = blockDim.x >> 5;
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

// The kScanItems (= 4) consecutive counts of a thread: one 16-byte load
// inside the table, element loads at its ragged end.
__device__ __forceinline__ uint4 load_counts(const uint32_t* __restrict__ count, uint32_t b0,
                                             uint32_t len) {
  if (b0 + 4u <= len) return *reinterpret_cast<const uint4*>(count + b0);
  uint4 v = make_uint4(0u, 0u, 0u, 0u);
  if (b0 < len) v.x = count[b0];
  if (b0 + 1u < len) v.y = count[b0 + 1u];
  if (b0 + 2u < len) v.z = count[b0 + 2u];
  return v;
}

__global__ void __launch_bounds__(kScanThreads)
k_scan_reduce(const uint32_t* __restrict__ count, uint32_t len,
              uint32_t* __restrict__ partial) {
  static_assert(kScanItems == 4, "one uint4 of counts per thread");
  pdl_enter();
  const uint32_t b0 = blockIdx.x * kScanBlock + threadIdx.x * kScanItems;
  const uint4 v = load_counts(count, b0, len);
  uint32_t total;
  block_excl_scan(v.x + v.y + v.z + v.w, &total);
  if (threadIdx.x == 0) partial[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kScanThreads)
k_scan_partials(uint32_t* __restrict__ partial, uint32_t nb,
                uint32_t* __restrict__ start, uint32_t len) {
  pdl_enter();
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

// Down-sweep. With `fold` the block totals in `partial` are raw (no
// k_scan_partials): each block sums the totals before it itself -- O(nb^2)
// reads in all, so the launcher folds only up to kScanFoldBlocks blocks --
// and the last block writes the grand total start[len]. The block's own
// counts are loaded first, so their latency overlaps the fold's reads, and
// one block pass both scans the counts and sums the fold.
__global__ void __launch_bounds__(kScanThreads)
k_scan_down(uint32_t* __restrict__ count, uint32_t len,
            const uint32_t* __restrict__ partial, uint32_t nb, int fold,
            uint32_t* __restrict__ start) {
  __shared__ uint32_t warp_scan[kScanThreads / 32], warp_fold[kScanThreads / 32];
  pdl_enter();
  const uint32_t b0 = blockIdx.x * kScanBlock + threadIdx.x * kScanItems;
  const uint4 v = load_counts(count, b0, len);
  uint32_t f = 0;
  if (fold) {
    for (uint32_t c = threadIdx.x; c < blockIdx.x; c += kScanThreads) f += partial[c];
  }
  const uint32_t s = v.x + v.y + v.z + v.w;
  const uint32_t lane = lane_id(), w = threadIdx.x >> 5;
  const uint32_t incl = warp_incl_scan(s);
#pragma unroll
  for (int d = 16; d >= 1; d >>= 1) f += __shfl_xor_sync(kFull, f, d);
  if (lane == 31) warp_scan[w] = incl;
  if (lane == 0) warp_fold[w] = f;
  __syncthreads();
  constexpr uint32_t kWarps = kScanThreads / 32;
  uint32_t before = 0, block_total = 0, base = 0;
#pragma unroll
  for (uint32_t u = 0; u < kWarps; ++u) {  // smem broadcasts: every lane reads the same word
    const uint32_t ws = warp_scan[u];
    before += u < w ? ws : 0u;
    block_total += ws;
    base += warp_fold[u];
  }
  if (!fold) base = partial[blockIdx.x];
  uint32_t run = base + before + incl - s;
  if (b0 + 4u <= len) {
    uint4 o;
    o.x = run;
    o.y = o.x + v.x;
    o.z = o.y + v.y;
    o.w = o.z + v.z;
    *reinterpret_cast<uint4*>(start + b0) = o;
    *reinterpret_cast<uint4*>(count + b0) = make_uint4(0u, 0u, 0u, 0u);  // next histogram
  } else {
    const uint32_t vv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
      if (b0 + k < len) {
        start[b0 + k] = run;
        count[b0 + k] = 0u;
      }
      run += vv[k];
    }
  }
  if (fold && blockIdx.x + 1 == nb && threadIdx.x == 0) start[len] = base + block_total;
}

// ----------------------------------------------------------------- scatter
__global__ void k_scatter(const uint2* __restrict__ tiles, uint32_t ntiles,
                          const uint4* __restrict__ keyrank,
                          const uint32_t* __restrict__ start, uint32_t total,
                          uint2* __restrict__ tmp_hi,
                          uint32_t* __restrict__ tmp_src, uint32_t* status) {
  pdl_enter();
  const uint32_t lane = lane_id();
  for (uint32_t t = warp_id_global(); t < ntiles; t += warps_total()) {
    const uint2 tile = tiles[t];
    const uint32_t s = tile.y + lane;
    if (lane >= tile_len(tile)) continue;
    const uint4 kr = keyrank[s];
    const uint32_t dst = start[kr.x] + kr.y;
    if (dst >= total) { flag(status, kStatusRange); continue; }
    tmp_hi[dst] = make_uint2(kr.z, kr.w);
    tmp_src[dst] = s;
  }
}

// ----------------------------------------------------------------- reorder
// Thread per bucketed slot: rank the particle inside its bucket by
// (cell index, particle index), recompute its gravity/prediction exactly as
// k_predict_hash did, and write the state to its final slot, plus the first
// slot of its cell (its run of equal cell index).
__global__ void k_reorder(const uint2* __restrict__ tiles, uint32_t ntiles,
                          const SceneDev* __restrict__ scenes,
                          const uint2* __restrict__ tmp_hi,
                          const uint32_t* __restrict__ tmp_src,
                          const uint32_t* __restrict__ start,
                          const float4* __restrict__ pos_in,
                          const float4* __restrict__ vel_in,
                          float4* __restrict__ pos_out,
                          float4* __restrict__ vel_out,
                          float4* __restrict__ pred,
                          uint32_t* __restrict__ hash_s,
                          uint32_t* __restrict__ cell_first,
                          uint32_t src_limit, uint32_t* status) {
  pdl_enter();
  const uint32_t lane = lane_id();
  for (uint32_t t = warp_id_global(); t < ntiles; t += warps_total()) {
    const uint2 tile = tiles[t];
    const SceneDev S = scenes[tile_scene(tile)];  // registers, not reloads
    const uint32_t slot = tile.y + lane;
    if (lane >= tile_len(tile)) continue;
    const uint2 me = tmp_hi[slot];
    const uint32_t src = tmp_src[slot];
    if (src >= src_limit) { flag(status, kStatusRange); continue; }
    const float4 p = pos_in[src];
    const float4 v = vel_in[src];
    float3 vn, pr;
    predict(S, p, v, vn, pr);
    // the cell index travelled with the entry: k_predict_hash (or the fused
    // prediction) computed it from this same prediction
    const uint32_t cell = me.x;
    const uint32_t key = table_key(S, cell);
    const uint32_t b0 = start[key], b1 = start[key + 1];
    if (slot < b0 || slot >= b1) {
      flag(status, kStatusRange);
      continue;
    }
    uint32_t rank = 0, below = 0;
    for (uint32_t u = b0; u < b1; ++u) {
      const uint2 o = tmp_hi[u];
      below += (o.x < me.x) ? 1u : 0u;
      rank += (o.x < me.x || (o.x == me.x && o.y < me.y)) ? 1u : 0u;
    }
    const uint32_t f = b0 + rank;
    pos_out[f] = p;
    vel_out[f] = make_float4(vn.x, vn.y, vn.z, 0.0f);
    pred[f] = make_float4(pr.x, pr.y, pr.z, __uint_as_float(cell));
    hash_s[f] = cell;
    cell_first[f] = b0 + below;
  }
}

// -------------------------------------------------------------- cell table
// The run of cell index `cell` in its key bucket [b0, b1). A bucket is
// sorted by cell index, so the cell's particles are one run and entries of
// other cells that share the bucket are left out, as the reference's
// float(hash) test leaves them out (:346); a bucket holding a single cell is
// the common case and is recognised from its first and last entries.
__device__ __forceinline__ uint2 bucket_run(uint32_t cell, uint32_t b0,
                                            uint32_t b1,
                                            const uint32_t* __restrict__ hash_s) {
  uint32_t first = b0, len = 0;
  if (b1 > b0) {
    const uint32_t h0 = __ldg(hash_s + b0), h1 = __ldg(hash_s + b1 - 1);
    if (h0 == cell && h1 == cell) {
      len = b1 - b0;
    } else if (h0 <= cell && cell <= h1) {
      for (uint32_t u = b0; u < b1; ++u) {
        const bool eq = __ldg(hash_s + u) == cell;
        if (eq && len == 0) first = u;
        len += eq ? 1u : 0u;
      }
    }
  }
  return make_uint2(first, len);
}

// For each cell (its first slot) of a scene with a bucket key table, the
// runs of its 27 neighbour cells as 9 rows (dy, dz) of three x-runs. The
// x-neighbours of a row have consecutive cell indices, hence consecutive
// keys; when their runs are adjacent in the layout (their buckets hold no
// other cell -- the usual case inside the box) the row is stored as one run
// flagged kRunMerged in its first entry (its other two entries are left
// unwritten: a third of the table's stores, which the readers skip). Lanes take (cell, row)
// pairs of the warp's tile in parallel; the warp's cell leaders are listed
// in shared memory (kCellTableBlock threads per block).
constexpr int kCellTableBlock = 256;

__global__ void __launch_bounds__(kCellTableBlock)
k_cell_table(const uint2* __restrict__ tiles, uint32_t ntiles,
             const SceneDev* __restrict__ scenes,
             const uint32_t* __restrict__ hash_s,
             const uint32_t* __restrict__ cell_first,
             const uint32_t* __restrict__ start, uint2* __restrict__ cell_tab) {
  pdl_enter();
  __shared__ uint8_t s_lead[kCellTableBlock / 32][32];
  uint8_t* lead = s_lead[threadIdx.x >> 5];
  const uint32_t lane = lane_id();
  for (uint32_t t = warp_id_global(); t < ntiles; t += warps_total()) {
    const uint2 tile = tiles[t];
    const SceneDev S = scenes[tile_scene(tile)];  // registers, not reloads
    if (S.direct) continue;  // its rows come from the start table
    const uint32_t i = tile.y + lane;
    const bool live = lane < tile_len(tile);
    const bool leader = live && cell_first[i] == i;
    const uint32_t lmask = __ballot_sync(kFull, leader);
    if (leader) lead[__popc(lmask & ((1u << lane) - 1u))] = static_cast<uint8_t>(lane);
    __syncwarp();
    const uint32_t pairs = __popc(lmask) * 9u;
    const uint32_t kmax = fastmod(0xffffffffu, S.fm, S.n);  // key of 2^32 - 1
    for (uint32_t q = lane; q < pairs; q += 32) {
      const uint32_t c = q / 9u, w = q - c * 9u;
      const uint32_t slot = tile.y + lead[c];
      const uint32_t dy = w / 3u - 1u, dz = w % 3u - 1u;  // mod 2^32
      const uint32_t mid = __ldg(hash_s + slot) + dy * S.gwy + dz * S.gwz;
      uint2* out = cell_tab + static_cast<uint64_t>(slot) * 27u + 3u * w;
      // keys of mid - 1, mid, mid + 1: neighbours of mid's key modulo n,
      // except across the 2^32 wrap of the index
      const uint32_t km = fastmod(mid, S.fm, S.n);
      const uint32_t kl = mid == 0u ? kmax : (km == 0u ? S.n - 1u : km - 1u);
      const uint32_t kh = mid == 0xffffffffu ? 0u : (km + 1u == S.n ? 0u : km + 1u);
      const uint32_t* st = start + S.tbase;
      const uint32_t l0 = __ldg(st + kl), l1 = __ldg(st + kl + 1);
      const uint32_t m0 = kl + 1u == km ? l1 : __ldg(st + km);
      const uint32_t m1 = __ldg(st + km + 1);
      const uint32_t h0 = kh == km + 1u ? m1 : __ldg(st + kh);
      const uint32_t h1 = __ldg(st + kh + 1);
      uint2 run[3];
      run[0] = bucket_run(mid - 1u, l0, l1, hash_s);
      run[1] = bucket_run(mid, m0, m1, hash_s);
      run[2] = bucket_run(mid + 1u, h0, h1, hash_s);
      uint32_t f = 0, e = 0;
      bool any = false, adjacent = true;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        if (run[k].y == 0) continue;
        if (!any) {
          f = run[k].x;
          e = f + run[k].y;
          any = true;
        } else if (run[k].x == e) {
          e += run[k].y;
        } else {
          adjacent = false;
        }
      }
      if (adjacent) {
        out[0] = make_uint2(f, (e - f) | kRunMerged);
      } else {
        out[0] = run[0];
        out[1] = run[1];
        out[2] = run[2];
      }
    }
    __syncwarp();  // the next tile rewrites the leader list
  }
}

// ----------------------------------------------------------------- density
// CalculateDensity (:325-365) for one particle (self included) and its
// neighbour list (dist <= r, self excluded) for the force passes, in two
// phases. Phase 1 walks the cell's runs with the FMA estimate of d2 and only
// appends candidates within cut_hi (a 2e-6 superset of the cutoff) to the
// list. Phase 2 re-reads the ~25 listed pairs, classifies each on the
// reference's exact d2 (dropping the rare band pairs) and accumulates the
// kernels; contributions vanish at the cutoff ((r-dist)^2), so the hardware
// square root serves the kernel value. The self pair contributes (r, r).
__device__ __forceinline__ void density_pair(const SceneDev& S, float d2,
                                             float& s2, float& s3) {
  const float w = S.r - sqrt_approx(d2);
  const float w2 = w * w;
  s2 += w2;
  s3 = fmaf(w2, w, s3);
}

__device__ __forceinline__ void density_store(const SceneDev& S, uint32_t i,
                                              float s2, float s3, uint32_t cnt,
                                              float2* __restrict__ dens_a,
                                              float4* __restrict__ dens_b,
                                              uint32_t* __restrict__ ncount) {
  const float rho = s2 * S.vol2, rhon = s3 * S.vol3;
  dens_a[i] = make_float2(rho, rhon);
  const float ir = 1.0f / rho, irn = 1.0f / rhon;
  const float P = (rho - S.rho0) * S.k, Pn = rhon * S.kn;
  dens_b[i] = make_float4(ir, P * ir, irn, Pn * irn);
  ncount[i] = cnt;
}

// Thread-per-particle form in one pass: each lane walks its cell's runs,
// classifies every candidate on the reference's exact d2 and accumulates the
// density and its list as it goes. Lanes of one cell walk identical runs, so
// their loads coincide. The walk is issue-bound: the cutoff and radius sit
// in registers for the whole walk, and the hit path is one short predicated
// block, at 32 registers (64 warps per SM; 40 measured slower).
template <int kTables>
__global__ void __maxnreg__(32) k_density_walk(const uint2* __restrict__ tiles,
                               uint32_t ntiles,
                               const SceneDev* __restrict__ scenes,
                               const float4* __restrict__ pred,
                               const uint32_t* __restrict__ start,
                               const uint32_t* __restrict__ cell_first,
                               const uint2* __restrict__ cell_tab,
                               float2* __restrict__ dens_a,
                               float4* __restrict__ dens_b,
                               uint32_t* __restrict__ nbr,
                               uint32_t* __restrict__ ncount,
                               uint32_t nbr_stride, uint32_t nbr_cap) {
  pdl_enter();
  const uint32_t lane = lane_id();
  for (uint32_t t = warp_id_global(); t < ntiles; t += warps_total()) {
    const uint2 tile = tiles[t];
    const SceneDev& S = scenes[tile_scene(tile)];
    if (lane >= tile_len(tile)) continue;
    const uint32_t i = tile.y + lane;
    const float4 me = pred[i];
    const float3 p = make_float3(me.x, me.y, me.z);
    float s2 = S.r2, s3 = S.r2 * S.r;  // self: w = r
    uint32_t cnt = 0;
    uint32_t* wp = nbr + i;  // next list entry (a bumped pointer is the
                             // cheapest append in the hit path)
    // Pairs with dist <= r (d2 <= cut_le) enter the list; the density takes
    // (r - dist)^2 and (r - dist)^3 of the same pairs: those with dist == r
    // exactly, which the reference leaves out, add (r - sqrt(d2))^2, the
    // square of a rounding error.
    const float cut = S.cut_le, r = S.r;
    const uint32_t cf = kTables == kTablesDirect ? 0u : cell_first[i];
    const float2 npxy = make_float2(-p.x, -p.y);
    walk_runs<kTables>(S, start, cell_tab, cf, __float_as_uint(me.w), pred, [&](uint32_t j, float4 q) {
      // dist2 with (dx, dy) as one packed FP32x2 pair (x and y are adjacent
      // in the record): every component rounded as the scalar code rounds
      // it, two instructions fewer per candidate
      const float2 dxy = __fadd2_rn(make_float2(q.x, q.y), npxy);
      const float2 sxy = __fmul2_rn(dxy, dxy);
      const float dz = q.z - p.z;
      const float d2 = __fadd_rn(__fadd_rn(sxy.x, sxy.y), __fmul_rn(dz, dz));
      if (d2 <= cut && j != i) {
        if (cnt < nbr_cap) {
          *wp = j;
          wp += nbr_stride;
        }
        ++cnt;
        const float w = r - sqrt_approx(d2);
        const float w2 = w * w;
        s2 += w2;
        s3 = fmaf(w2, w, s3);
      }
    });
    density_store(S, i, s2, s3, cnt, dens_a, dens_b, ncount);
  }
}

// Phase 1 is warp-cooperative over the cells of the warp's 32 slots: for
// each cell, lanes 0..26 fetch its 27 runs, a warp scan gives their offsets
// in the cell's flat candidate sequence, and each lane holds kChunks of those
// candidates in registers (its slot found by a shuffle binary search over
// the run offsets) -- a cell tile of kChunks*32 candidates. Every particle of
// the cell is then tested against the whole tile at once: one ballot per 32
// pairs appends the hits to that particle's list. Longer candidate sequences
// are processed tile by tile.
template <int kChunks>
__global__ void k_density(const uint2* __restrict__ tiles, uint32_t ntiles,
                          const SceneDev* __restrict__ scenes,
                          const float4* __restrict__ pred,
                          const uint32_t* __restrict__ start,
                          const uint32_t* __restrict__ cell_first,
                          const uint2* __restrict__ cell_tab,
                          float2* __restrict__ dens_a,
                          float4* __restrict__ dens_b,
                          uint32_t* __restrict__ nbr,
                          uint32_t* __restrict__ ncount, uint32_t nbr_stride,
                          uint32_t nbr_cap) {
  pdl_enter();
  const uint32_t lane = lane_id();
  const uint32_t lt_mask = (1u << lane) - 1u;
  for (uint32_t t = warp_id_global(); t < ntiles; t += warps_total()) {
    const uint2 tile = tiles[t];
    const SceneDev S = scenes[tile_scene(tile)];  // registers, not reloads
    const uint32_t i = tile.y + lane;
    const bool live = lane < tile_len(tile);
    const float4 me = live ? pred[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    const uint32_t cf = live ? cell_first[i] : 0xffffffffu;
    const uint32_t cf_prev = __shfl_up_sync(kFull, cf, 1);
    const uint32_t lead = __ballot_sync(kFull, live && (lane == 0 || cf != cf_prev));
    const uint32_t live_end = tile_len(tile);
    // phase 1: candidate lists (FMA estimate of d2 within cut_hi)
    uint32_t cnt = 0;  // list length of this lane's particle
    for (uint32_t cells = lead; cells != 0;) {
      const int c0 = __ffs(cells) - 1;
      cells &= cells - 1;
      const int c1 = cells ? __ffs(cells) - 1 : static_cast<int>(live_end);
      const uint32_t cfc = __shfl_sync(kFull, cf, c0);
      const uint32_t cellc = __shfl_sync(kFull, __float_as_uint(me.w), c0);
      uint2 run = make_uint2(0u, 0u);
      if (S.direct) {
        if (lane < 27u && lane % 3u == 0u)
          run = direct_row(S, start, S.tbase + cellc - S.gwy - S.gwz, static_cast<int>(lane / 3u));
      } else if (lane < 27) {
        run = __ldg(cell_tab + static_cast<uint64_t>(cfc) * 27u + lane);
      }
      // a merged row keeps its run in its first entry; the other two are unused
      const uint32_t heads =
          __ballot_sync(kFull, lane < 27u && lane % 3u == 0u && (run.y & kRunMerged));
      if (lane < 27u && lane % 3u != 0u && ((heads >> (lane - lane % 3u)) & 1u)) run.y = 0u;
      run.y &= ~kRunMerged;
      const uint32_t incl = warp_incl_scan(run.y);
      const uint32_t excl = incl - run.y;
      const uint32_t total = __shfl_sync(kFull, incl, 31);
      for (uint32_t seg = 0; seg < total; seg += kChunks * 32u) {
        float4 q[kChunks];
        uint32_t js[kChunks];
#pragma unroll
        for (int c = 0; c < kChunks; ++c) {
          const uint32_t e = seg + c * 32u + lane;
          // o = number of runs ending at or before e (incl is ascending)
          uint32_t o = 0;
#pragma unroll
          for (uint32_t step = 16; step >= 1; step >>= 1) {
            const uint32_t probe = o + step - 1u;
            const uint32_t v = __shfl_sync(kFull, incl, probe < 27u ? probe : 26u);
            if (probe < 27u && v <= e) o += step;
          }
          const uint32_t src = o < 27u ? o : 26u;
          const uint32_t rx = __shfl_sync(kFull, run.x, src);
          const uint32_t rex = __shfl_sync(kFull, excl, src);
          js[c] = rx + (e - rex);
          q[c] = e < total ? __ldg(pred + js[c])
                           : make_float4(__int_as_float(0x7f800000), 0.f, 0.f, 0.f);
        }
        for (int pp = c0; pp < c1; ++pp) {
          const float px = __shfl_sync(kFull, me.x, pp);
          const float py = __shfl_sync(kFull, me.y, pp);
          const float pz = __shfl_sync(kFull, me.z, pp);
          const uint32_t ip = tile.y + static_cast<uint32_t>(pp);
          uint32_t base = __shfl_sync(kFull, cnt, pp);
#pragma unroll
          for (int c = 0; c < kChunks; ++c) {
            if (seg + c * 32u >= total) break;
            const float d2f = dist2_fast(q[c].x - px, q[c].y - py, q[c].z - pz);
            const bool hit = d2f <= S.cut_hi && js[c] != ip;
            const uint32_t hm = __ballot_sync(kFull, hit);
            if (hit) {
              const uint32_t k = base + __popc(hm & lt_mask);
              if (k < nbr_cap) nbr[nbr_index(ip, k, nbr_stride)] = js[c];
            }
            base += __popc(hm);
          }
          if (lane == static_cast<uint32_t>(pp)) cnt = base;
        }
      }
    }
    if (!live) continue;
    const float3 p = make_float3(me.x, me.y, me.z);
    // phase 2: exact classification and the density sums
    float s2 = S.r2, s3 = S.r2 * S.r;  // self: w = r
    if (cnt <= nbr_cap) {
      uint32_t kept = 0;
      for (uint32_t k = 0; k < cnt; ++k) {
        const uint32_t j = nbr[nbr_index(i, k, nbr_stride)];
        const float4 q = __ldg(pred + j);
        const float d2 = dist2(q.x - p.x, q.y - p.y, q.z - p.z);
        if (d2 <= S.cut_lt) density_pair(S, d2, s2, s3);
        if (d2 <= S.cut_le) {
          if (kept != k) nbr[nbr_index(i, kept, nbr_stride)] = j;
          ++kept;
        }
      }
      cnt = kept;
    } else {
      // list overflow: sum directly; the force passes walk the runs too
      walk_runs<kTablesMixed>(S, start, cell_tab, cf, __float_as_uint(me.w), pred,
                              [&](uint32_t j, float4 q) {
        const float d2 = dist2(q.x - p.x, q.y - p.y, q.z - p.z);
        if (j != i && d2 <= S.cut_lt) density_pair(S, d2, s2, s3);
      });
    }
    density_store(S, i, s2, s3, cnt, dens_a, dens_b, ncount);
  }
}

// ---------------------------------------------------------------- pressure
// CalculatePressureForce (:367-422) over the particle's neighbour list (self
// excluded, dist <= r). shared/rho_j = 0.5*(Pi*(1/rho_j) + Pj/rho_j); the 0.5
// is folded into ds2h/ds3h. The list is read kGather (2, 3, 4 or 8, tuned)
// entries at a time so their neighbours' gathers are in flight together, the
// next batch's entries loading meanwhile. A list that overflowed
// falls back to the walk of the cell's runs.
__device__ __forceinline__ void pressure_pair(const SceneDev& S, float3 p,
                                              float Pi, float Pni, float4 q,
                                              float4 b, float3& f) {
  const float dx = q.x - p.x, dy = q.y - p.y, dz = q.z - p.z;
  const float d2 = dist2(dx, dy, dz);
  const float dist = __fsqrt_rn(d2);
  const float w = S.r - dist;
  const float a2 = S.ds2h * fmaf(Pi, b.x, b.y);
  const float a3 = S.ds3h * w * fmaf(Pni, b.z, b.w);
  const float tsum = -w * (a2 + a3);
  if (d2 > 0.0f) {
    const float s = tsum * rsqrtf(d2);
    f.x = fmaf(dx, s, f.x);
    f.y = fmaf(dy, s, f.y);
    f.z = fmaf(dz, s, f.z);
  } else {
    f.y += tsum;  // dir = (0,1,0) for coincident particles (:414)
  }
}



// kLanes lanes per particle (tuning.particles_per_warp = 32 / kLanes): a
// warp takes its tile's 32 particles in kLanes passes of 32 / kLanes; lane
// pair (l, l + 16) shares a particle, each summing every other list entry,
// and one shuffle combines the halves. The sums then run in another order
// than with one lane, so the two forms agree to rounding, not bit for bit.
template <int kGather, int kTables, int kLanes>
__global__ void k_pressure(const uint2* __restrict__ tiles, uint32_t ntiles,
                           const SceneDev* __restrict__ scenes,
                           const float4* __restrict__ pred,
                           const uint32_t* __restrict__ start,
                           const uint32_t* __restrict__ cell_first,
                           const uint2* __restrict__ cell_tab,
                           const float2* __restrict__ dens_a,
                           const float4* __restrict__ dens_b,
                           const uint32_t* __restrict__ nbr,
                           const uint32_t* __restrict__ ncount,
                           uint32_t nbr_stride, uint32_t nbr_cap,
                           const float4* __restrict__ vel,
                           float4* __restrict__ rec_v,
                           float4* __restrict__ dbg_accp) {
  static_assert(kLanes == 1 || kLanes == 2, "one or two lanes per particle");
  pdl_enter();
  const uint32_t lane = lane_id();
  constexpr uint32_t kPer = 32 / kLanes;  // particles per pass
  const uint32_t sub = lane / kPer;       // this lane's share of the list
  for (uint32_t t = warp_id_global(); t < ntiles; t += warps_total()) {
    const uint2 tile = tiles[t];
    const SceneDev S = scenes[tile_scene(tile)];  // registers, not reloads
#pragma unroll 1
    for (uint32_t h = 0; h < kLanes; ++h) {
      const uint32_t li = h * kPer + lane % kPer;
      if (kLanes == 1 && li >= tile_len(tile)) break;
      const bool live = li < tile_len(tile);
      const uint32_t i = tile.y + (live ? li : 0u);
      const float4 pi = pred[i];
      const float3 p = make_float3(pi.x, pi.y, pi.z);
      const float2 di = dens_a[i];
      const float Pi = (di.x - S.rho0) * S.k, Pni = di.y * S.kn;
      float3 f = make_float3(0.0f, 0.0f, 0.0f);
      const uint32_t cnt = live ? ncount[i] : 0u;
      if (cnt <= nbr_cap) {
        uint32_t jn[kGather];
        if (sub < cnt) load_nbr_batch<kGather, kLanes>(nbr, i, sub, nbr_stride, cnt, jn);
        for (uint32_t k0 = sub; k0 < cnt; k0 += kLanes * kGather) {
          uint32_t j[kGather];
          float4 q[kGather], b[kGather];
#pragma unroll
          for (int u = 0; u < kGather; ++u) j[u] = (k0 + kLanes * u < cnt) ? jn[u] : i;
          // the next batch's entries load while this batch's gathers fly
          if (k0 + kLanes * kGather < cnt)
            load_nbr_batch<kGather, kLanes>(nbr, i, k0 + kLanes * kGather, nbr_stride, cnt, jn);
#pragma unroll
          for (int u = 0; u < kGather; ++u) {
            q[u] = __ldg(pred + j[u]);
            b[u] = __ldg(dens_b + j[u]);
          }
#pragma unroll
          for (int u = 0; u < kGather; ++u)
            if (k0 + kLanes * u < cnt) pressure_pair(S, p, Pi, Pni, q[u], b[u], f);
        }
      } else if (sub == 0) {
        walk_runs<kTables>(S, start, cell_tab, cell_first[i], __float_as_uint(pi.w), pred,
                           [&](uint32_t j, float4 q) {
          if (j == i) return;
          const float dx = q.x - p.x, dy = q.y - p.y, dz = q.z - p.z;
          if (dist2(dx, dy, dz) <= S.cut_le)
            pressure_pair(S, p, Pi, Pni, q, __ldg(dens_b + j), f);
        });
      }
      if (kLanes == 2) {
        f.x += __shfl_xor_sync(kFull, f.x, 16);
        f.y += __shfl_xor_sync(kFull, f.y, 16);
        f.z += __shfl_xor_sync(kFull, f.z, 16);
      }
      if (!live || sub != 0) continue;
      const float inv_rho = 1.0f / di.x;
      const float ax = f.x * inv_rho, ay = f.y * inv_rho, az = f.z * inv_rho;
      const float4 v = vel[i];
      // viscosity record rec_v[i] = (predicted position, post-pressure velocity)
      store_rec(rec_v, i, pi,
                make_float4(v.x + ax * S.dt, v.y + ay * S.dt, v.z + az * S.dt, 0.f));
      if (dbg_accp) dbg_accp[i] = make_float4(ax, ay, az, 0.0f);
    }
  }
}

// ------------------------------------------------ viscosity + integrate
// CalculateViscosityForce (:424-464) over the neighbour list reading the
// post-pressure snapshot (Jacobi); poly6 = (r^2 - d^2)^3 for dist < r. Then
// pos += v*dt and the box collision (:81-108). With fuse_next the next
// substep's prediction / cell index / histogram (k_predict_hash) runs here on the
// new state.
__device__ __forceinline__ void visc_pair(const SceneDev& S, float3 p,
                                          float4 vi, float4 q, float4 vj,
                                          float3& f) {
  const float dx = q.x - p.x, dy = q.y - p.y, dz = q.z - p.z;
  const float d2 = dist2(dx, dy, dz);
  if (d2 <= S.cut_lt) {
    const float w = S.r2 - d2;
    const float w3 = w * w * w;
    f.x = fmaf(vj.x - vi.x, w3, f.x);
    f.y = fmaf(vj.y - vi.y, w3, f.y);
    f.z = fmaf(vj.z - vi.z, w3, f.z);
  }
}

// kLanes lanes per particle as in k_pressure.
template <int kGather, int kTables, int kLanes>
__global__ void k_visc_integrate(
    const uint2* __restrict__ tiles, uint32_t ntiles,
    const SceneDev* __restrict__ scenes, const float4* __restrict__ pred,
    const uint32_t* __restrict__ start,
    const uint32_t* __restrict__ cell_first, const uint2* __restrict__ cell_tab,
    const uint32_t* __restrict__ nbr, const uint32_t* __restrict__ ncount,
    uint32_t nbr_stride, uint32_t nbr_cap, const float4* __restrict__ rec_v,
    float4* __restrict__ pos, float4* __restrict__ vel,
    float4* __restrict__ out4, int fuse_next, uint32_t* __restrict__ count,
    uint4* __restrict__ keyrank, float4* __restrict__ dbg_velv,
    uint32_t* status) {
  static_assert(kLanes == 1 || kLanes == 2, "one or two lanes per particle");
  pdl_enter();
  const uint32_t lane = lane_id();
  constexpr uint32_t kPer = 32 / kLanes;  // particles per pass
  const uint32_t sub = lane / kPer;       // this lane's share of the list
  for (uint32_t t = warp_id_global(); t < ntiles; t += warps_total()) {
    const uint2 tile = tiles[t];
    const SceneDev S = scenes[tile_scene(tile)];  // registers, not reloads
#pragma unroll 1
    for (uint32_t h = 0; h < kLanes; ++h) {
      const uint32_t li = h * kPer + lane % kPer;
      const bool in_tile = li < tile_len(tile);
      const bool live = in_tile && sub == 0;  // the lane that owns the particle
      const uint32_t i = tile.y + (in_tile ? li : 0u);
      bool bad = false;
      uint32_t key = 0, cell = 0, id = 0;
      float4 pi, vi;
      float3 f = make_float3(0.0f, 0.0f, 0.0f);
      if (in_tile) {
        load_rec(rec_v, i, pi, vi);
        const float3 p = make_float3(pi.x, pi.y, pi.z);
        const uint32_t cnt = ncount[i];
        if (cnt <= nbr_cap) {
          uint32_t jn[kGather];
          if (sub < cnt) load_nbr_batch<kGather, kLanes>(nbr, i, sub, nbr_stride, cnt, jn);
          for (uint32_t k0 = sub; k0 < cnt; k0 += kLanes * kGather) {
            uint32_t j[kGather];
            float4 q[kGather], vj[kGather];
#pragma unroll
            for (int u = 0; u < kGather; ++u) j[u] = (k0 + kLanes * u < cnt) ? jn[u] : i;
            if (k0 + kLanes * kGather < cnt)
              load_nbr_batch<kGather, kLanes>(nbr, i, k0 + kLanes * kGather, nbr_stride, cnt,
                                              jn);
#pragma unroll
            for (int u = 0; u < kGather; ++u) load_rec(rec_v, j[u], q[u], vj[u]);
#pragma unroll
            for (int u = 0; u < kGather; ++u)
              if (k0 + kLanes * u < cnt) visc_pair(S, p, vi, q[u], vj[u], f);
          }
        } else if (sub == 0) {
          walk_runs<kTables>(S, start, cell_tab, cell_first[i], __float_as_uint(pi.w), pred,
                             [&](uint32_t j, float4 q) {
            if (j != i) visc_pair(S, p, vi, q, __ldg(rec_v + 2ull * j + 1), f);
          });
        }
      }
      if (kLanes == 2) {
        f.x += __shfl_xor_sync(kFull, f.x, 16);
        f.y += __shfl_xor_sync(kFull, f.y, 16);
        f.z += __shfl_xor_sync(kFull, f.z, 16);
      }
      if (live) {
        const float c = S.vscale * S.mu * S.dt;
        float3 v = make_float3(vi.x + f.x * c, vi.y + f.y * c, vi.z + f.z * c);
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
        id = __float_as_uint(x.w);
        if (out4) {
          if (id < S.n) out4[S.base + id] = make_float4(x.x, x.y, x.z, 0.34f);
          else bad = true;
        }
        // the grid constants are read here, not kept in registers through the loop
        if (fuse_next) predict_key(scenes[tile_scene(tile)], x, v4, key, cell);
      }
      if (fuse_next) {
        const uint32_t r = aggregated_rank(count, key, live);
        if (live) keyrank[i] = make_uint4(key, r, cell, id);
      }
      if (__any_sync(kFull, bad) && lane == 0) flag(status, kStatusNonFinite);
    }
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
  if (oids) oids[k] = id;
  if (id >= n) return;
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

// Caller index -> slot for scene slots [first, first + n): the inverse of
// the ids the slots carry.
__global__ void k_slot_map(uint32_t first, uint32_t n, const float4* __restrict__ pos,
                           uint32_t* __restrict__ slot_of) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const uint32_t id = __float_as_uint(pos[first + k].w);
  if (id < n) slot_of[id] = first + k;
}

// This lane's W floats of row i0 + lane (lane < rows) into the warp's staging
// row buffer, then the warp's rows out as 16-byte words: 32 full rows are
// 8W aligned words (out is 16-byte aligned and i0 a multiple of 32); a
// partial last group goes out word by word.
template <int W>
__device__ __forceinline__ void store_rows(float* buf, float* __restrict__ out, uint32_t i0,
                                           uint32_t rows, uint32_t lane, const float* v) {
  if (lane < rows) {
#pragma unroll
    for (int c = 0; c < W; ++c) buf[W * lane + c] = v[c];
  }
  __syncwarp();
  float* dst = out + static_cast<uint64_t>(W) * i0;
  if (rows == 32u) {
    if (lane < 8u * W)
      reinterpret_cast<float4*>(dst)[lane] = reinterpret_cast<const float4*>(buf)[lane];
  } else {
    for (uint32_t f = lane; f < W * rows; f += 32u) dst[f] = buf[f];
  }
  __syncwarp();
}

// Caller-order rows written straight into host memory the device maps
// (pinned, 16-byte aligned), a warp per 32 consecutive caller indices: the
// warp gathers its rows' slots through slot_of and stores whole aligned
// 16-byte words, so the host link carries full lines (scattered 12-byte row
// stores over the link run at a tenth of its rate). A caller index whose
// slot_of entry is not a slot of the scene (ids that are no permutation: the
// status flags report the lost slot) gets a zero row.
__global__ void __launch_bounds__(256) k_export_rows(uint32_t first, uint32_t n,
                                                     const uint32_t* __restrict__ slot_of,
                                                     const float4* __restrict__ pos,
                                                     const float4* __restrict__ vel,
                                                     const float2* __restrict__ dens,
                                                     float* __restrict__ opos,
                                                     float* __restrict__ ovel,
                                                     float* __restrict__ odens) {
  __shared__ __align__(16) float buf[8][96];
  const uint32_t lane = threadIdx.x & 31u, w = threadIdx.x >> 5;
  const uint32_t i0 = (blockIdx.x * 8u + w) * 32u;
  if (i0 >= n) return;
  const uint32_t rows = min(32u, n - i0);
  const uint32_t s = lane < rows ? slot_of[i0 + lane] : first;
  const bool ok = lane < rows && s - first < n;
  if (opos) {
    const float4 p = ok ? pos[s] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float v[3] = {p.x, p.y, p.z};
    store_rows<3>(buf[w], opos, i0, rows, lane, v);
  }
  if (ovel) {
    const float4 q = ok ? vel[s] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float v[3] = {q.x, q.y, q.z};
    store_rows<3>(buf[w], ovel, i0, rows, lane, v);
  }
  if (odens) {
    const float2 d = ok ? dens[s] : make_float2(0.f, 0.f);
    const float v[2] = {d.x, d.y};
    store_rows<2>(buf[w], odens, i0, rows, lane, v);
  }
}

// ------------------------------------------------------ reference lookup
// The reference's spatial lookup of a captured substep (UpdateSpatialLookup,
// physicsWorld.cc:466-496) from the predicted positions of the sorted
// layout, by a counting sort of its own: HashCell and key = hash % n of every
// particle (written by particle index), entries in (key, particle index)
// order, and the start of every key.
__global__ void k_ref_hash(const uint2* __restrict__ tiles, uint32_t ntiles,
                           const SceneDev* __restrict__ scenes,
                           const float4* __restrict__ pred,
                           const float4* __restrict__ pos,
                           uint32_t* __restrict__ count,
                           uint2* __restrict__ keyrank,
                           uint32_t* __restrict__ ohash,
                           uint32_t* __restrict__ okey, uint32_t* status) {
  pdl_enter();
  const uint32_t lane = lane_id();
  for (uint32_t t = warp_id_global(); t < ntiles; t += warps_total()) {
    const uint2 tile = tiles[t];
    const SceneDev S = scenes[tile_scene(tile)];
    const uint32_t s = tile.y + lane;
    const bool live = lane < tile_len(tile);
    uint32_t key = 0, hash = 0, id = 0;
    if (live) {
      const float4 q = pred[s];
      hash = hash_of(S, make_float3(q.x, q.y, q.z));
      key = S.base + fastmod(hash, S.fm, S.n);
      id = __float_as_uint(pos[s].w);
    }
    const uint32_t r = aggregated_rank(count, key, live);
    if (!live) continue;
    keyrank[s] = make_uint2(key, r);
    if (id < S.n) {
      ohash[S.base + id] = hash;
      okey[S.base + id] = key - S.base;
    } else {
      flag(status, kStatusRange);
    }
  }
}

// Bucket every particle index at start[key] + arrival rank.
__global__ void k_ref_scatter(const uint2* __restrict__ tiles, uint32_t ntiles,
                              const float4* __restrict__ pos,
                              const uint2* __restrict__ keyrank,
                              const uint32_t* __restrict__ start,
                              uint32_t total, uint32_t* __restrict__ tmp,
                              uint32_t* status) {
  pdl_enter();
  const uint32_t lane = lane_id();
  for (uint32_t t = warp_id_global(); t < ntiles; t += warps_total()) {
    const uint2 tile = tiles[t];
    const uint32_t s = tile.y + lane;
    if (lane >= tile_len(tile)) continue;
    const uint2 kr = keyrank[s];
    const uint32_t dst = start[kr.x] + kr.y;
    if (dst >= total) { flag(status, kStatusRange); continue; }
    tmp[dst] = __float_as_uint(pos[s].w);
  }
}

// Order every bucket by particle index: the canonical (key, index) order.
__global__ void k_ref_order(const uint2* __restrict__ tiles, uint32_t ntiles,
                            const float4* __restrict__ pos,
                            const uint2* __restrict__ keyrank,
                            const uint32_t* __restrict__ start,
                            const uint32_t* __restrict__ tmp,
                            uint32_t* __restrict__ sorted) {
  pdl_enter();
  const uint32_t lane = lane_id();
  for (uint32_t t = warp_id_global(); t < ntiles; t += warps_total()) {
    const uint2 tile = tiles[t];
    const uint32_t s = tile.y + lane;
    if (lane >= tile_len(tile)) continue;
    const uint32_t key = keyrank[s].x;
    const uint32_t id = __float_as_uint(pos[s].w);
    const uint32_t b0 = start[key], b1 = start[key + 1];
    uint32_t rank = 0;
    for (uint32_t u = b0; u < b1; ++u) rank += tmp[u] < id ? 1u : 0u;
    if (b0 + rank < b1) sorted[b0 + rank] = id;
  }
}

// Per-slot debug intermediates of one scene to caller order.
__global__ void k_export_debug(uint32_t first, uint32_t n,
                               const float4* __restrict__ pos,
                               const float4* __restrict__ accp,
                               const float4* __restrict__ velp,
                               const float4* __restrict__ velv,
                               float* __restrict__ oaccp,
                               float* __restrict__ ovelp,
                               float* __restrict__ ovelv) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const uint32_t s = first + k;
  const uint32_t id = __float_as_uint(pos[s].w);
  if (id >= n) return;
  const float4 a = accp[s], b = velp[s], c = velv[s];
  oaccp[3 * id] = a.x; oaccp[3 * id + 1] = a.y; oaccp[3 * id + 2] = a.z;
  ovelp[3 * id] = b.x; ovelp[3 * id + 1] = b.y; ovelp[3 * id + 2] = b.z;
  ovelv[3 * id] = c.x; ovelv[3 * id + 1] = c.y; ovelv[3 * id + 2] = c.z;
}

// The timed sort's own layout of a captured substep, per slot of one scene:
// the particle at each slot (slot_ids, slot order), and per particle (caller
// order) its internal cell index (pred.w, written by k_reorder) and its
// entry in the scene's key table.
__global__ void k_export_layout(uint32_t first, uint32_t n,
                                const SceneDev* __restrict__ scene,
                                const float4* __restrict__ pos,
                                const float4* __restrict__ pred,
                                uint32_t* __restrict__ ocell,
                                uint32_t* __restrict__ okey,
                                uint32_t* __restrict__ oslot) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const uint32_t s = first + k;
  const uint32_t id = __float_as_uint(pos[s].w);
  const uint32_t cell = __float_as_uint(pred[s].w);
  oslot[k] = id;
  if (id >= n) return;
  const SceneDev& S = *scene;
  ocell[id] = cell;
  okey[id] = table_key(S, cell) - S.tbase;
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

// Upload straight from host memory (pinned buffers the device can address,
// read over the CPU link): the caller-order float3 rows of 32 consecutive
// particles are 384 contiguous bytes, 24 float4. Each warp reads its chunk as
// aligned float4 (the link's transactions stay full) and transposes it
// through shared memory; a partial last chunk goes by scalar loads, so
// nothing outside the 3n floats is touched. The arrays must be 16-byte
// aligned (checked by the launcher's caller).
constexpr int kXferBlock = 256;
constexpr int kXferWarps = kXferBlock / 32;

// With `scene` the kernel also predicts the next step's first substep for
// the imported state exactly as k_predict_hash would (key, arrival rank,
// cell, caller index, and the histogram), so that step can skip it.
__global__ void __launch_bounds__(kXferBlock)
k_import_rows(uint32_t first, uint32_t n, const float* __restrict__ ipos,
              const float* __restrict__ ivel, float4* __restrict__ pos,
              float4* __restrict__ vel, const SceneDev* __restrict__ scene,
              uint32_t* __restrict__ count, uint4* __restrict__ keyrank) {
  __shared__ __align__(16) float s_rows[kXferWarps][2][96];
  const uint32_t lane = lane_id(), w = threadIdx.x >> 5;
  const uint32_t k0 = (blockIdx.x * kXferWarps + w) * 32u;
  if (k0 >= n) return;  // whole warp
  const uint32_t cnt = min(32u, n - k0);
  float* sp = s_rows[w][0];
  float* sv = s_rows[w][1];
  const uint64_t f0 = 3ull * k0;
  if (cnt == 32u) {
    if (lane < 24u) {
      reinterpret_cast<float4*>(sp)[lane] =
          __ldcs(reinterpret_cast<const float4*>(ipos + f0) + lane);
      if (ivel)
        reinterpret_cast<float4*>(sv)[lane] =
            __ldcs(reinterpret_cast<const float4*>(ivel + f0) + lane);
    }
  } else {
    for (uint32_t e = lane; e < 3u * cnt; e += 32u) {
      sp[e] = ipos[f0 + e];
      if (ivel) sv[e] = ivel[f0 + e];
    }
  }
  __syncwarp();
  const bool live = lane < cnt;
  const uint32_t k = k0 + lane;
  float4 p4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f), v4 = p4;
  if (live) {
    p4 = make_float4(sp[3 * lane], sp[3 * lane + 1], sp[3 * lane + 2], __uint_as_float(k));
    if (ivel) v4 = make_float4(sv[3 * lane], sv[3 * lane + 1], sv[3 * lane + 2], 0.0f);
    pos[first + k] = p4;
    vel[first + k] = v4;
  }
  if (scene) {  // every lane of the warp takes part (warp-aggregated atomics)
    const SceneDev S = *scene;
    uint32_t key = 0, cell = 0;
    if (live) predict_key(S, p4, v4, key, cell);
    const uint32_t r = aggregated_rank(count, key, live);
    if (live) keyrank[first + k] = make_uint4(key, r, cell, k);
  }
}

}  // namespace

// ------------------------------------------------------------- launchers
// Substep kernels go out with programmatic stream serialisation: the next
// kernel is scheduled during its predecessor's last wave and waits for it in
// pdl_enter(), which hides the launch and ramp-up between the seven to nine
// kernels of a substep (inside a graph these become programmatic edges).
template <class... KArgs, class... Args>
cudaError_t launch_pdl(bool pdl, void (*kernel)(KArgs...), uint32_t grid, int block,
                       cudaStream_t st, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(static_cast<unsigned>(block));
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = pdl ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

cudaError_t launch_predict_hash(const LaunchCtx& c, const Tiles& old_tiles,
                                cudaStream_t st) {
  if (old_tiles.n == 0) return cudaSuccess;
  return launch_pdl(c.pdl, k_predict_hash, grid_for(old_tiles.n, c.block_misc, c.max_blocks),
                    c.block_misc, st, old_tiles.d, old_tiles.n, c.scenes, c.pos,
                    c.vel, c.count, c.keyrank);
}

cudaError_t launch_scan(const LaunchCtx& c, uint32_t len, cudaStream_t st) {
  const uint32_t nb = (len + kScanBlock - 1) / kScanBlock;
  if (nb == 0) return cudaSuccess;
  const int fold = nb <= kScanFoldBlocks ? 1 : 0;
  cudaError_t e = launch_pdl(c.pdl, k_scan_reduce, nb, kScanThreads, st, c.count, len, c.partial);
  if (e == cudaSuccess && !fold)
    e = launch_pdl(c.pdl, k_scan_partials, 1, kScanThreads, st, c.partial, nb, c.start, len);
  if (e == cudaSuccess)
    e = launch_pdl(c.pdl, k_scan_down, nb, kScanThreads, st, c.count, len, c.partial, nb,
                   fold, c.start);
  return e;
}

int kernels_per_substep(uint32_t keys, int tables) {
  const uint32_t nb = (keys + kScanBlock - 1) / kScanBlock;
  return (nb <= kScanFoldBlocks ? 8 : 9) - (tables == kTablesDirect ? 1 : 0);
}

uint32_t scan_partials_needed(uint64_t len) {
  return static_cast<uint32_t>((len + kScanBlock - 1) / kScanBlock) + 1;
}

cudaError_t launch_sort_reorder(const LaunchCtx& c, const Tiles& old_tiles,
                                const Tiles& new_tiles, uint32_t total,
                                cudaStream_t st) {
  cudaError_t e = cudaSuccess;
  if (old_tiles.n)
    e = launch_pdl(c.pdl, k_scatter, grid_for(old_tiles.n, c.block_misc, c.max_blocks),
                   c.block_misc, st, old_tiles.d, old_tiles.n, c.keyrank, c.start,
                   total, c.tmp_hi, c.tmp_src, c.status);
  if (new_tiles.n && e == cudaSuccess) {
    e = launch_pdl(c.pdl, k_reorder, grid_for(new_tiles.n, c.block_misc, c.max_blocks),
                   c.block_misc, st, new_tiles.d, new_tiles.n, c.scenes, c.tmp_hi,
                   c.tmp_src, c.start, c.pos, c.vel, c.pos2, c.vel2, c.pred,
                   c.hash_s, c.cell_first, c.src_limit, c.status);
    if (e == cudaSuccess && c.tables != kTablesDirect)
      e = launch_pdl(c.pdl, k_cell_table, grid_for(new_tiles.n, kCellTableBlock, c.max_blocks),
                     kCellTableBlock, st, new_tiles.d, new_tiles.n, c.scenes,
                     c.hash_s, c.cell_first, c.start, c.cell_tab);
  }
  return e;
}

cudaError_t launch_density(const LaunchCtx& c, const Tiles& tiles,
                           cudaStream_t st) {
  if (tiles.n == 0) return cudaSuccess;
  const int b = c.block_nbr;
  const uint32_t g = grid_for(tiles.n, b, c.max_blocks);
  if (c.cell_tile <= 1)
    return launch_pdl(c.pdl,
                      c.tables == kTablesDirect    ? k_density_walk<kTablesDirect>
                      : c.tables == kTablesBuckets ? k_density_walk<kTablesBuckets>
                                                   : k_density_walk<kTablesMixed>,
                      g, b, st, tiles.d, tiles.n, c.scenes, c.pred,
                      c.start, c.cell_first, c.cell_tab, c.dens_a, c.dens_b, c.nbr,
                      c.ncount, c.nbr_stride, c.nbr_cap);
  auto kern = c.cell_tile <= 64    ? k_density<2>
              : c.cell_tile <= 128 ? k_density<4>
              : c.cell_tile <= 192 ? k_density<6>
                                   : k_density<8>;
  return launch_pdl(c.pdl, kern, g, b, st, tiles.d, tiles.n, c.scenes, c.pred,
                    c.start, c.cell_first, c.cell_tab, c.dens_a, c.dens_b, c.nbr,
                    c.ncount, c.nbr_stride, c.nbr_cap);
}

// The instantiations for a gather batch (2, 3, 4 or 8) and the launch's
// table forms.
template <int kTables, int kLanes>
auto pressure_kernel(int gather) {
  return gather == 2   ? k_pressure<2, kTables, kLanes>
         : gather == 3 ? k_pressure<3, kTables, kLanes>
         : gather == 8 ? k_pressure<8, kTables, kLanes>
                       : k_pressure<4, kTables, kLanes>;
}

template <int kTables>
auto pressure_kernel(int gather, int lanes) {
  return lanes == 2 ? pressure_kernel<kTables, 2>(gather) : pressure_kernel<kTables, 1>(gather);
}

template <int kTables, int kLanes>
auto visc_kernel(int gather) {
  return gather == 2   ? k_visc_integrate<2, kTables, kLanes>
         : gather == 3 ? k_visc_integrate<3, kTables, kLanes>
         : gather == 8 ? k_visc_integrate<8, kTables, kLanes>
                       : k_visc_integrate<4, kTables, kLanes>;
}

template <int kTables>
auto visc_kernel(int gather, int lanes) {
  return lanes == 2 ? visc_kernel<kTables, 2>(gather) : visc_kernel<kTables, 1>(gather);
}

cudaError_t launch_pressure(const LaunchCtx& c, const Tiles& tiles,
                            cudaStream_t st) {
  if (tiles.n == 0) return cudaSuccess;
  const int b = c.block_force;
  auto kern = c.tables == kTablesDirect    ? pressure_kernel<kTablesDirect>(c.gather, c.lanes)
              : c.tables == kTablesBuckets ? pressure_kernel<kTablesBuckets>(c.gather, c.lanes)
                                           : pressure_kernel<kTablesMixed>(c.gather, c.lanes);
  return launch_pdl(c.pdl, kern, grid_for(tiles.n, b, c.max_blocks), b, st, tiles.d,
                    tiles.n, c.scenes, c.pred, c.start, c.cell_first, c.cell_tab,
                    c.dens_a, c.dens_b, c.nbr, c.ncount, c.nbr_stride, c.nbr_cap,
                    c.vel2, c.rec_v, c.dbg_accp);
}

cudaError_t launch_visc_integrate(const LaunchCtx& c, const Tiles& tiles,
                                  int fuse_next, int write_out,
                                  cudaStream_t st) {
  if (tiles.n == 0) return cudaSuccess;
  const int b = c.block_force;
  auto kern = c.tables == kTablesDirect    ? visc_kernel<kTablesDirect>(c.gather, c.lanes)
              : c.tables == kTablesBuckets ? visc_kernel<kTablesBuckets>(c.gather, c.lanes)
                                           : visc_kernel<kTablesMixed>(c.gather, c.lanes);
  return launch_pdl(c.pdl, kern, grid_for(tiles.n, b, c.max_blocks), b, st, tiles.d,
                    tiles.n, c.scenes, c.pred, c.start, c.cell_first, c.cell_tab, c.nbr,
                    c.ncount, c.nbr_stride, c.nbr_cap, c.rec_v, c.pos2, c.vel2,
                    write_out ? c.out4 : nullptr, fuse_next, c.count, c.keyrank,
                    c.dbg_velv, c.status);
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

cudaError_t launch_export_rows(uint32_t first, uint32_t n, const float4* pos,
                              const float4* vel, const float2* dens, uint32_t* slot_of,
                              float* opos, float* ovel, float* odens, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  k_slot_map<<<(n + 255) / 256, 256, 0, st>>>(first, n, pos, slot_of);
  k_export_rows<<<(n + 255) / 256, 256, 0, st>>>(first, n, slot_of, pos, vel, dens, opos,
                                                 ovel, odens);
  return cudaGetLastError();
}

cudaError_t launch_export_debug(uint32_t first, uint32_t n, const float4* pos,
                                const float4* accp, const float4* velp,
                                const float4* velv, float* oaccp, float* ovelp,
                                float* ovelv, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  k_export_debug<<<(n + 255) / 256, 256, 0, st>>>(first, n, pos, accp, velp,
                                                  velv, oaccp, ovelp, ovelv);
  return cudaGetLastError();
}

cudaError_t launch_export_layout(uint32_t first, uint32_t n, const SceneDev* scene,
                                 const float4* pos, const float4* pred, uint32_t* ocell,
                                 uint32_t* okey, uint32_t* oslot, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  k_export_layout<<<(n + 255) / 256, 256, 0, st>>>(first, n, scene, pos, pred, ocell,
                                                  okey, oslot);
  return cudaGetLastError();
}

cudaError_t launch_ref_lookup(const LaunchCtx& c, const Tiles& new_tiles,
                              uint32_t total, cudaStream_t st) {
  if (new_tiles.n == 0) return cudaSuccess;
  const uint32_t g = grid_for(new_tiles.n, c.block_misc, c.max_blocks);
  cudaError_t e = launch_pdl(c.pdl, k_ref_hash, g, c.block_misc, st, new_tiles.d,
                             new_tiles.n, c.scenes, c.pred, c.pos2, c.dbg_count,
                             c.dbg_keyrank, c.dbg_hash, c.dbg_key, c.status);
  LaunchCtx d = c;  // the scan over the lookup's own histogram
  d.count = c.dbg_count;
  d.start = c.dbg_start;
  d.partial = c.dbg_partial;
  if (e == cudaSuccess) e = launch_scan(d, total, st);
  if (e == cudaSuccess)
    e = launch_pdl(c.pdl, k_ref_scatter, g, c.block_misc, st, new_tiles.d, new_tiles.n,
                   c.pos2, c.dbg_keyrank, c.dbg_start, total, c.dbg_tmp, c.status);
  if (e == cudaSuccess)
    e = launch_pdl(c.pdl, k_ref_order, g, c.block_misc, st, new_tiles.d, new_tiles.n,
                   c.pos2, c.dbg_keyrank, c.dbg_start, c.dbg_tmp, c.dbg_sorted);
  return e;
}

cudaError_t launch_import(uint32_t first, uint32_t n, const float* ipos,
                          const float* ivel, float4* pos, float4* vel,
                          cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  k_import<<<(n + 255) / 256, 256, 0, st>>>(first, n, ipos, ivel, pos, vel);
  return cudaGetLastError();
}

cudaError_t launch_import_rows(uint32_t first, uint32_t n, const float* ipos,
                               const float* ivel, float4* pos, float4* vel,
                               const SceneDev* scene, uint32_t* count, uint4* keyrank,
                               cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  const uint32_t warps = (n + 31) / 32;
  k_import_rows<<<(warps + kXferWarps - 1) / kXferWarps, kXferBlock, 0, st>>>(
      first, n, ipos, ivel, pos, vel, scene, count, keyrank);
  return cudaGetLastError();
}

}  // namespace sph
