// Spatial lookup that allocates no device memory.
//
// Some callers cannot allocate device memory: an interactive render loop
// (like the reference's GL app) must not call cudaMalloc/cudaFree mid-frame
// because they synchronise the whole device and stall the frame; engines that
// own a fixed memory budget or a pool forbid allocations from plug-ins.
// sph_spatial_lookup_static serves them: the caller passes its own device
// buffers for inputs and outputs, and the working memory (histogram and
// bucket cursors) is the file-scope array below, 8 B per particle for up to
// SPH_STATIC_LOOKUP_MAX particles -- 512 KiB that every GPU loading this
// library keeps until the process exits.
//
// The entry point has no counterpart in the reference; it builds the same
// lookup as the main path's sort (hash, key = hash % n, the canonical
// (key, index) order, the start table with 0x7fffffff for empty keys), in one
// single-block kernel whose work is linear in n whatever the keys: the
// ordering is a stable scatter in index order, so a scene whose particles all
// share one key costs what any other scene of its size does.
#include <cstdint>
#include <mutex>
#include <string>

#include <cuda_runtime.h>

#include "../../include/sph_gb300.h"
#include "sph_device.cuh"

namespace sph {

namespace {

constexpr uint32_t kMax = SPH_STATIC_LOOKUP_MAX;
constexpr int kThreads = 1024;
constexpr int kMaxDevices = 64;

// count | cursor, kMax entries each.
__device__ __align__(256) uint32_t g_lookup_scratch[2 * kMax];

std::mutex g_mu;
uint32_t* g_scratch_addr[kMaxDevices] = {};
std::string g_static_error;

__device__ __forceinline__ uint32_t block_excl_scan_static(uint32_t x,
                                                           uint32_t* total) {
  __shared__ uint32_t sums[32];
  const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint32_t incl = x;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, incl, d);
    if (lane >= static_cast<uint32_t>(d)) incl += y;
  }
  if (lane == 31) sums[w] = incl;
  __syncthreads();
  if (w == 0) {
    uint32_t v = lane < (blockDim.x >> 5) ? sums[lane] : 0u;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, v, d);
      if (lane >= static_cast<uint32_t>(d)) v += y;
    }
    sums[lane] = v;
  }
  __syncthreads();
  const uint32_t before = w > 0 ? sums[w - 1] : 0u;
  *total = sums[(blockDim.x >> 5) - 1];
  __syncthreads();
  return before + incl - x;
}

// One block does every phase, with __syncthreads between them.
__global__ void __launch_bounds__(kThreads)
k_lookup_static(const float* __restrict__ pred3, uint32_t n, float r,
                uint64_t fm, uint32_t* __restrict__ scratch,
                uint32_t* __restrict__ ohash, uint32_t* __restrict__ okey,
                uint32_t* __restrict__ osorted, uint32_t* __restrict__ ostart) {
  uint32_t* cnt = scratch;
  uint32_t* cur = scratch + kMax;
  // The array keeps the previous call's contents: clear the histogram.
  for (uint32_t k = threadIdx.x; k < n; k += kThreads) cnt[k] = 0u;
  __syncthreads();
  // HashCell(PositionToCellCoord(pred)), key = hash % n
  // (physicsWorld.cc:499-516), and the key histogram.
  for (uint32_t i = threadIdx.x; i < n; i += kThreads) {
    const float3 p = make_float3(pred3[3 * i], pred3[3 * i + 1], pred3[3 * i + 2]);
    const uint32_t h = hash_cell(cell_of(p.x, r), cell_of(p.y, r), cell_of(p.z, r));
    const uint32_t key = fastmod(h, fm, n);
    ohash[i] = h;
    okey[i] = key;
    atomicAdd(cnt + key, 1u);
  }
  __syncthreads();
  // Exclusive prefix of the histogram = first sorted slot of each key.
  uint32_t carry = 0;
  for (uint32_t base = 0; base < n; base += kThreads) {
    const uint32_t k = base + threadIdx.x;
    const uint32_t c = k < n ? cnt[k] : 0u;
    uint32_t total;
    const uint32_t ex = block_excl_scan_static(c, &total);
    if (k < n) {
      cur[k] = carry + ex;
      ostart[k] = c ? carry + ex : 0x7fffffffu;
    }
    carry += total;
  }
  __syncthreads();
  // Stable scatter in index order: the first warp walks the particles 32 at
  // a time; lanes with equal keys take consecutive slots of their bucket in
  // lane (= index) order, from the bucket's cursor, which the leader of the
  // equal-key lanes advances. n / 32 warp steps, whatever the keys.
  if (threadIdx.x < 32) {
    const uint32_t lane = threadIdx.x;
    for (uint32_t base = 0; base < n; base += 32) {
      const uint32_t i = base + lane;
      const bool valid = i < n;
      const uint32_t am = __ballot_sync(0xffffffffu, valid);
      if (valid) {
        const uint32_t key = okey[i];
        const uint32_t peers = __match_any_sync(am, key);
        const int leader = __ffs(peers) - 1;
        uint32_t b = 0;
        if (static_cast<int>(lane) == leader) {
          b = cur[key];
          cur[key] = b + __popc(peers);
        }
        b = __shfl_sync(peers, b, leader);
        osorted[b + __popc(peers & ((1u << lane) - 1u))] = i;
      }
      __syncwarp();  // the cursors' updates are seen by the next step's leaders
    }
  }
}

}  // namespace

}  // namespace sph

extern "C" const char* sph_static_error(void) {
  std::lock_guard<std::mutex> lock(sph::g_mu);
  return sph::g_static_error.c_str();
}

extern "C" int sph_spatial_lookup_static(const float* dpred3, uint32_t n,
                                         float radius, uint32_t* dhash,
                                         uint32_t* dkey, uint32_t* dsorted_ids,
                                         uint32_t* dstart, void* stream) {
  using namespace sph;
  auto fail = [](int code, const std::string& msg) {
    std::lock_guard<std::mutex> lock(g_mu);
    g_static_error = msg;
    return code;
  };
  if (n == 0 || n > kMax)
    return fail(SPH_ERR_INVALID,
                "sph_spatial_lookup_static: n must be in [1, " +
                    std::to_string(kMax) + "], got " + std::to_string(n));
  if (!dpred3 || !dhash || !dkey || !dsorted_ids || !dstart)
    return fail(SPH_ERR_INVALID, "sph_spatial_lookup_static: null buffer");
  if (!(radius > 0.0f))
    return fail(SPH_ERR_INVALID, "sph_spatial_lookup_static: radius must be > 0");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess)
    return fail(SPH_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices)
    return fail(SPH_ERR_INVALID, "sph_spatial_lookup_static: device index too large");
  uint32_t* scratch = nullptr;
  {
    // First call on a device: resolve the array's device address with that
    // device current (a host-side use of the symbol is not a device address).
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_addr[dev]) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_lookup_scratch);
      if (e != cudaSuccess) {
        g_static_error = std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e);
        return SPH_ERR_CUDA;
      }
      g_scratch_addr[dev] = static_cast<uint32_t*>(p);
    }
    scratch = g_scratch_addr[dev];
  }
  const uint64_t fm = (~static_cast<uint64_t>(0)) / n + 1;
  k_lookup_static<<<1, kThreads, 0, static_cast<cudaStream_t>(stream)>>>(
      dpred3, n, radius, fm, scratch, dhash, dkey, dsorted_ids, dstart);
  e = cudaGetLastError();
  if (e != cudaSuccess)
    return fail(SPH_ERR_CUDA, std::string("lookup kernel: ") + cudaGetErrorString(e));
  return SPH_OK;
}
