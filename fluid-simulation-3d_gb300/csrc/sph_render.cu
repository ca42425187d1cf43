// Headless render of a scene's particles: the billboard splats of
// bin/shaders/particleRender.vs/.fs with the speed colour gradient of
// FluidSimCPU::updateColors (projects/Simulation/code/simulations/
// fluidSimCPU.cc:100-124), drawn into an RGBA8 + depth image instead of a
// GL framebuffer.
//
// What the shaders compute, per particle at position c with scale s:
//  - a screen-aligned quad: corners c_clip + P * (+-s/2, +-s/2, 0, 0), with
//    c_clip = ViewProj * (c, 1) (particleRender.vs:34-41);
//  - fragments whose interpolated offset P * (o, 0) is longer than s / 4
//    are discarded (particleRender.fs:12-13), which leaves an ellipse;
//  - depth test GL_LESS (gameApp.cc:158), colour = the particle's colour.
// Here every quantity that decides coverage, depth or colour is evaluated
// with explicitly rounded operations in a fixed order (no contraction), so
// the CPU restatement in the oracle reproduces the image bit for bit:
//  - clip = (m0 x + m1 y) + (m2 z + m3), glm's order for mat4 * vec4;
//  - window x = (clip.x +- a s/2) / clip.w * W/2 + W/2 per corner, likewise
//    y; depth = clip.z / clip.w * 1/2 + 1/2 (the quad has one depth);
//  - pixel centres (px + 1/2, py + 1/2) inside [X0, X1) x (Y0, Y1] (GL's
//    top-left rule in its y-up window coordinates);
//  - the offset at a pixel centre is linear across the quad: v = f (2 o) - o
//    with f = (centre - X0) * (1 / (X1 - X0)) the centre's fraction of the
//    quad; discard if vx^2 + vy^2 > (s / 4)^2;
//  - the nearest fragment wins, ties to the lower particle index (first
//    drawn under GL_LESS), through a 64-bit atomicMin of (depth bits,
//    caller index): deterministic whatever the launch order;
//  - colour components convert to 8 bits by round(clamp(c, 0, 1) * 255), as
//    GL converts to an UNORM8 colour buffer.
#include <cuda_runtime.h>

#include <cstdint>

#include "sph_render.h"

namespace sph {
namespace {

__device__ __forceinline__ float fm(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fa(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fs(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fd(float a, float b) { return __fdiv_rn(a, b); }

// Gradient of FluidSimCPU::updateColors over getSpeedNormalzied
// (physicsWorld.cc:178-182): clamp(|v|, 0, 1.5) / 1.5 through the colours
// of fluidSimCPU.h:26-29 with breakpoints 0.33 and 0.66.
__device__ uint32_t speed_colour(float vx, float vy, float vz) {
  const float len = __fsqrt_rn(fa(fa(fm(vx, vx), fm(vy, vy)), fm(vz, vz)));
  const float nrm = fd(fminf(fmaxf(len, 0.0f), 1.5f), 1.5f);
  const float b1 = 0.33f, b2 = 0.66f;
  const float4 c1 = make_float4(0.0f, 0.75f, 1.0f, 1.0f);
  const float4 c2 = make_float4(0.0f, 1.0f, 0.0f, 1.0f);
  const float4 c3 = make_float4(1.0f, 1.0f, 0.0f, 1.0f);
  const float4 c4 = make_float4(1.0f, 0.0f, 0.0f, 1.0f);
  float t;
  float4 lo, hi;
  if (nrm <= b1) {
    t = fd(nrm, b1);
    lo = c1;
    hi = c2;
  } else if (nrm <= b2) {
    t = fd(fs(nrm, b1), fs(b2, b1));
    lo = c2;
    hi = c3;
  } else {
    t = fd(fs(nrm, b2), fs(1.0f, b2));
    lo = c3;
    hi = c4;
  }
  const float u = fs(1.0f, t);
  const float c[4] = {fa(fm(u, lo.x), fm(t, hi.x)), fa(fm(u, lo.y), fm(t, hi.y)),
                      fa(fm(u, lo.z), fm(t, hi.z)), fa(fm(u, lo.w), fm(t, hi.w))};
  uint32_t out = 0;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const uint32_t b = __float2uint_rn(fm(fminf(fmaxf(c[k], 0.0f), 1.0f), 255.0f));
    out |= b << (8 * k);
  }
  return out;
}

__device__ __forceinline__ float row_dot(const float* m, int r, float x, float y, float z) {
  return fa(fa(fm(m[r], x), fm(m[4 + r], y)), fa(fm(m[8 + r], z), m[12 + r]));
}

// The discard and depth tests of particleRender.fs at the centre of pixel
// (px, py) of a splat whose quad spans [x0, x1) x (y0, y1] in window
// coordinates (idx, idy: the reciprocal widths).
__device__ __forceinline__ void splat_pixel(const RenderView& v, int px, float vy2, float x0,
                                            float idx, float q2, unsigned long long key,
                                            unsigned long long* __restrict__ row) {
  const float fx = fm(fs(fa(static_cast<float>(px), 0.5f), x0), idx);
  const float vx = fs(fm(fx, fa(v.ox, v.ox)), v.ox);
  if (fa(fm(vx, vx), vy2) > q2) return;  // discard: |offset| > s/4
  atomicMin(row + px, key);
}

__device__ __forceinline__ float splat_vy2(const RenderView& v, int py, float y0, float idy) {
  const float fy = fm(fs(fa(static_cast<float>(py), 0.5f), y0), idy);
  const float vy = fs(fm(fy, fa(v.oy, v.oy)), v.oy);
  return fm(vy, vy);
}

// Particles of the scene's slots [first, first + n), one per thread: its
// colour (by caller index) and its splat into the (depth, index) buffer.
// A splat of more than kWarpSplat pixels (a particle close to the camera)
// is drawn by the whole warp, the lanes taking its pixels in turn.
constexpr int kWarpSplat = 64;

__global__ void k_splat(uint32_t first, uint32_t n, const float4* __restrict__ pos,
                        const float4* __restrict__ vel, RenderView v,
                        unsigned long long* __restrict__ keys,
                        uint32_t* __restrict__ colours) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t lane = threadIdx.x & 31u;
  bool live = k < n;
  uint32_t id = 0;
  float4 p = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  if (live) {
    p = pos[first + k];
    id = __float_as_uint(p.w);
    live = id < n;
  }
  if (live) {
    const float4 vv = vel[first + k];
    colours[id] = speed_colour(vv.x, vv.y, vv.z);
  }
  float x0 = 0.0f, x1 = 0.0f, y0 = 0.0f, y1 = 0.0f, depth = 0.0f;
  if (live) {
    const float cx = row_dot(v.vp, 0, p.x, p.y, p.z);
    const float cy = row_dot(v.vp, 1, p.x, p.y, p.z);
    const float cz = row_dot(v.vp, 2, p.x, p.y, p.z);
    const float cw = row_dot(v.vp, 3, p.x, p.y, p.z);
    live = cw > 0.0f && cz >= -cw && cz <= cw;  // else behind / outside near-far
    if (live) {
      x0 = fa(fm(fd(fs(cx, v.ox), cw), v.hw), v.hw);
      x1 = fa(fm(fd(fa(cx, v.ox), cw), v.hw), v.hw);
      y0 = fa(fm(fd(fs(cy, v.oy), cw), v.hh), v.hh);
      y1 = fa(fm(fd(fa(cy, v.oy), cw), v.hh), v.hh);
      depth = fa(fm(fd(cz, cw), 0.5f), 0.5f);
      live = x1 > x0 && y1 > y0;  // degenerate (also NaN)
    }
  }
  // covered centres: x0 <= px + 1/2 < x1, y0 < py + 1/2 <= y1; clamped to the
  // image in float before the integer conversion
  int xa = 0, xb = -1, ya = 0, yb = -1;
  if (live) {
    const float fw = static_cast<float>(v.width), fh = static_cast<float>(v.height);
    const int px0 = static_cast<int>(ceilf(fminf(fmaxf(fs(x0, 0.5f), -1.0f), fw)));
    const int px1 = static_cast<int>(ceilf(fminf(fmaxf(fs(x1, 0.5f), -1.0f), fw))) - 1;
    const int py0 = static_cast<int>(floorf(fminf(fmaxf(fs(y0, 0.5f), -1.0f), fh))) + 1;
    const int py1 = static_cast<int>(floorf(fminf(fmaxf(fs(y1, 0.5f), -1.0f), fh)));
    xa = max(px0, 0);
    xb = min(px1, static_cast<int>(v.width) - 1);
    ya = max(py0, 0);
    yb = min(py1, static_cast<int>(v.height) - 1);
    live = xa <= xb && ya <= yb;
  }
  const unsigned long long key =
      (static_cast<unsigned long long>(__float_as_uint(depth)) << 32) | id;
  const float q2 = fm(v.q, v.q);
  const bool big = live && (xb - xa + 1) * (yb - ya + 1) > kWarpSplat;
  if (live && !big) {
    const float idx = fd(1.0f, fs(x1, x0)), idy = fd(1.0f, fs(y1, y0));
    for (int py = ya; py <= yb; ++py) {
      const float vy2 = splat_vy2(v, py, y0, idy);
      unsigned long long* row = keys + static_cast<uint64_t>(py) * v.width;
      for (int px = xa; px <= xb; ++px) splat_pixel(v, px, vy2, x0, idx, q2, key, row);
    }
  }
  // large splats, one at a time across the warp (every lane arrives here)
  for (uint32_t m = __ballot_sync(0xffffffffu, big); m; m &= m - 1u) {
    const int src = __ffs(m) - 1;
    const int bxa = __shfl_sync(0xffffffffu, xa, src), bxb = __shfl_sync(0xffffffffu, xb, src);
    const int bya = __shfl_sync(0xffffffffu, ya, src), byb = __shfl_sync(0xffffffffu, yb, src);
    const float bx0 = __shfl_sync(0xffffffffu, x0, src), bx1 = __shfl_sync(0xffffffffu, x1, src);
    const float by0 = __shfl_sync(0xffffffffu, y0, src), by1 = __shfl_sync(0xffffffffu, y1, src);
    const uint32_t klo = __shfl_sync(0xffffffffu, static_cast<uint32_t>(key), src);
    const uint32_t khi = __shfl_sync(0xffffffffu, static_cast<uint32_t>(key >> 32), src);
    const unsigned long long bkey = (static_cast<unsigned long long>(khi) << 32) | klo;
    const float idx = fd(1.0f, fs(bx1, bx0)), idy = fd(1.0f, fs(by1, by0));
    const int w = bxb - bxa + 1, area = w * (byb - bya + 1);
    for (int t = static_cast<int>(lane); t < area; t += 32) {
      const int py = bya + t / w;
      splat_pixel(v, bxa + t % w, splat_vy2(v, py, by0, idy), bx0, idx, q2, bkey,
                  keys + static_cast<uint64_t>(py) * v.width);
    }
  }
}

// Thread per pixel: the winning particle's colour and depth, else the clear
// colour and depth 1.
__global__ void k_resolve(uint32_t pixels, const unsigned long long* __restrict__ keys,
                          const uint32_t* __restrict__ colours, uint32_t clear,
                          uint32_t* __restrict__ rgba, float* __restrict__ depth) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= pixels) return;
  const unsigned long long key = keys[i];
  if (key == ~0ull) {
    rgba[i] = clear;
    depth[i] = 1.0f;
  } else {
    rgba[i] = colours[static_cast<uint32_t>(key)];
    depth[i] = __uint_as_float(static_cast<uint32_t>(key >> 32));
  }
}

}  // namespace

cudaError_t launch_render(uint32_t first, uint32_t n, const float4* pos, const float4* vel,
                          const RenderView& view, unsigned long long* keys,
                          uint32_t* colours, uint32_t* rgba, float* depth,
                          cudaStream_t st) {
  const uint64_t pixels = static_cast<uint64_t>(view.width) * view.height;
  cudaError_t e = cudaMemsetAsync(keys, 0xff, sizeof(unsigned long long) * pixels, st);
  if (e != cudaSuccess) return e;
  if (n) {
    k_splat<<<(n + 255) / 256, 256, 0, st>>>(first, n, pos, vel, view, keys, colours);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  const uint32_t px = static_cast<uint32_t>(pixels);
  k_resolve<<<(px + 255) / 256, 256, 0, st>>>(px, keys, colours, view.clear, rgba, depth);
  return cudaGetLastError();
}

}  // namespace sph
