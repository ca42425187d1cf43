// Headless particle render (sph_render.cu): the parameters the kernels take
// and their launcher.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace sph {

// A view prepared on the host from sph_view (exact float products only).
struct RenderView {
  float vp[16];            // ViewProj, column-major
  float ox, oy;            // a * s/2, b * s/2: the quad's half extent in clip
                           // space (a, b = projection columns 0 and 1)
  float hw, hh;            // W/2, H/2
  float q;                 // s/4, the discard radius (particleRender.fs:12)
  uint32_t width, height;  // pixels
  uint32_t clear;          // clear colour, RGBA8
};

// Clears keys[W*H], splats the scene's slots [first, first + n) of
// (pos, vel) -- pos.w holds the caller index -- and resolves rgba[W*H] and
// depth[W*H]; colours[n] receives every particle's colour by caller index.
cudaError_t launch_render(uint32_t first, uint32_t n, const float4* pos, const float4* vel,
                          const RenderView& view, unsigned long long* keys,
                          uint32_t* colours, uint32_t* rgba, float* depth,
                          cudaStream_t st);

}  // namespace sph
