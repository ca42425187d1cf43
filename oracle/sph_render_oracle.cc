// CPU restatement of the headless particle render -- TEST INFRASTRUCTURE
// ONLY (the product library never links or calls it).
//
// It restates what the reference draws for a frame:
//  - FluidSimCPU::updateColors (projects/Simulation/code/simulations/
//    fluidSimCPU.cc:100-124) over getSpeedNormalzied (engine/physics/
//    physicsWorld.cc:178-182) and the colours of fluidSimCPU.h:26-29;
//  - the billboard splat of bin/shaders/particleRender.vs:32-43 and its
//    circular discard in particleRender.fs:12-13, with the billboard matrix
//    of fluidSimCPU.cc:64-70 (only the projection acts on the offset);
//  - glClearColor / GL_LESS depth testing of gameApp.cc:150,158;
// as a software rasteriser with one fixed float evaluation order (see the
// header of fluid-simulation-3d_gb300/csrc/sph_render.cu, which the GPU
// path follows operation for operation). Built with -ffp-contract=off, so
// every product and sum is rounded as written.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

// getSpeedNormalzied (physicsWorld.cc:178-182): clamp(glm::length(v), 0,
// 1.5) / 1.5, the length as sqrt((x*x + y*y) + z*z).
float SpeedNormalized(float vx, float vy, float vz) {
  const float len = std::sqrt((vx * vx + vy * vy) + vz * vz);
  return std::fmin(std::fmax(len, 0.0f), 1.5f) / 1.5f;
}

uint32_t SpeedColour(float vx, float vy, float vz) {
  const float nrm = SpeedNormalized(vx, vy, vz);
  const float b1 = 0.33f, b2 = 0.66f;
  const float c1[4] = {0.0f, 0.75f, 1.0f, 1.0f};
  const float c2[4] = {0.0f, 1.0f, 0.0f, 1.0f};
  const float c3[4] = {1.0f, 1.0f, 0.0f, 1.0f};
  const float c4[4] = {1.0f, 0.0f, 0.0f, 1.0f};
  float t;
  const float *lo, *hi;
  if (nrm <= b1) {
    t = nrm / b1;
    lo = c1;
    hi = c2;
  } else if (nrm <= b2) {
    t = (nrm - b1) / (b2 - b1);
    lo = c2;
    hi = c3;
  } else {
    t = (nrm - b2) / (1.0f - b2);
    lo = c3;
    hi = c4;
  }
  const float u = 1.0f - t;
  uint32_t out = 0;
  for (int k = 0; k < 4; ++k) {
    const float c = u * lo[k] + t * hi[k];
    const float b = std::fmin(std::fmax(c, 0.0f), 1.0f) * 255.0f;
    out |= static_cast<uint32_t>(std::lrint(b)) << (8 * k);
  }
  return out;
}

float RowDot(const float* m, int r, float x, float y, float z) {
  return (m[r] * x + m[4 + r] * y) + (m[8 + r] * z + m[12 + r]);
}

}  // namespace

extern "C" {

/* pos3/vel3 [3n] in caller order; vp, proj column-major; rgba [4*W*H],
 * depth [W*H] (either may be NULL), rows bottom to top. Returns 0, or -1 on
 * bad arguments. */
int sph_oracle_render(const float* pos3, const float* vel3, uint32_t n, const float* vp,
                      const float* proj, uint32_t width, uint32_t height, float scale,
                      const float* clear, uint8_t* rgba, float* depth) {
  if (!pos3 || !vel3 || !vp || !proj || !clear || width == 0 || height == 0) return -1;
  const uint64_t pixels = static_cast<uint64_t>(width) * height;
  std::vector<uint64_t> keys(pixels, ~0ull);
  std::vector<uint32_t> colour(n);
  const float hs = 0.5f * scale;
  const float ox = proj[0] * hs, oy = proj[5] * hs;
  const float hw = 0.5f * static_cast<float>(width);
  const float hh = 0.5f * static_cast<float>(height);
  const float q = scale * 0.25f;
  const float fw = static_cast<float>(width), fh = static_cast<float>(height);
  for (uint32_t id = 0; id < n; ++id) {
    const float* p = pos3 + 3ull * id;
    const float* v = vel3 + 3ull * id;
    colour[id] = SpeedColour(v[0], v[1], v[2]);
    const float cx = RowDot(vp, 0, p[0], p[1], p[2]);
    const float cy = RowDot(vp, 1, p[0], p[1], p[2]);
    const float cz = RowDot(vp, 2, p[0], p[1], p[2]);
    const float cw = RowDot(vp, 3, p[0], p[1], p[2]);
    if (!(cw > 0.0f) || !(cz >= -cw && cz <= cw)) continue;
    const float x0 = ((cx - ox) / cw) * hw + hw;
    const float x1 = ((cx + ox) / cw) * hw + hw;
    const float y0 = ((cy - oy) / cw) * hh + hh;
    const float y1 = ((cy + oy) / cw) * hh + hh;
    if (!(x1 > x0) || !(y1 > y0)) continue;
    const float dep = (cz / cw) * 0.5f + 0.5f;
    const int px0 = static_cast<int>(std::ceil(std::fmin(std::fmax(x0 - 0.5f, -1.0f), fw)));
    const int px1 = static_cast<int>(std::ceil(std::fmin(std::fmax(x1 - 0.5f, -1.0f), fw))) - 1;
    const int py0 = static_cast<int>(std::floor(std::fmin(std::fmax(y0 - 0.5f, -1.0f), fh))) + 1;
    const int py1 = static_cast<int>(std::floor(std::fmin(std::fmax(y1 - 0.5f, -1.0f), fh)));
    const int xa = std::max(px0, 0), xb = std::min(px1, static_cast<int>(width) - 1);
    const int ya = std::max(py0, 0), yb = std::min(py1, static_cast<int>(height) - 1);
    if (xa > xb || ya > yb) continue;
    const float idx = 1.0f / (x1 - x0), idy = 1.0f / (y1 - y0);
    const float two_ox = ox + ox, two_oy = oy + oy;
    const float q2 = q * q;
    uint32_t dbits;
    std::memcpy(&dbits, &dep, 4);
    const uint64_t key = (static_cast<uint64_t>(dbits) << 32) | id;
    for (int py = ya; py <= yb; ++py) {
      const float fy = ((static_cast<float>(py) + 0.5f) - y0) * idy;
      const float vyy = fy * two_oy - oy;
      const float vy2 = vyy * vyy;
      for (int px = xa; px <= xb; ++px) {
        const float fx = ((static_cast<float>(px) + 0.5f) - x0) * idx;
        const float vxx = fx * two_ox - ox;
        if (vxx * vxx + vy2 > q2) continue;  // discard: |offset| > s/4
        uint64_t& k = keys[static_cast<uint64_t>(py) * width + px];
        if (key < k) k = key;
      }
    }
  }
  uint32_t clear8 = 0;
  for (int k = 0; k < 4; ++k) {
    const float c = std::fmin(std::fmax(clear[k], 0.0f), 1.0f) * 255.0f;
    clear8 |= static_cast<uint32_t>(std::lrint(c)) << (8 * k);
  }
  for (uint64_t i = 0; i < pixels; ++i) {
    uint32_t c = clear8;
    float d = 1.0f;
    if (keys[i] != ~0ull) {
      c = colour[static_cast<uint32_t>(keys[i])];
      const uint32_t bits = static_cast<uint32_t>(keys[i] >> 32);
      std::memcpy(&d, &bits, 4);
    }
    if (rgba)
      for (int k = 0; k < 4; ++k) rgba[4 * i + k] = static_cast<uint8_t>(c >> (8 * k));
    if (depth) depth[i] = d;
  }
  return 0;
}

}  // extern "C"

extern "C" int sph_oracle_speed_normalized(const float* vel3, uint32_t n, float* out) {
  if (!vel3 || !out) return -1;
  for (uint32_t i = 0; i < n; ++i)
    out[i] = SpeedNormalized(vel3[3 * i], vel3[3 * i + 1], vel3[3 * i + 2]);
  return 0;
}
