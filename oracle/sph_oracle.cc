// CPU restatement of the reference SPH substep -- test infrastructure only.
//
// This file is the ORACLE. Only tests/, __graft_entry__.smoke() and the CPU
// baseline leg of bench.py load it; the product library never does.
//
// Every function cites the reference file:line it restates
// (Allkams/Fluid-Simulation-3D). FP32 code keeps the reference's operation
// order (glm component-wise vector ops, no FMA contraction: build with
// -ffp-contract=off) so that with the same bucket order it matches the
// reference bit for bit.
#include "sph_oracle.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>

namespace {

// glm::pi<float>() / glm::pi<double>() (exts/glm/gtc/constants.inl).
template <typename T> constexpr T kPi() {
  return static_cast<T>(3.14159265358979323846264338327950288);
}

// Hash multipliers of HashCell (physicsWorld.cc:507-509).
constexpr uint32_t kHashX = 15823u;
constexpr uint32_t kHashY = 9737333u;
constexpr uint32_t kHashZ = 440817757u;

// Neighbour offsets in the reference's table order (physicsWorld.h:131-143):
// dx outermost, dz innermost.
struct Off { int x, y, z; };
static const Off kOffsets[27] = {
    {-1, -1, -1}, {-1, -1, 0}, {-1, -1, 1}, {-1, 0, -1}, {-1, 0, 0}, {-1, 0, 1},
    {-1, 1, -1},  {-1, 1, 0},  {-1, 1, 1},  {0, -1, -1}, {0, -1, 0}, {0, -1, 1},
    {0, 0, -1},   {0, 0, 0},   {0, 0, 1},   {0, 1, -1},  {0, 1, 0},  {0, 1, 1},
    {1, -1, -1},  {1, -1, 0},  {1, -1, 1},  {1, 0, -1},  {1, 0, 0},  {1, 0, 1},
    {1, 1, -1},   {1, 1, 0},   {1, 1, 1}};

inline float Pow(float x, float e) { return powf(x, e); }
inline double Pow(double x, double e) { return std::pow(x, e); }

// Smoothing-kernel constants, same expressions as kernels.h:28,40,52,64,76
// (the `abs` of kernels.h:77 taken as the float overload, i.e. |r|).
template <typename T> struct KernelConsts {
  T r;
  T vol2;    // 15 / (2*pi*r^5)             kernels.h:28
  T vol3;    // 15 / (pi*r^6)               kernels.h:40
  T dscale2; // 15 / (r^5*pi)               kernels.h:52
  T dscale3; // 45 / (r^6*pi)               kernels.h:64
  T vscale;  // 315 / (64*pi*|r|^9)         kernels.h:76
  explicit KernelConsts(T radius) : r(radius) {
    const T pi = kPi<T>();
    vol2 = T(15) / (T(2) * pi * Pow(r, T(5)));
    vol3 = T(15) / (pi * Pow(r, T(6)));
    dscale2 = T(15) / (Pow(r, T(5)) * pi);
    dscale3 = T(45) / (Pow(r, T(6)) * pi);
    vscale = T(315) / (T(64) * pi * Pow(std::fabs(r), T(9)));
  }
  // SmoothingPow2, kernels.h:25-34
  T pow2(T dist) const {
    if (dist < r) { T v = r - dist; return v * v * vol2; }
    return 0;
  }
  // SmoothingPow3, kernels.h:37-46
  T pow3(T dist) const {
    if (dist < r) { T v = r - dist; return v * v * v * vol3; }
    return 0;
  }
  // SmoothingDerivativePow2, kernels.h:49-58
  T dpow2(T dist) const {
    if (dist <= r) { T v = r - dist; return -v * dscale2; }
    return 0;
  }
  // SmoothingDerivativePow3, kernels.h:61-70
  T dpow3(T dist) const {
    if (dist <= r) { T v = r - dist; return -v * v * dscale3; }
    return 0;
  }
  // SmoothingViscoPoly6, kernels.h:73-82
  T poly6(T dist) const {
    if (dist < r) { T v = r * r - dist * dist; return v * v * v * vscale; }
    return 0;
  }
};

// glm dot(vec3, vec3): tmp = a*b; tmp.x + tmp.y + tmp.z (func_geometric.inl).
template <typename T> inline T Dot3(T x, T y, T z) {
  T tx = x * x, ty = y * y, tz = z * z;
  return tx + ty + tz;
}

// PositionToCellCoord, physicsWorld.cc:499-503: floor(pos / r), then (int).
template <typename T> inline int32_t CellCoord(T p, T r) {
  return static_cast<int32_t>(std::floor(p / r));
}

// HashCell, physicsWorld.cc:505-511, with the float->uint32 cast taken as the
// x86-64 wrap (uint32)(int32)c on every host.
inline uint32_t HashCell(int32_t cx, int32_t cy, int32_t cz) {
  uint32_t a = static_cast<uint32_t>(cx) * kHashX;
  uint32_t b = static_cast<uint32_t>(cy) * kHashY;
  uint32_t c = static_cast<uint32_t>(cz) * kHashZ;
  return a + b + c;
}

int HwThreads() {
  unsigned h = std::thread::hardware_concurrency();
  return h == 0 ? 1 : static_cast<int>(h);
}

// Static-chunked parallel loop over [0, n) (stands in for
// std::for_each(std::execution::par, ...) of physicsWorld.cc:42,63,72,81,306).
template <typename F> void ParallelFor(uint32_t n, int nthreads, F&& f) {
  if (nthreads <= 0) nthreads = HwThreads();
  if (nthreads == 1 || n < 4096) {
    for (uint32_t i = 0; i < n; ++i) f(i);
    return;
  }
  std::vector<std::thread> pool;
  const uint32_t chunk = (n + nthreads - 1) / nthreads;
  for (int t = 0; t < nthreads; ++t) {
    uint32_t b = static_cast<uint32_t>(t) * chunk;
    uint32_t e = std::min<uint32_t>(n, b + chunk);
    if (b >= e) break;
    pool.emplace_back([b, e, &f] { for (uint32_t i = b; i < e; ++i) f(i); });
  }
  for (auto& th : pool) th.join();
}

// Spatial lookup of UpdateSpatialLookup, physicsWorld.cc:466-498, with the
// canonical (key asc, index asc) order in place of the unstable std::sort.
struct Lookup {
  std::vector<uint32_t> id, hash, key;  // sorted entries {index, hash, key}
  std::vector<uint32_t> start;          // startIndices, 0x7fffffff = empty
};

template <typename T>
void BuildLookup(const T* pred, uint32_t n, T r, int nthreads, Lookup& L,
                 std::vector<uint32_t>& hashOf, std::vector<uint32_t>& keyOf) {
  hashOf.resize(n);
  keyOf.resize(n);
  ParallelFor(n, nthreads, [&](uint32_t i) {
    int32_t cx = CellCoord(pred[3 * i + 0], r);
    int32_t cy = CellCoord(pred[3 * i + 1], r);
    int32_t cz = CellCoord(pred[3 * i + 2], r);
    uint32_t h = HashCell(cx, cy, cz);
    hashOf[i] = h;
    keyOf[i] = h % n;  // GetKeyFromHash, physicsWorld.cc:513-516
  });
  // Stable counting sort by key (key < n).
  std::vector<uint32_t> count(static_cast<size_t>(n) + 1, 0);
  for (uint32_t i = 0; i < n; ++i) count[keyOf[i] + 1]++;
  for (uint32_t k = 0; k < n; ++k) count[k + 1] += count[k];
  L.id.assign(n, 0);
  L.hash.assign(n, 0);
  L.key.assign(n, 0);
  L.start.assign(n, 0x7fffffffu);  // startIndices[i] = INT_MAX, :481
  std::vector<uint32_t> fill(count.begin(), count.end() - 1);
  for (uint32_t i = 0; i < n; ++i) {
    uint32_t s = fill[keyOf[i]]++;
    L.id[s] = i;
    L.hash[s] = hashOf[i];
    L.key[s] = keyOf[i];
  }
  // startIndices[key] = first sorted index of key, :486-496
  for (uint32_t s = 0; s < n; ++s)
    if (s == 0 || L.key[s] != L.key[s - 1]) L.start[L.key[s]] = s;
}

// Walk of the 27 neighbour buckets shared by CalculateDensity (:331-363),
// CalculatePressureForce (:378-419) and CalculateViscosityForce (:432-462):
// scan from startIndices[key] until the key changes, skip entries whose
// float(hash) differs from the cell's (the lookup stores floats, :480).
template <typename T, typename F>
inline void ForNeighbours(const Lookup& L, uint32_t n, T r, const T* p,
                          F&& visit) {
  const int32_t cx = CellCoord(p[0], r), cy = CellCoord(p[1], r),
                cz = CellCoord(p[2], r);
  for (int o = 0; o < 27; ++o) {
    uint32_t hash = HashCell(cx + kOffsets[o].x, cy + kOffsets[o].y,
                             cz + kOffsets[o].z);
    uint32_t key = hash % n;
    const float hashF = static_cast<float>(hash);
    uint32_t cur = L.start[key];
    while (cur < n) {
      uint32_t s = cur++;
      if (L.key[s] != key) break;
      if (static_cast<float>(L.hash[s]) != hashF) continue;
      visit(L.id[s]);
    }
  }
}

template <typename T> struct Settings {
  T r, cut2, rho0, k, kn, mu, gy, hx, hy, hz, damp, pdt;
  explicit Settings(const oracle_params* p) {
    r = static_cast<T>(p->radius);
    cut2 = static_cast<T>(p->cutoff_sq);
    rho0 = static_cast<T>(p->target_density);
    k = static_cast<T>(p->pressure_mult);
    kn = static_cast<T>(p->near_pressure_mult);
    mu = static_cast<T>(p->viscosity);
    // CalculateExternalFoce, physicsWorld.cc:313-323
    gy = p->gravity_on ? -static_cast<T>(p->gravity_scale) : T(0);
    // halfSize = BoundScale * 0.5f, physicsWorld.cc:88
    hx = static_cast<T>(p->bound[0]) * T(0.5);
    hy = static_cast<T>(p->bound[1]) * T(0.5);
    hz = static_cast<T>(p->bound[2]) * T(0.5);
    damp = static_cast<T>(p->damping);
    pdt = static_cast<T>(p->predict_dt);
  }
};

template <typename T> inline T Sign(T x) {
  return static_cast<T>(T(0) < x) - static_cast<T>(x < T(0));
}

// One substep: physicsWorld.cc:39-111 with a canonical lookup order and,
// unless gs, Jacobi viscosity.
template <typename T>
void Substep(const oracle_params* prm, uint32_t n, T* pos, T* vel, T dt,
             bool gs, int nthreads, uint32_t* oHash, uint32_t* oKey,
             uint32_t* oSorted, uint32_t* oStart, T* oPred, T* oDens,
             T* oAccP, T* oVelP, T* oVelV, T* oAbsP, T* oAbsV) {
  const Settings<T> S(prm);
  const KernelConsts<T> K(S.r);
  std::vector<T> pred(3 * static_cast<size_t>(n));
  std::vector<T> dens(2 * static_cast<size_t>(n));

  // 1. External force + prediction, :42-48.
  ParallelFor(n, nthreads, [&](uint32_t i) {
    T gx = T(0) * dt, gyv = S.gy * dt, gz = T(0) * dt;
    vel[3 * i + 0] = vel[3 * i + 0] + gx;
    vel[3 * i + 1] = vel[3 * i + 1] + gyv;
    vel[3 * i + 2] = vel[3 * i + 2] + gz;
    for (int c = 0; c < 3; ++c)
      pred[3 * i + c] = pos[3 * i + c] + vel[3 * i + c] * S.pdt;
  });

  // 2. Spatial lookup, :466-498.
  Lookup L;
  std::vector<uint32_t> hashOf, keyOf;
  BuildLookup(pred.data(), n, S.r, nthreads, L, hashOf, keyOf);

  // 3. Densities, :304-311 and CalculateDensity :325-365 (self included).
  ParallelFor(n, nthreads, [&](uint32_t i) {
    const T* p = &pred[3 * i];
    T d = 0, nd = 0;
    ForNeighbours(L, n, S.r, p, [&](uint32_t j) {
      const T* q = &pred[3 * j];
      T ox = q[0] - p[0], oy = q[1] - p[1], oz = q[2] - p[2];
      T sq = Dot3(ox, oy, oz);
      if (sq > S.cut2) return;
      T dist = std::sqrt(sq);
      d += K.pow2(dist);
      nd += K.pow3(dist);
    });
    dens[2 * i + 0] = d;
    dens[2 * i + 1] = nd;
  });

  // 4. Pressure force, CalculatePressureForce :367-422 (self skipped).
  ParallelFor(n, nthreads, [&](uint32_t i) {
    const T density = dens[2 * i + 0];
    const T nearDensity = dens[2 * i + 1];
    const T pressure = (density - S.rho0) * S.k;
    const T nearPressure = nearDensity * S.kn;
    T fx = 0, fy = 0, fz = 0;
    double absSum = 0.0;
    const T* p = &pred[3 * i];
    ForNeighbours(L, n, S.r, p, [&](uint32_t j) {
      if (j == i) return;
      const T* q = &pred[3 * j];
      T ox = q[0] - p[0], oy = q[1] - p[1], oz = q[2] - p[2];
      T sq = Dot3(ox, oy, oz);
      if (sq > S.cut2) return;
      const T nbD = dens[2 * j + 0];
      const T nbND = dens[2 * j + 1];
      const T nbP = (nbD - S.rho0) * S.k;
      const T nbNP = nbND * S.kn;
      const T sharedP = (pressure + nbP) * T(0.5);
      const T sharedNP = (nearPressure + nbNP) * T(0.5);
      const T dist = std::sqrt(sq);
      T dx, dy, dz;
      if (dist > 0) { dx = ox / dist; dy = oy / dist; dz = oz / dist; }
      else { dx = 0; dy = 1; dz = 0; }
      const T k2 = K.dpow2(dist), k3 = K.dpow3(dist);
      // dir * k2 * shared / nbD, component-wise in glm's order (:416)
      T ax = dx * k2 * sharedP / nbD, ay = dy * k2 * sharedP / nbD,
        az = dz * k2 * sharedP / nbD;
      fx += ax; fy += ay; fz += az;
      T bx = dx * k3 * sharedNP / nbND, by = dy * k3 * sharedNP / nbND,
        bz = dz * k3 * sharedNP / nbND;  // :417
      fx += bx; fy += by; fz += bz;
      absSum += std::sqrt(double(ax) * ax + double(ay) * ay + double(az) * az) +
                std::sqrt(double(bx) * bx + double(by) * by + double(bz) * bz);
    });
    // velocity += (pressureForce / density) * deltatime, :421
    const T apx = fx / density, apy = fy / density, apz = fz / density;
    if (oAccP) { oAccP[3 * i] = apx; oAccP[3 * i + 1] = apy; oAccP[3 * i + 2] = apz; }
    if (oAbsP) oAbsP[i] = static_cast<T>(absSum / std::fabs(double(density)));
    vel[3 * i + 0] = vel[3 * i + 0] + apx * dt;
    vel[3 * i + 1] = vel[3 * i + 1] + apy * dt;
    vel[3 * i + 2] = vel[3 * i + 2] + apz * dt;
  });
  if (oVelP) std::memcpy(oVelP, vel, sizeof(T) * 3 * n);

  // 5. Viscosity, CalculateViscosityForce :424-464. Jacobi reads the
  //    post-pressure snapshot; gs reproduces the serial in-place sweep.
  auto viscOne = [&](uint32_t i, const T* vsrc, T* vdst) {
    const T* p = &pred[3 * i];
    const T vix = vsrc[3 * i], viy = vsrc[3 * i + 1], viz = vsrc[3 * i + 2];
    T fx = 0, fy = 0, fz = 0;
    double absSum = 0.0;
    ForNeighbours(L, n, S.r, p, [&](uint32_t j) {
      if (j == i) return;
      const T* q = &pred[3 * j];
      T ox = q[0] - p[0], oy = q[1] - p[1], oz = q[2] - p[2];
      T sq = Dot3(ox, oy, oz);
      if (sq > S.cut2) return;
      const T dist = std::sqrt(sq);
      const T infl = K.poly6(dist);
      T tx = (vsrc[3 * j] - vix) * infl, ty = (vsrc[3 * j + 1] - viy) * infl,
        tz = (vsrc[3 * j + 2] - viz) * infl;
      fx += tx; fy += ty; fz += tz;
      absSum += std::sqrt(double(tx) * tx + double(ty) * ty + double(tz) * tz);
    });
    // velocity += viscosityForce * viscosityStrength * deltatime, :463
    vdst[3 * i + 0] = vix + fx * S.mu * dt;
    vdst[3 * i + 1] = viy + fy * S.mu * dt;
    vdst[3 * i + 2] = viz + fz * S.mu * dt;
    if (oAbsV) oAbsV[i] = static_cast<T>(absSum * std::fabs(double(S.mu)));
  };
  if (gs) {
    for (uint32_t i = 0; i < n; ++i) viscOne(i, vel, vel);
  } else {
    std::vector<T> snap(vel, vel + 3 * static_cast<size_t>(n));
    ParallelFor(n, nthreads, [&](uint32_t i) { viscOne(i, snap.data(), vel); });
  }
  if (oVelV) std::memcpy(oVelV, vel, sizeof(T) * 3 * n);

  // 6. Integrate and box collision, :81-108.
  ParallelFor(n, nthreads, [&](uint32_t i) {
    T* x = &pos[3 * i];
    T* v = &vel[3 * i];
    const T half[3] = {S.hx, S.hy, S.hz};
    for (int c = 0; c < 3; ++c) x[c] = x[c] + v[c] * dt;
    for (int c = 0; c < 3; ++c) {
      T edge = half[c] - std::fabs(x[c]);
      if (edge <= 0) {
        x[c] = half[c] * Sign(x[c]);
        v[c] *= -S.damp;  // velocity *= -1 * dampFactor, :94
      }
    }
  });

  if (oHash) std::memcpy(oHash, hashOf.data(), sizeof(uint32_t) * n);
  if (oKey) std::memcpy(oKey, keyOf.data(), sizeof(uint32_t) * n);
  if (oSorted) std::memcpy(oSorted, L.id.data(), sizeof(uint32_t) * n);
  if (oStart) std::memcpy(oStart, L.start.data(), sizeof(uint32_t) * n);
  if (oPred) std::memcpy(oPred, pred.data(), sizeof(T) * 3 * n);
  if (oDens) std::memcpy(oDens, dens.data(), sizeof(T) * 2 * n);
}

bool ParamsOk(const oracle_params* p, uint32_t n) {
  return p != nullptr && n > 0 && n < (1u << 24) && p->radius > 0.0f;
}

}  // namespace

extern "C" {

int sph_oracle_hw_threads(void) { return HwThreads(); }

int sph_oracle_substep_f32(const oracle_params* p, uint32_t n, float* pos,
                           float* vel, float dt, int gauss_seidel,
                           int nthreads, oracle_debug_f32* d) {
  if (!ParamsOk(p, n) || !pos || !vel) return -1;
  oracle_debug_f32 z{};
  if (!d) d = &z;
  Substep<float>(p, n, pos, vel, dt, gauss_seidel != 0, nthreads, d->hash,
                 d->key, d->sorted_ids, d->start, d->pred, d->dens, d->acc_p,
                 d->vel_p, d->vel_v, d->abs_p, d->abs_v);
  return 0;
}

int sph_oracle_substep_f64(const oracle_params* p, uint32_t n, double* pos,
                           double* vel, double dt, int nthreads,
                           oracle_debug_f64* d) {
  if (!ParamsOk(p, n) || !pos || !vel) return -1;
  oracle_debug_f64 z{};
  if (!d) d = &z;
  Substep<double>(p, n, pos, vel, dt, false, nthreads, nullptr, nullptr,
                  nullptr, nullptr, nullptr, d->dens, d->acc_p, d->vel_p,
                  d->vel_v, nullptr, nullptr);
  return 0;
}

int sph_oracle_subset_f64(const oracle_params* p, uint32_t n, const float* pred,
                          uint32_t m, const uint32_t* subset, int nthreads,
                          double* out_dens, double* out_acc, double* out_abs,
                          double* out_sens, double* out_dsens) {
  if (!ParamsOk(p, n) || !pred || (m && !subset)) return -1;
  for (uint32_t t = 0; t < m; ++t)
    if (subset[t] >= n) return -2;
  const Settings<double> S(p);
  const KernelConsts<double> K(S.r);
  std::vector<double> pd(pred, pred + 3 * static_cast<size_t>(n));
  Lookup L;
  std::vector<uint32_t> hashOf, keyOf;
  BuildLookup(pd.data(), n, S.r, nthreads, L, hashOf, keyOf);
  std::vector<double> dens(2 * static_cast<size_t>(n));
  ParallelFor(n, nthreads, [&](uint32_t i) {
    const double* q0 = &pd[3 * i];
    double d = 0, nd = 0;
    ForNeighbours(L, n, S.r, q0, [&](uint32_t j) {
      const double* q = &pd[3 * j];
      double sq = Dot3(q[0] - q0[0], q[1] - q0[1], q[2] - q0[2]);
      if (sq > S.cut2) return;
      double dist = std::sqrt(sq);
      d += K.pow2(dist);
      nd += K.pow3(dist);
    });
    dens[2 * i] = d;
    dens[2 * i + 1] = nd;
  });
  ParallelFor(m, nthreads, [&](uint32_t t) {
    const uint32_t i = subset[t];
    const double* q0 = &pd[3 * i];
    const double density = dens[2 * i], nearDensity = dens[2 * i + 1];
    const double pressure = (density - S.rho0) * S.k;
    const double nearPressure = nearDensity * S.kn;
    double fx = 0, fy = 0, fz = 0, absSum = 0, sens = 0, dsens = 0;
    ForNeighbours(L, n, S.r, q0, [&](uint32_t j) {
      if (j == i) return;
      const double* q = &pd[3 * j];
      double ox = q[0] - q0[0], oy = q[1] - q0[1], oz = q[2] - q0[2];
      double sq = Dot3(ox, oy, oz);
      if (sq > S.cut2) return;
      double dist = std::sqrt(sq);
      double dx = 0, dy = 1, dz = 0;
      if (dist > 0) { dx = ox / dist; dy = oy / dist; dz = oz / dist; }
      double sp = (pressure + (dens[2 * j] - S.rho0) * S.k) * 0.5;
      double snp = (nearPressure + dens[2 * j + 1] * S.kn) * 0.5;
      double a = K.dpow2(dist) * sp / dens[2 * j];
      double b = K.dpow3(dist) * snp / dens[2 * j + 1];
      fx += dx * (a + b); fy += dy * (a + b); fz += dz * (a + b);
      absSum += std::fabs(a) + std::fabs(b);
      // d(term)/d(log rho) for rho_i and rho_j: what an FP32 rounding of
      // the densities moves the term by, (rho - rho0) * k cancelling
      sens += std::fabs(K.dpow2(dist)) * 0.5 * S.k *
              (dens[2 * i] + dens[2 * j]) / dens[2 * j];
      // d(term)/d(dist): what a rounding of the positions moves the term by
      // (a pair at the edge of the support has a term linear in r - dist)
      if (dist <= S.r)
        dsens += K.dscale2 * std::fabs(sp / dens[2 * j]) +
                 2.0 * (S.r - dist) * K.dscale3 * std::fabs(snp / dens[2 * j + 1]);
    });
    if (out_abs) out_abs[t] = absSum / std::fabs(density);
    if (out_sens) out_sens[t] = sens / std::fabs(density);
    if (out_dsens) out_dsens[t] = dsens / std::fabs(density);
    if (out_dens) { out_dens[2 * t] = density; out_dens[2 * t + 1] = nearDensity; }
    if (out_acc) {
      out_acc[3 * t] = fx / density;
      out_acc[3 * t + 1] = fy / density;
      out_acc[3 * t + 2] = fz / density;
    }
  });
  return 0;
}

int sph_oracle_subset_visc_f64(const oracle_params* p, uint32_t n, const float* pred,
                               const float* velp, uint32_t m, const uint32_t* subset,
                               double dt, int nthreads, double* out_dv, double* out_abs,
                               double* out_dsens) {
  if (!ParamsOk(p, n) || !pred || !velp || (m && !subset)) return -1;
  for (uint32_t t = 0; t < m; ++t)
    if (subset[t] >= n) return -2;
  const Settings<double> S(p);
  const KernelConsts<double> K(S.r);
  std::vector<double> pd(pred, pred + 3 * static_cast<size_t>(n));
  Lookup L;
  std::vector<uint32_t> hashOf, keyOf;
  BuildLookup(pd.data(), n, S.r, nthreads, L, hashOf, keyOf);
  const double c = S.mu * dt;
  ParallelFor(m, nthreads, [&](uint32_t t) {
    const uint32_t i = subset[t];
    const double* q0 = &pd[3 * i];
    const double vix = velp[3 * i], viy = velp[3 * i + 1], viz = velp[3 * i + 2];
    double fx = 0, fy = 0, fz = 0, absSum = 0, dsens = 0;
    // CalculateViscosityForce, physicsWorld.cc:424-464, reading the
    // post-pressure snapshot of every neighbour (Jacobi)
    ForNeighbours(L, n, S.r, q0, [&](uint32_t j) {
      if (j == i) return;
      const double* q = &pd[3 * j];
      const double sq = Dot3(q[0] - q0[0], q[1] - q0[1], q[2] - q0[2]);
      if (sq > S.cut2) return;
      const double infl = K.poly6(std::sqrt(sq));
      const double ux = velp[3 * j] - vix, uy = velp[3 * j + 1] - viy,
                   uz = velp[3 * j + 2] - viz;
      fx += ux * infl; fy += uy * infl; fz += uz * infl;
      const double du = std::sqrt(ux * ux + uy * uy + uz * uz);
      absSum += du * infl;
      // |d infl / d dist| = 6 dist (r^2 - dist^2)^2 * scale inside the support
      if (sq < S.r * S.r) {
        const double w = S.r * S.r - sq;
        dsens += du * 6.0 * std::sqrt(sq) * w * w * K.vscale;
      }
    });
    if (out_dv) {
      out_dv[3 * t] = fx * c;
      out_dv[3 * t + 1] = fy * c;
      out_dv[3 * t + 2] = fz * c;
    }
    if (out_abs) out_abs[t] = absSum * std::fabs(c);
    if (out_dsens) out_dsens[t] = dsens * std::fabs(c);
  });
  return 0;
}

}  // extern "C"
