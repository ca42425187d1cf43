/*
 * CPU restatement of the reference SPH substep (test infrastructure only).
 *
 * This is the ORACLE: tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg use it as the checker / CPU reference. The product library
 * (libsph_gb300.so) never links, loads or calls it.
 *
 * It restates engine/physics/physicsWorld.cc:39-111 (Update), :304-516
 * (density, pressure, viscosity, spatial lookup, hashing) and
 * engine/physics/kernels.h:25-82 (smoothing kernels) of
 * Allkams/Fluid-Simulation-3D in plain C++ with the same float operation
 * order, so that, given the same sorted bucket order, it reproduces the
 * reference bit for bit in FP32 (pinned by tests/test_oracle_golden.py
 * against fixtures the reference itself, compiled by oracle/Makefile,
 * produced).
 *
 * Contract choices that the reference leaves open:
 *  - sorted order inside a key bucket is canonical: (key asc, index asc);
 *    the reference's std::sort is unstable (physicsWorld.cc:484);
 *  - the float->uint32 cell cast wraps modulo 2^32 ((uint32)(int32)c), the
 *    x86-64 behaviour of physicsWorld.cc:507-509 on every host;
 *  - viscosity is Jacobi (every particle reads the post-pressure velocity
 *    snapshot) unless gauss_seidel != 0, which reproduces the reference's
 *    serial in-place sweep (physicsWorld.cc:430,460,463).
 */
#ifndef SPH_ORACLE_H
#define SPH_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Settings of physicsWorld.h:96-106,145 plus the hard-coded constants of
 * physicsWorld.cc:47 (prediction look-ahead) and :87 (collision damping). */
typedef struct oracle_params {
  float radius;             /* interactionRadius            physicsWorld.h:97 */
  float cutoff_sq;          /* sqrRadius (stale 0.35^2)     physicsWorld.h:96 */
  float target_density;     /* TargetDensity                physicsWorld.h:98 */
  float pressure_mult;      /* pressureMultiplier           physicsWorld.h:99 */
  float near_pressure_mult; /* nearPressureMultiplier       physicsWorld.h:100 */
  float viscosity;          /* viscosityStrength            physicsWorld.h:101 */
  float gravity_scale;      /* gravityScale                 physicsWorld.h:106 */
  int32_t gravity_on;       /* gravity                      physicsWorld.h:105 */
  float bound[3];           /* BoundScale                   physicsWorld.h:145 */
  float damping;            /* dampFactor                   physicsWorld.cc:87 */
  float predict_dt;         /* 1/120 look-ahead             physicsWorld.cc:47 */
} oracle_params;

/* Optional per-substep outputs, all indexed by ORIGINAL particle index
 * except sorted_ids / start. Any pointer may be NULL. */
typedef struct oracle_debug_f32 {
  uint32_t *hash;      /* [n]   HashCell(cell(pred))                  */
  uint32_t *key;       /* [n]   hash % n                              */
  uint32_t *sorted_ids;/* [n]   canonical (key, index) order          */
  uint32_t *start;     /* [n]   startIndices (0x7fffffff = empty)     */
  float *pred;         /* [3n]  predicted positions                   */
  float *dens;         /* [2n]  density, near density                 */
  float *acc_p;        /* [3n]  pressureForce / density               */
  float *vel_p;        /* [3n]  velocity after the pressure pass      */
  float *vel_v;        /* [3n]  velocity after the viscosity pass     */
  float *abs_p;        /* [n]   sum of |pressure terms| / density     */
  float *abs_v;        /* [n]   sum of |viscosity terms| * strength   */
} oracle_debug_f32;

typedef struct oracle_debug_f64 {
  double *dens;   /* [2n] */
  double *acc_p;  /* [3n] */
  double *vel_p;  /* [3n] */
  double *vel_v;  /* [3n] */
} oracle_debug_f64;

/* One substep in FP32 (physicsWorld.cc:39-111). pos/vel are [3n] AoS and are
 * updated in place. Returns 0 on success, negative on bad arguments. */
int sph_oracle_substep_f32(const oracle_params *p, uint32_t n, float *pos,
                           float *vel, float dt, int gauss_seidel,
                           int nthreads, oracle_debug_f32 *dbg);

/* Same substep in FP64 (inputs promoted, grid built from FP64 positions;
 * Jacobi viscosity). */
int sph_oracle_substep_f64(const oracle_params *p, uint32_t n, double *pos,
                           double *vel, double dt, int nthreads,
                           oracle_debug_f64 *dbg);

/* FP64 density / near density and pressure acceleration for a subset of the
 * particles of a scene whose predicted positions `pred` ([3n], FP32) are
 * given: densities of every particle are recomputed in FP64 from the FP32
 * predicted positions (the physics does not depend on the grid), then the
 * pressure acceleration (pressureForce/density, physicsWorld.cc:367-421) is
 * evaluated for the `m` listed particles. out_dens [2m], out_acc [3m],
 * out_abs [m] = sum over neighbours of |pressure term| / density (the scale
 * of the cancelling sum), out_sens [m] = sum over neighbours of the terms'
 * sensitivity to a relative change of the densities (pressure (rho-rho0)*k
 * cancels near rho0, so FP32 rounding of rho moves the terms by about
 * out_sens * 2^-24), out_dsens [m] = sum over neighbours of
 * |d term / d dist| / density (a pair at the edge of the support has a term
 * linear in r - dist, so a rounding of the positions by e moves the
 * acceleration by up to out_dsens * e); any output may be NULL. */
int sph_oracle_subset_f64(const oracle_params *p, uint32_t n, const float *pred,
                          uint32_t m, const uint32_t *subset, int nthreads,
                          double *out_dens, double *out_acc, double *out_abs,
                          double *out_sens, double *out_dsens);

/* FP64 Jacobi viscosity velocity increment (CalculateViscosityForce,
 * physicsWorld.cc:424-464: mu * dt * sum over neighbours j != i of
 * (v_j - v_i) * poly6(dist)) for the `m` listed particles of a scene whose
 * FP32 predicted positions `pred` [3n] and post-pressure velocities `velp`
 * [3n] are given (promoted to FP64; neighbours found by a fresh lookup).
 * out_dv [3m]; out_abs [m] = mu * dt * sum of |term| (the scale of the
 * sum); out_dsens [m] = mu * dt * sum of |d term / d dist| (what a rounding
 * of the positions moves the increment by); any output may be NULL. */
int sph_oracle_subset_visc_f64(const oracle_params *p, uint32_t n, const float *pred,
                               const float *velp, uint32_t m, const uint32_t *subset,
                               double dt, int nthreads, double *out_dv, double *out_abs,
                               double *out_dsens);

/* The headless render of sph_render (sph_render_oracle.cc): pos3/vel3 [3n]
 * in caller order, vp = ViewProj and proj = Projection (column-major),
 * rgba [4 * width * height] and depth [width * height] (either may be
 * NULL), rows bottom to top. */
int sph_oracle_render(const float *pos3, const float *vel3, uint32_t n,
                      const float *vp, const float *proj, uint32_t width,
                      uint32_t height, float scale, const float *clear,
                      uint8_t *rgba, float *depth);

/* The speed normalisation the render's colours use (getSpeedNormalzied,
 * physicsWorld.cc:178-182) of velocities vel3 [3n]: out [n]. */
int sph_oracle_speed_normalized(const float *vel3, uint32_t n, float *out);

/* Number of hardware threads the oracle would use for nthreads <= 0. */
int sph_oracle_hw_threads(void);

#ifdef __cplusplus
}
#endif
#endif
