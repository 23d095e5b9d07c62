// common.cuh -- shared device-side types and helpers of the GB300 ensemble tracer.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/rapt_gpu.h"

namespace rapt {

// Physical constants, rapt/__init__.py:5-10.
constexpr double kC = 299792458.0;
constexpr double kB0 = 3.07e-5;
constexpr double kRe = 6378137.0;
constexpr double kPi = 3.141592653589793;
constexpr double kRe3 = kRe * kRe * kRe;

constexpr unsigned kFull = 0xffffffffu;

// Field model parameters as seen by the kernels (passed by value: they live in
// the kernel-parameter constant bank, uniform across the grid).
struct FieldP {
  int model;
  int is_static;      // _Field.static
  double p[8];        // constructor parameters
  double gradstep;    // _Field.gradientstepsize
  double timestep;    // _Field.timederivstepsize
  double inv2d;       // 1 / (2 gradstep)
  double c0, c1, c2;  // model constants precomputed on the host
  float dh[4], dl[4]; // float-float model constants (hi, lo) for the FP32 form
  // FP32 form, dipole models in units of L = 2^22 m with B = c F(r): the stencil
  // step d / L, the second dipole's position (m) and strength, |c|, and the
  // quotients |c| / (2 d) and sign(c) / (2 d) of the realised step, as
  // float-float (hi, lo) pairs
  float sd, sxh, sxl, skh, skl, cah, cal, sgh, sgl, sch, scl;
  // RAPT_GRID: axes and [nt][nx][ny][nz][3] snapshots resident on the device
  const double *gt, *gx, *gy, *gz;
  const double *gB, *gE;  // gE null: zero electric field
  double ginv[4];         // (n - 1) / (g[n-1] - g[0]) per axis (t, x, y, z): the cell guess
  int nt, nx, ny, nz;
};

// rapt.params plus device options, resolved on the host.
struct KParams {
  FieldP f;
  double rtol, atol, cycres, gctimestep, epss, epst;
  double rkf_tol, rkf_hmin;
  int enforce_eq, tableau, gc_eom, nsteps, kind, form;
  long long budget;        // RK step attempts per thread per launch
  int max_rows, max_sw;    // per-tracer output capacity
  int max_segments;        // Adaptive: cap on advance() calls per tracer
  // step-size MLP (learned forms) and training-sample collection
  const uint32_t* mlp_w;   // packed BF16 weights
  const float* mlp_p;      // FP32 biases and normalisation
  float learn_scale;       // multiplier on the learned step proposal
  float* samp;             // [samp_cap][18] collected samples
  unsigned long long* samp_count;
  long long samp_cap;
  unsigned long long samp_mask;  // an accepted step is sampled when its hash & mask == 0
  int collect;             // learned kernels: also record samples (on-policy data)
  int learn_every;         // run the MLP on every k-th accepted step, reuse its correction between
  // bounce-period cadence (gctimestep == 0): per-thread field-line scratch
  double bounceres, flres; // params["bounceresolution"], params["fieldlineresolution"]
  double* fl_scratch;      // fl_stride doubles per thread of the launch
  long long fl_stride;
  int fl_cap;              // trace points per direction
};

// Device SoA ensemble (all arrays length n unless noted).
struct DevEnsemble {
  int64_t n;
  int8_t* mode;
  int32_t* status;
  int32_t* flags;
  double* t_int;     // integrator time r.t
  double* t_row;     // time of the last trajectory row
  double* tcur;
  double* s[6];
  double* mu;
  double* v;
  double* mass;
  double* charge;
  int64_t* naccept;
  int64_t* nreject;
  int64_t* nfcn;
  int32_t* nswitch;
  // per-call advance bookkeeping
  double* delta;       // the delta of this call (Particle/GC advance, or Adaptive delta)
  double* seg_stop;    // t0 + delta of the current tracer.advance() call
  double* seg_dt;      // output cadence of the current call
  double* seg_gm;      // gamma*m frozen at the start of a Particle.advance call
  // dense-output guiding-centre integration carried between steps and launches:
  // step size (0: not started), facold, steps since the last row
  double* carry_h;
  double* carry_fac;
  double* carry_nst;
  int8_t* seg_active;  // 1 while a tracer.advance() call is in progress
  int32_t* nseg;       // advance() calls made by Adaptive in this call
  // outputs
  double* rows;        // [n][max_rows][7]
  int8_t* row_mode;    // [n][max_rows]
  int32_t* nrows;
  double* sw_time;     // [n][max_sw]
  int8_t* sw_mode;     // [n][max_sw]
  // work-queue order: queue position q hands out tracer order[q] (a permutation,
  // longest expected work first); null: index order
  const int32_t* order;
};

// Scratch words used by the persistent kernels (one block of device memory).
struct Scratch {
  unsigned long long queue[2];   // work-queue heads (particle kernel, GC kernel)
  unsigned long long pending;    // tracers left unfinished by the last launch pair
  unsigned long long accepted, rejected, rhs, switches, done, failed;
};

// FP64 reciprocal and square root for quantities that need about 14 digits
// (error norms, tolerance scales): the FP32 approximation (one MUFU
// instruction) refined by one Newton-Raphson step in FP64, which squares its
// relative error (2^-23 -> ~1e-14). Each costs 2-4 FP64-pipe instructions where
// the correctly rounded FP64 division or square root costs several more, and
// GB300 issues FP64 at 1/64 of the FP32 rate. Arguments outside the FP32
// normal range fall back to the IEEE operation.
__device__ __forceinline__ float rcp_approx_f32(float x) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float rsqrt_approx_f32(float x) {
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
// (The range tests are made on the FP32 value the seed needs anyway: FP32
// compares leave the FP64 pipe alone.)
__device__ __forceinline__ double rcp_nr(double x) {
  const float xf = (float)x;
  if (!(fabsf(xf) > 1e-36f && fabsf(xf) < 1e36f)) return 1.0 / x;
  const double y = (double)rcp_approx_f32(xf);
  return fma(y, fma(-x, y, 1.0), y);  // y (2 - x y)
}
__device__ __forceinline__ double sqrt_nr(double x) {
  const float xf = (float)x;
  if (!(xf > 1e-36f && xf < 1e36f)) return sqrt(x);
  const double y = (double)rsqrt_approx_f32(xf);
  const double s = x * y;                   // sqrt(x) to 2^-23
  return fma(0.5 * y, fma(-s, s, x), s);    // s + (x - s^2) / (2 sqrt(x))
}

// log2 and exp2 in FP64 for the step-size controllers' powers err^a: FP64
// pow costs ~80 FP64 instructions on GB300 (measured), these ~16 each.
// log2: x = 2^e m with m in [sqrt(1/2), sqrt(2)); ln m = 2 atanh(s) with
// s = (m - 1) / (m + 1), |s| <= 0.1716, summed as the odd series to s^21
// (truncation below 1e-19). exp2: y = n + f with n = rint(y), |f| <= 1/2;
// e^(f ln 2) by its Taylor series to degree 14 (truncation below 1e-19), scaled
// by 2^n. Both are accurate to a few ulp for the normal, positive arguments the
// controllers pass (errors and step ratios).
__device__ __forceinline__ double log2_fp64(double x) {
  int e;
  double m = frexp(x, &e);  // m in [0.5, 1)
  if (m < 0.70710678118654752440) { m *= 2.0; e -= 1; }
  const double s = (m - 1.0) / (m + 1.0), s2 = s * s;
  constexpr double c[10] = {1.0 / 3.0,  1.0 / 5.0,  1.0 / 7.0,  1.0 / 9.0,  1.0 / 11.0,
                            1.0 / 13.0, 1.0 / 15.0, 1.0 / 17.0, 1.0 / 19.0, 1.0 / 21.0};
  double p = c[9];
#pragma unroll
  for (int k = 8; k >= 0; --k) p = fma(p, s2, c[k]);
  const double ln_m = fma(2.0 * s * s2, p, 2.0 * s);
  return fma(ln_m, 1.4426950408889634074, (double)e);
}
__device__ __forceinline__ double exp2_fp64(double y) {
  if (!(y > -1020.0)) return y != y ? y : 0.0;  // NaN stays NaN; underflow to 0
  if (y > 1020.0) return __longlong_as_double(0x7ff0000000000000LL);
  const double n = rint(y);
  const double t = (y - n) * 0.69314718055994530942;
  // 1 / k!, k = 0 .. 14
  constexpr double inv_fact[15] = {1.0, 1.0, 1.0 / 2.0, 1.0 / 6.0, 1.0 / 24.0, 1.0 / 120.0, 1.0 / 720.0,
                                   1.0 / 5040.0, 1.0 / 40320.0, 1.0 / 362880.0, 1.0 / 3628800.0,
                                   1.0 / 39916800.0, 1.0 / 479001600.0, 1.0 / 6227020800.0,
                                   1.0 / 87178291200.0};
  double p = inv_fact[14];
#pragma unroll
  for (int k = 13; k >= 0; --k) p = fma(p, t, inv_fact[k]);
  return ldexp(p, (int)n);
}
// x^a for x > 0 (0 for x == 0 and a > 0)
__device__ __forceinline__ double pow_fp64(double x, double a) {
  if (x == 0.0) return a > 0.0 ? 0.0 : 1.0 / x;
  if (isinf(x)) return a > 0.0 ? x : 0.0;
  return exp2_fp64(a * log2_fp64(x));
}

__device__ __forceinline__ double dot3(const double* a, const double* b) {
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}
__device__ __forceinline__ void cross3(const double* a, const double* b, double* o) {
  o[0] = a[1] * b[2] - a[2] * b[1];
  o[1] = a[2] * b[0] - a[0] * b[2];
  o[2] = a[0] * b[1] - a[1] * b[0];
}

}  // namespace rapt
