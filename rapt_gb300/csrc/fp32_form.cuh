// fp32_form.cuh -- the FP32 form: stages on the FP32 pipe, compensated.
//
// Stage arithmetic runs on FP32 hardware with compensated (float-float)
// arithmetic: the state, the stage derivatives, the tableau coefficients, the
// field at the stage point and the dominant terms of the equations of motion are
// hi + lo pairs of floats (df.cuh), so stage values keep ~48 bits. FP64 hardware
// is kept for time, the error norm, the step size, and -- for guiding centres --
// the finite-difference grad|B|, curl b and db/dt (the plain form's stencil).
// The error estimate is therefore accurate enough for the reference's norm
// (rtol 1e-8 with a scalar atol applied to near-zero components), and the
// controller follows the plain form's rules; its step-size factor err^(1/q) is
// evaluated with FP32 exp2/log2.
//
// Units: momentum as u = p / (m c) and dipole positions scaled by 1/Re; in SI,
// p^2 ~ 1e-40 and r^-5 ~ 1e-39 fall below FP32's normal range.
#pragma once
#include "df.cuh"
#include "tracer_kernels.cuh"

namespace rapt {

struct DFc {  // compile-time float-float constant
  float hi, lo;
  __host__ __device__ constexpr DFc(double v) : hi((float)v), lo((float)(v - (double)(float)v)) {}
  __device__ __forceinline__ operator DF() const { return DF{hi, lo}; }
};

__device__ __forceinline__ DF dfd(double v) { return df_from_double(v); }
// model constant i of the FP32 form, precomputed on the host
__device__ __forceinline__ DF fconst(const FieldP& f, int i) { return DF{f.dh[i], f.dl[i]}; }
// small correction terms (finite-difference gradients): float precision suffices
__device__ __forceinline__ DF dff(double v) { return DF{(float)v, 0.f}; }

// ---------------------------------------------------------------- field models in float-float
// Generic: FP64 model evaluated at the float-float point, rounded to float-float.
template <int M>
struct FieldDF {
  static constexpr bool kDF = false;  // evaluated in FP64 and rounded to float-float
  __device__ __forceinline__ static void B(const FieldP& f, double t, const DF* X, DF* o) {
    double b[3];
    Field<M>::B(f, t, df_to_double(X[0]), df_to_double(X[1]), df_to_double(X[2]), b);
    o[0] = dfd(b[0]); o[1] = dfd(b[1]); o[2] = dfd(b[2]);
  }
  __device__ __forceinline__ static void E(const FieldP& f, double t, const DF* X, DF* o) {
    double e[3];
    Field<M>::E(f, t, df_to_double(X[0]), df_to_double(X[1]), df_to_double(X[2]), e);
    o[0] = dfd(e[0]); o[1] = dfd(e[1]); o[2] = dfd(e[2]);
  }
};

__device__ __forceinline__ DF inv_re() { return DF(DFc(1.0 / kRe)); }

template <>
struct FieldDF<RAPT_EARTH_DIPOLE> {
  static constexpr bool kDF = true;
  // B = -3 B0 (rx rz, ry rz, rz^2 - r^2/3) / r^5 with r = x / Re
  __device__ __forceinline__ static void B(const FieldP& f, double, const DF* X, DF* o) {
    const DF x = X[0] * inv_re(), y = X[1] * inv_re(), z = X[2] * inv_re();
    const DF r2 = x * x + y * y + z * z;
    const DF ri = df_rsqrt(r2);
    const DF ri2 = ri * ri;
    const DF s = (ri2 * ri2 * ri) * fconst(f, 0);
    o[0] = s * (x * z);
    o[1] = s * (y * z);
    o[2] = s * (z * z - r2 * DF(DFc(1.0 / 3.0)));
  }
  __device__ __forceinline__ static void E(const FieldP&, double, const DF*, DF* o) {
    o[0] = o[1] = o[2] = DF{0.f, 0.f};
  }
};

template <>
struct FieldDF<RAPT_DOUBLE_DIPOLE> {
  static constexpr bool kDF = true;
  __device__ __forceinline__ static void B(const FieldP& f, double, const DF* X, DF* o) {
    const DF x = X[0] * inv_re(), y = X[1] * inv_re(), z = X[2] * inv_re();
    const DF yz2 = y * y + z * z;
    const DF ia = df_rsqrt(x * x + yz2), ia2 = ia * ia, sa = ia2 * ia2 * ia;
    const DF x2 = x - fconst(f, 1);
    const DF ib = df_rsqrt(x2 * x2 + yz2), ib2 = ib * ib, sb = (ib2 * ib2 * ib) * fconst(f, 2);
    const DF tz = z * 3.f, zz2 = (z * z) * 2.f;
    const DF c0 = fconst(f, 0);
    o[0] = c0 * (tz * (x * sa + x2 * sb));
    o[1] = c0 * (tz * y * (sa + sb));
    o[2] = c0 * ((zz2 - x * x - y * y) * sa + (zz2 - x2 * x2 - y * y) * sb);
  }
  __device__ __forceinline__ static void E(const FieldP&, double, const DF*, DF* o) {
    o[0] = o[1] = o[2] = DF{0.f, 0.f};
  }
};

// grad|B| and curl b by the reference's central differences (fields.py:155-200,
// the 6-point stencil of stencil_gradB_curlb): the six field samples, their
// magnitudes and unit vectors in float-float (about 48 bits), the differences
// of the samples in float-float (exact for these nearby values), and the
// difference quotients in FP64. The samples' rounding adds about 1e-10
// relative to the gradients, far below the stencil's own truncation error
// ((gradstep / r)^2, about 4e-8 at 5 Re).
// One stencil sample: |B| and B at x, float-float. Not inlined, so that the
// kernel holds one copy of the field code for all six samples (the kernel runs
// at high occupancy and its instruction cache is the limit).
template <int M>
__device__ __noinline__ void stencil_sample_df(const FieldP& f, double t, DF x0, DF x1, DF x2, DF* mag, DF* u) {
  const DF x[3] = {x0, x1, x2};
  DF b[3];
  FieldDF<M>::B(f, t, x, b);
  const DF s2 = b[0] * b[0] + b[1] * b[1] + b[2] * b[2];
  const DF ib = df_rsqrt(s2);
  *mag = s2 * ib;
  u[0] = b[0] * ib; u[1] = b[1] * ib; u[2] = b[2] * ib;
}

template <int M>
__device__ __forceinline__ void stencil_gradB_curlb_df(const FieldP& f, double t, const DF* Y, double* gB,
                                                       double* cb) {
  const DF d = dfd(f.gradstep);
  double c0 = 0.0, c1 = 0.0, c2 = 0.0;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    DF xp[3] = {Y[0], Y[1], Y[2]}, xm[3] = {Y[0], Y[1], Y[2]};
    xp[a] = Y[a] + d;
    xm[a] = Y[a] - d;
    DF mp, mm, up[3], um[3];
    stencil_sample_df<M>(f, t, xp[0], xp[1], xp[2], &mp, up);
    stencil_sample_df<M>(f, t, xm[0], xm[1], xm[2], &mm, um);
    gB[a] = df_to_double(mp - mm) * f.inv2d;
    auto du = [&](int i) { return df_to_double(up[i] - um[i]); };
    if (a == 0) { c1 -= du(2); c2 += du(1); }
    if (a == 1) { c0 += du(2); c2 -= du(0); }
    if (a == 2) { c0 -= du(1); c1 += du(0); }
  }
  cb[0] = c0 * f.inv2d; cb[1] = c1 * f.inv2d; cb[2] = c2 * f.inv2d;
}

// ---------------------------------------------------------------- right-hand sides
// Particle, Y = (x, y, z [m], ux, uy, uz [p/(m c)]):
// dx/dt = c u / gamma, du/dt = q/(m c) E + (q/m) (u x B) / gamma.
template <int M>
struct ParticleRHSdf {
  FieldP f;
  DF qmc, qm, igam;  // q/(m c), q/m, 1/gamma frozen at the start of advance() (static fields)
  bool eq;
  __device__ __forceinline__ void operator()(double t, const DF* Y, DF* o) const {
    DF ig = igam;
    if (!field_static<M>(f)) ig = df_rsqrt(DF{1.f, 0.f} + Y[3] * Y[3] + Y[4] * Y[4] + Y[5] * Y[5]);
    DF B[3], E[3];
    FieldDF<M>::B(f, t, Y, B);
    FieldDF<M>::E(f, t, Y, E);
    const DF cg = ig * DF(DFc(kC));
    o[0] = Y[3] * cg; o[1] = Y[4] * cg; o[2] = Y[5] * cg;
    const DF a = qm * ig;
    o[3] = qmc * E[0] + a * (Y[4] * B[2] - Y[5] * B[1]);
    o[4] = qmc * E[1] + a * (Y[5] * B[0] - Y[3] * B[2]);
    o[5] = qmc * E[2] + a * (Y[3] * B[1] - Y[4] * B[0]);
    if (eq) { o[2] = DF{0.f, 0.f}; o[5] = DF{0.f, 0.f}; }
  }
};

// Guiding centre (Tao-Chan-Brizard, GuidingCenter.py:329-355), Y = (x, y, z [m],
// u = ppar/(m c)). Centre field and the TCB algebra in float-float; grad|B|,
// curl b and db/dt from the FP64 stencil of the plain form.
template <int M>
struct GcRHSdf {
  FieldP f;
  DF kmu, mcq, muq, qmc;  // 2 mu/(m c^2), m c/q, mu/q, q/(m c)
  bool eq;
  // not inlined: one copy serves HINIT, the first slope and the rolled stages
  __device__ __noinline__ void operator()(double t, const DF* Y, DF* o) const {
    const DF u = Y[3];
    DF B[3];
    FieldDF<M>::B(f, t, Y, B);
    const DF b2 = B[0] * B[0] + B[1] * B[1] + B[2] * B[2];
    const DF ib = df_rsqrt(b2);
    const DF Bmag = b2 * ib;
    const DF ub[3] = {B[0] * ib, B[1] * ib, B[2] * ib};
    double gBd[3], cbd[3], dbd[3];
    if constexpr (FieldDF<M>::kDF) {
      stencil_gradB_curlb_df<M>(f, t, Y, gBd, cbd);
      dbd[0] = dbd[1] = dbd[2] = 0.0;
      static_assert(!FieldDF<M>::kDF || Field<M>::kStatic, "float-float field models are static");
    } else {
      const double Xd[3] = {df_to_double(Y[0]), df_to_double(Y[1]), df_to_double(Y[2])};
      stencil_gradB_curlb<M>(f, t, Xd, gBd, cbd);
      dbdt<M>(f, t, Xd, dbd);
    }
    DF E[3];
    FieldDF<M>::E(f, t, Y, E);
    const DF rg = df_rsqrt(DF{1.f, 0.f} + kmu * Bmag + u * u);
    const DF pq = mcq * u;  // ppar / q
    DF Bs[3], Es[3];
    const DF mg = muq * rg;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      Bs[i] = B[i] + pq * dff(cbd[i]);
      Es[i] = E[i] - (pq * dff(dbd[i]) + mg * dff(gBd[i]));
    }
    const DF iBsp = df_rcp(Bs[0] * ub[0] + Bs[1] * ub[1] + Bs[2] * ub[2]);
    const DF Exb[3] = {Es[1] * ub[2] - Es[2] * ub[1], Es[2] * ub[0] - Es[0] * ub[2], Es[0] * ub[1] - Es[1] * ub[0]};
    const DF a = (u * rg) * DF(DFc(kC));
#pragma unroll
    for (int i = 0; i < 3; ++i) o[i] = (a * Bs[i] + Exb[i]) * iBsp;
    o[3] = qmc * (Es[0] * Bs[0] + Es[1] * Bs[1] + Es[2] * Bs[2]) * iBsp;
    if (eq) { o[2] = DF{0.f, 0.f}; o[3] = DF{0.f, 0.f}; }
  }
};

// ---------------------------------------------------------------- steps
// Error term of one component: the plain form's norm on SI values.
__device__ __forceinline__ double err_sk(DF y0, DF y1, double scale, double rtol, double atol) {
  return atol + rtol * fmax(fabs(df_to_double(y0)), fabs(df_to_double(y1))) * scale;
}

// DOPRI5 attempt (same stages, error estimate and norm as dopri5_attempt).
template <int NV, class F>
__device__ __forceinline__ void dopri5_attempt_df(const F& f, double x, const DF* y, const DF* k1, double h,
                                                  const double* scale, double rtol, double atol, DF* y1, DF* k7,
                                                  double& err) {
  using namespace dp5;
  const DF hd = dfd(h);
  DF k2[NV], k3[NV], k4[NV], k5[NV], k6[NV], yt[NV];
#pragma unroll
  for (int i = 0; i < NV; ++i) yt[i] = y[i] + hd * (k1[i] * DF(DFc(a21)));
  f(x + c2 * h, yt, k2);
#pragma unroll
  for (int i = 0; i < NV; ++i) yt[i] = y[i] + hd * (k1[i] * DF(DFc(a31)) + k2[i] * DF(DFc(a32)));
  f(x + c3 * h, yt, k3);
#pragma unroll
  for (int i = 0; i < NV; ++i)
    yt[i] = y[i] + hd * (k1[i] * DF(DFc(a41)) + k2[i] * DF(DFc(a42)) + k3[i] * DF(DFc(a43)));
  f(x + c4 * h, yt, k4);
#pragma unroll
  for (int i = 0; i < NV; ++i)
    yt[i] = y[i] + hd * (k1[i] * DF(DFc(a51)) + k2[i] * DF(DFc(a52)) + k3[i] * DF(DFc(a53)) + k4[i] * DF(DFc(a54)));
  f(x + c5 * h, yt, k5);
#pragma unroll
  for (int i = 0; i < NV; ++i)
    yt[i] = y[i] + hd * (k1[i] * DF(DFc(a61)) + k2[i] * DF(DFc(a62)) + k3[i] * DF(DFc(a63)) +
                         k4[i] * DF(DFc(a64)) + k5[i] * DF(DFc(a65)));
  const double xph = x + h;
  f(xph, yt, k6);
#pragma unroll
  for (int i = 0; i < NV; ++i)
    y1[i] = y[i] + hd * (k1[i] * DF(DFc(a71)) + k3[i] * DF(DFc(a73)) + k4[i] * DF(DFc(a74)) +
                         k5[i] * DF(DFc(a75)) + k6[i] * DF(DFc(a76)));
  f(xph, y1, k7);
  double e = 0.0;
#pragma unroll
  for (int i = 0; i < NV; ++i) {
    const DF ei = k1[i] * DF(DFc(e1)) + k3[i] * DF(DFc(e3)) + k4[i] * DF(DFc(e4)) + k5[i] * DF(DFc(e5)) +
                  k6[i] * DF(DFc(e6)) + k7[i] * DF(DFc(e7));
    const double r = df_to_double(ei) * h * scale[i] / err_sk(y[i], y1[i], scale[i], rtol, atol);
    e += r * r;
  }
  err = sqrt(e * (1.0 / NV));
}

// The DOPRI5 tableau as float-float pairs in constant memory (rows as kDp5A).
struct DFpair {
  float hi, lo;
};
constexpr DFpair dfp(double v) { return DFpair{(float)v, (float)(v - (double)(float)v)}; }
static __constant__ DFpair kDp5Adf[7][6] = {
    {dfp(0), dfp(0), dfp(0), dfp(0), dfp(0), dfp(0)},
    {dfp(dp5::a21), dfp(0), dfp(0), dfp(0), dfp(0), dfp(0)},
    {dfp(dp5::a31), dfp(dp5::a32), dfp(0), dfp(0), dfp(0), dfp(0)},
    {dfp(dp5::a41), dfp(dp5::a42), dfp(dp5::a43), dfp(0), dfp(0), dfp(0)},
    {dfp(dp5::a51), dfp(dp5::a52), dfp(dp5::a53), dfp(dp5::a54), dfp(0), dfp(0)},
    {dfp(dp5::a61), dfp(dp5::a62), dfp(dp5::a63), dfp(dp5::a64), dfp(dp5::a65), dfp(0)},
    {dfp(dp5::a71), dfp(0), dfp(dp5::a73), dfp(dp5::a74), dfp(dp5::a75), dfp(dp5::a76)}};

// The same DOPRI5 attempt with the six right-hand sides in one rolled loop:
// the right-hand side (float-float field, stencil and equations) is emitted
// once instead of six times, which keeps the kernel inside the instruction
// cache at the high occupancy this form runs at. The zero coefficients add
// exact zeros, so the results equal dopri5_attempt_df's.
template <int NV, class F>
__device__ __forceinline__ void dopri5_attempt_df_rolled(const F& f, double x, const DF* y, const DF* k1, double h,
                                                         const double* scale, double rtol, double atol, DF* y1,
                                                         DF* k7, double& err) {
  using namespace dp5;
  const DF hd = dfd(h);
  DF k2[NV], k3[NV], k4[NV], k5[NV], k6[NV], yt[NV], kt[NV];
#pragma unroll
  for (int i = 0; i < NV; ++i) k2[i] = k3[i] = k4[i] = k5[i] = k6[i] = DF{0.f, 0.f};
#pragma unroll 1
  for (int s = 1; s <= 6; ++s) {
    const DFpair* A = kDp5Adf[s];
    const DF a0{A[0].hi, A[0].lo}, a1{A[1].hi, A[1].lo}, a2{A[2].hi, A[2].lo}, a3{A[3].hi, A[3].lo},
        a4{A[4].hi, A[4].lo}, a5{A[5].hi, A[5].lo};
#pragma unroll
    for (int i = 0; i < NV; ++i)
      yt[i] = y[i] + hd * (k1[i] * a0 + k2[i] * a1 + k3[i] * a2 + k4[i] * a3 + k5[i] * a4 + k6[i] * a5);
    f(x + kDp5C[s] * h, yt, kt);
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      if (s == 1) k2[i] = kt[i];
      if (s == 2) k3[i] = kt[i];
      if (s == 3) k4[i] = kt[i];
      if (s == 4) k5[i] = kt[i];
      if (s == 5) k6[i] = kt[i];
      if (s == 6) { k7[i] = kt[i]; y1[i] = yt[i]; }
    }
  }
  double e = 0.0;
#pragma unroll
  for (int i = 0; i < NV; ++i) {
    const DF ei = k1[i] * DF(DFc(e1)) + k3[i] * DF(DFc(e3)) + k4[i] * DF(DFc(e4)) + k5[i] * DF(DFc(e5)) +
                  k6[i] * DF(DFc(e6)) + k7[i] * DF(DFc(e7));
    const double r = df_to_double(ei) * h * scale[i] / err_sk(y[i], y1[i], scale[i], rtol, atol);
    e += r * r;
  }
  err = sqrt(e * (1.0 / NV));
}

// DOP853 attempt.
template <int NV, class F>
__device__ __forceinline__ void dop853_attempt_df(const F& f, double x, const DF* y, const DF* k1, double h,
                                                  const double* scale, double rtol, double atol, DF* y1,
                                                  double& err) {
  using namespace dp8;
  const DF hd = dfd(h);
  DF k2[NV], k3[NV], k4[NV], k5[NV], k6[NV], k7[NV], k8[NV], k9[NV], k10[NV], yt[NV];
#define RAPT_C(a) DF(DFc(a))
#pragma unroll
  for (int i = 0; i < NV; ++i) yt[i] = y[i] + hd * (k1[i] * RAPT_C(a21));
  f(x + c2 * h, yt, k2);
#pragma unroll
  for (int i = 0; i < NV; ++i) yt[i] = y[i] + hd * (k1[i] * RAPT_C(a31) + k2[i] * RAPT_C(a32));
  f(x + c3 * h, yt, k3);
#pragma unroll
  for (int i = 0; i < NV; ++i) yt[i] = y[i] + hd * (k1[i] * RAPT_C(a41) + k3[i] * RAPT_C(a43));
  f(x + c4 * h, yt, k4);
#pragma unroll
  for (int i = 0; i < NV; ++i)
    yt[i] = y[i] + hd * (k1[i] * RAPT_C(a51) + k3[i] * RAPT_C(a53) + k4[i] * RAPT_C(a54));
  f(x + c5 * h, yt, k5);
#pragma unroll
  for (int i = 0; i < NV; ++i)
    yt[i] = y[i] + hd * (k1[i] * RAPT_C(a61) + k4[i] * RAPT_C(a64) + k5[i] * RAPT_C(a65));
  f(x + c6 * h, yt, k6);
#pragma unroll
  for (int i = 0; i < NV; ++i)
    yt[i] = y[i] + hd * (k1[i] * RAPT_C(a71) + k4[i] * RAPT_C(a74) + k5[i] * RAPT_C(a75) + k6[i] * RAPT_C(a76));
  f(x + c7 * h, yt, k7);
#pragma unroll
  for (int i = 0; i < NV; ++i)
    yt[i] = y[i] + hd * (k1[i] * RAPT_C(a81) + k4[i] * RAPT_C(a84) + k5[i] * RAPT_C(a85) + k6[i] * RAPT_C(a86) +
                         k7[i] * RAPT_C(a87));
  f(x + c8 * h, yt, k8);
#pragma unroll
  for (int i = 0; i < NV; ++i)
    yt[i] = y[i] + hd * (k1[i] * RAPT_C(a91) + k4[i] * RAPT_C(a94) + k5[i] * RAPT_C(a95) + k6[i] * RAPT_C(a96) +
                         k7[i] * RAPT_C(a97) + k8[i] * RAPT_C(a98));
  f(x + c9 * h, yt, k9);
#pragma unroll
  for (int i = 0; i < NV; ++i)
    yt[i] = y[i] + hd * (k1[i] * RAPT_C(a101) + k4[i] * RAPT_C(a104) + k5[i] * RAPT_C(a105) +
                         k6[i] * RAPT_C(a106) + k7[i] * RAPT_C(a107) + k8[i] * RAPT_C(a108) + k9[i] * RAPT_C(a109));
  f(x + c10 * h, yt, k10);
#pragma unroll
  for (int i = 0; i < NV; ++i)
    yt[i] = y[i] + hd * (k1[i] * RAPT_C(a111) + k4[i] * RAPT_C(a114) + k5[i] * RAPT_C(a115) +
                         k6[i] * RAPT_C(a116) + k7[i] * RAPT_C(a117) + k8[i] * RAPT_C(a118) +
                         k9[i] * RAPT_C(a119) + k10[i] * RAPT_C(a1110));
  f(x + c11 * h, yt, k2);
  const double xph = x + h;
#pragma unroll
  for (int i = 0; i < NV; ++i)
    yt[i] = y[i] + hd * (k1[i] * RAPT_C(a121) + k4[i] * RAPT_C(a124) + k5[i] * RAPT_C(a125) +
                         k6[i] * RAPT_C(a126) + k7[i] * RAPT_C(a127) + k8[i] * RAPT_C(a128) +
                         k9[i] * RAPT_C(a129) + k10[i] * RAPT_C(a1210) + k2[i] * RAPT_C(a1211));
  f(xph, yt, k3);
  double e5s = 0.0, e3s = 0.0;
#pragma unroll
  for (int i = 0; i < NV; ++i) {
    const DF bs = k1[i] * RAPT_C(b1) + k6[i] * RAPT_C(b6) + k7[i] * RAPT_C(b7) + k8[i] * RAPT_C(b8) +
                  k9[i] * RAPT_C(b9) + k10[i] * RAPT_C(b10) + k2[i] * RAPT_C(b11) + k3[i] * RAPT_C(b12);
    y1[i] = y[i] + hd * bs;
    const double isk = scale[i] / err_sk(y[i], y1[i], scale[i], rtol, atol);
    const double r3 = df_to_double(bs - k1[i] * RAPT_C(bhh1) - k9[i] * RAPT_C(bhh2) - k3[i] * RAPT_C(bhh3)) * isk;
    const double r5 = df_to_double(k1[i] * RAPT_C(er1) + k6[i] * RAPT_C(er6) + k7[i] * RAPT_C(er7) +
                                   k8[i] * RAPT_C(er8) + k9[i] * RAPT_C(er9) + k10[i] * RAPT_C(er10) +
                                   k2[i] * RAPT_C(er11) + k3[i] * RAPT_C(er12)) * isk;
    e3s += r3 * r3;
    e5s += r5 * r5;
  }
#undef RAPT_C
  double deno = e5s + 0.01 * e3s;
  if (deno <= 0.0) deno = 1.0;
  err = fabs(h) * e5s * sqrt(1.0 / (NV * deno));
}

// HINIT with float-float right-hand sides; norms in FP64 on SI values.
template <int NV, class F>
__device__ __forceinline__ double hinit_df(const F& f, double x, const DF* y, const DF* f0, const double* scale,
                                           double posneg, double iord_inv, double hmax, double rtol, double atol) {
  double dnf = 0.0, dny = 0.0, isk[NV];
#pragma unroll
  for (int i = 0; i < NV; ++i) {
    const double yi = df_to_double(y[i]) * scale[i];
    isk[i] = 1.0 / (atol + rtol * fabs(yi));
    const double a = df_to_double(f0[i]) * scale[i] * isk[i], b = yi * isk[i];
    dnf += a * a;
    dny += b * b;
  }
  double h = (dnf <= 1e-10 || dny <= 1e-10) ? 1e-6 : sqrt(dny / dnf) * 0.01;
  h = fmin(h, hmax);
  h = copysign(h, posneg);
  DF y1[NV], f1[NV];
  const DF hd = dfd(h);
#pragma unroll
  for (int i = 0; i < NV; ++i) y1[i] = y[i] + hd * f0[i];
  f(x + h, y1, f1);
  double der2 = 0.0;
#pragma unroll
  for (int i = 0; i < NV; ++i) {
    const double a = df_to_double(f1[i] - f0[i]) * scale[i] * isk[i];
    der2 += a * a;
  }
  der2 = sqrt(der2) / h;
  const double der12 = fmax(fabs(der2), sqrt(dnf));
  const double h1 = (der12 <= 1e-15) ? fmax(1e-6, fabs(h) * 1e-3) : pow(0.01 / der12, iord_inv);
  h = fmin(fmin(100.0 * fabs(h), h1), hmax);
  return copysign(h, posneg);
}

// err^p with FP32 exp2/log2 (relative error ~1e-7 of the factor).
__device__ __forceinline__ double powf_fast(double err, float p) {
  const float e = (float)fmax(err, 1e-30);
  return (double)exp2f(p * __log2f(e));
}

}  // namespace rapt
