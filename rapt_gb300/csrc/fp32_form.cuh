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
// magnitudes and unit vectors in float-float (about 48 bits) and the
// differences of the samples in float-float (nearly exact for these nearby
// values, so the cancellation that makes single-precision samples useless
// loses nothing here); the difference quotients in FP32. Their consumer is the
// FP32 drift term of the equations, and the stencil's own truncation error,
// (gradstep / r)^2 = 4e-8 at 5 Re, is larger than FP32 rounding; an FP64
// quotient would cost ~45 FP64 instructions per right-hand side on a pipe that
// runs at 1/64 of the FP32 rate.
// One stencil sample: |B| and the unit vector b at x, float-float. Not
// inlined, so that the kernel holds one copy of the field code for all seven
// samples of a right-hand side (the kernel runs at high occupancy and its
// instruction cache is a limit); arguments and result pass by value, in
// registers, not through local memory.
struct DFSample {
  DF mag, u0, u1, u2;
};
template <int M>
__device__ __noinline__ DFSample stencil_sample_df(const FieldP& f, double t, DF x0, DF x1, DF x2) {
  const DF x[3] = {x0, x1, x2};
  DF b[3];
  FieldDF<M>::B(f, t, x, b);
  const DF s2 = b[0] * b[0] + b[1] * b[1] + b[2] * b[2];
  const DF ib = df_rsqrt(s2);
  return DFSample{s2 * ib, b[0] * ib, b[1] * ib, b[2] * ib};
}

template <int M>
__device__ __forceinline__ void stencil_gradB_curlb_df(const FieldP& f, double t, const DF* Y, float* gB,
                                                       float* cb) {
  const DF d{f.gsh, f.gsl};
  const float s = f.inv2df;
  float c0 = 0.f, c1 = 0.f, c2 = 0.f;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    DF xp[3] = {Y[0], Y[1], Y[2]}, xm[3] = {Y[0], Y[1], Y[2]};
    xp[a] = Y[a] + d;
    xm[a] = Y[a] - d;
    const DFSample sp = stencil_sample_df<M>(f, t, xp[0], xp[1], xp[2]);
    const DFSample sm = stencil_sample_df<M>(f, t, xm[0], xm[1], xm[2]);
    gB[a] = df_f(sp.mag - sm.mag) * s;
    const DF up[3] = {sp.u0, sp.u1, sp.u2}, um[3] = {sm.u0, sm.u1, sm.u2};
    auto du = [&](int i) { return df_f(up[i] - um[i]); };
    if (a == 0) { c1 -= du(2); c2 += du(1); }
    if (a == 1) { c0 += du(2); c2 -= du(0); }
    if (a == 2) { c0 -= du(1); c1 += du(0); }
  }
  cb[0] = c0 * s; cb[1] = c1 * s; cb[2] = c2 * s;
}

// ---------------------------------------------------------------- right-hand sides
// Particle, Y = (x, y, z [m], ux, uy, uz [p/(m c)]):
// dx/dt = c u / gamma, du/dt = q/(m c) E + (q/m) (u x B) / gamma.
template <int M>
struct ParticleRHSdf {
  // field parameters referenced in the kernel's parameter space (__grid_constant__)
  const FieldP& f;
  DF qmc, qm, igam;  // q/(m c), q/m, 1/gamma frozen at the start of advance() (static fields)
  bool eq;
  // The equations are one non-inlined function taking and returning the state
  // by value: DOP853 calls them at 12 stages, and one copy keeps the kernel's
  // hot code small.
  struct DF6 {
    DF v0, v1, v2, v3, v4, v5;
  };
  __device__ __forceinline__ void operator()(double t, const DF* Y, DF* o) const {
    const DF6 r = eval(t, DF6{Y[0], Y[1], Y[2], Y[3], Y[4], Y[5]});
    o[0] = r.v0; o[1] = r.v1; o[2] = r.v2; o[3] = r.v3; o[4] = r.v4; o[5] = r.v5;
  }
  __device__ __noinline__ DF6 eval(double t, DF6 Yv) const {
    const DF Y[6] = {Yv.v0, Yv.v1, Yv.v2, Yv.v3, Yv.v4, Yv.v5};
    DF o[6];
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
    return DF6{o[0], o[1], o[2], o[3], o[4], o[5]};
  }
};

// Guiding centre (Tao-Chan-Brizard, GuidingCenter.py:329-355), Y = (x, y, z [m],
// u = ppar/(m c)). Centre field and the TCB algebra in float-float; grad|B| and
// curl b from the float-float stencil above (models with a float-float field),
// or from the FP64 stencil and db/dt of the plain form (other models).
template <int M>
struct GcRHSdf {
  // the field parameters stay in the kernel's parameter space (the kernel takes
  // them as __grid_constant__): the object handed to this non-inlined call holds
  // a reference, not a ~260-byte copy written to local memory on every attempt
  const FieldP& f;
  DF kmu, mcq, muq, qmc;  // 2 mu/(m c^2), m c/q, mu/q, q/(m c)
  bool eq;
  // The equations are one non-inlined function (one copy serves HINIT, the
  // first slope and the rolled stages) taking and returning the state by value.
  struct DF4 {
    DF v0, v1, v2, v3;
  };
  __device__ __forceinline__ void operator()(double t, const DF* Y, DF* o) const {
    const DF4 r = eval(t, DF4{Y[0], Y[1], Y[2], Y[3]});
    o[0] = r.v0; o[1] = r.v1; o[2] = r.v2; o[3] = r.v3;
  }
  __device__ __noinline__ DF4 eval(double t, DF4 Yv) const {
    const DF Y[4] = {Yv.v0, Yv.v1, Yv.v2, Yv.v3};
    DF o[4];
    const DF u = Y[3];
    DF B[3], Bmag, ub[3];
    if constexpr (FieldDF<M>::kDF) {
      // the centre through the stencil's sample routine (one copy of the field
      // code in the kernel), B = |B| b
      const DFSample c = stencil_sample_df<M>(f, t, Y[0], Y[1], Y[2]);
      Bmag = c.mag;
      ub[0] = c.u0; ub[1] = c.u1; ub[2] = c.u2;
      B[0] = ub[0] * Bmag; B[1] = ub[1] * Bmag; B[2] = ub[2] * Bmag;
    } else {
      FieldDF<M>::B(f, t, Y, B);
      const DF b2 = B[0] * B[0] + B[1] * B[1] + B[2] * B[2];
      const DF ib = df_rsqrt(b2);
      Bmag = b2 * ib;
      ub[0] = B[0] * ib; ub[1] = B[1] * ib; ub[2] = B[2] * ib;
    }
    float gB[3], cb[3], db[3] = {0.f, 0.f, 0.f};
    if constexpr (FieldDF<M>::kDF) {
      static_assert(!FieldDF<M>::kDF || Field<M>::kStatic, "float-float field models are static");
      stencil_gradB_curlb_df<M>(f, t, Y, gB, cb);
    } else {
      const double Xd[3] = {df_to_double(Y[0]), df_to_double(Y[1]), df_to_double(Y[2])};
      double gBd[3], cbd[3], dbd[3];
      stencil_gradB_curlb<M>(f, t, Xd, gBd, cbd);
      dbdt<M>(f, t, Xd, dbd);
#pragma unroll
      for (int i = 0; i < 3; ++i) { gB[i] = (float)gBd[i]; cb[i] = (float)cbd[i]; db[i] = (float)dbd[i]; }
    }
    const DF rg = df_rsqrt(DF{1.f, 0.f} + kmu * Bmag + u * u);
    const DF pq = mcq * u;  // ppar / q
    const DF mg = muq * rg;
    const DF a = (u * rg) * DF(DFc(kC));
    DF Bs[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) Bs[i] = B[i] + pq * cb[i];
    const DF iBsp = df_rcp(Bs[0] * ub[0] + Bs[1] * ub[1] + Bs[2] * ub[2]);
    if constexpr (FieldDF<M>::kDF) {
      // static field, no E: E* = -(mu / (gamma q)) grad|B| carries the FP32
      // quotient of the stencil, so E*, E* x b and E* . B* are FP32 (the drift
      // is ~1e-4 of the velocity: its FP32 rounding is ~1e-11 of a slope)
      const float mgf = df_f(mg);
      const float Es[3] = {-mgf * gB[0], -mgf * gB[1], -mgf * gB[2]};
      const float u0 = df_f(ub[0]), u1 = df_f(ub[1]), u2 = df_f(ub[2]);
      const float Exb[3] = {Es[1] * u2 - Es[2] * u1, Es[2] * u0 - Es[0] * u2, Es[0] * u1 - Es[1] * u0};
#pragma unroll
      for (int i = 0; i < 3; ++i) o[i] = (a * Bs[i] + Exb[i]) * iBsp;
      const float EsBs = Es[0] * df_f(Bs[0]) + Es[1] * df_f(Bs[1]) + Es[2] * df_f(Bs[2]);
      o[3] = (qmc * EsBs) * iBsp;
    } else {
      DF E[3], Es[3];
      FieldDF<M>::E(f, t, Y, E);
#pragma unroll
      for (int i = 0; i < 3; ++i) Es[i] = E[i] - (pq * db[i] + mg * gB[i]);
      const DF Exb[3] = {Es[1] * ub[2] - Es[2] * ub[1], Es[2] * ub[0] - Es[0] * ub[2],
                         Es[0] * ub[1] - Es[1] * ub[0]};
#pragma unroll
      for (int i = 0; i < 3; ++i) o[i] = (a * Bs[i] + Exb[i]) * iBsp;
      o[3] = qmc * (Es[0] * Bs[0] + Es[1] * Bs[1] + Es[2] * Bs[2]) * iBsp;
    }
    if (eq) { o[2] = DF{0.f, 0.f}; o[3] = DF{0.f, 0.f}; }
    return DF4{o[0], o[1], o[2], o[3]};
  }
};

// ---------------------------------------------------------------- steps
// Error ratio of one component, |e| / (atol + rtol max(|y0|, |y1|)), the plain
// form's norm on SI values: e_si is the FP64 error estimate; the scale's |y| is
// taken from the float parts (a tolerance scale needs a few digits) and the
// quotient is a Newton-refined reciprocal (rcp_nr, ~1e-14).
__device__ __forceinline__ double err_ratio(double e_si, DF y0, DF y1, double scale, double rtol, double atol) {
  const float ym = fmaxf(fabsf(y0.hi), fabsf(y1.hi));
  return e_si * rcp_nr(fma(rtol * scale, (double)ym, atol));
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
// exact zeros.
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
    const double r = err_ratio(df_to_double(ei) * (h * scale[i]), y[i], y1[i], scale[i], rtol, atol);
    e = fma(r, r, e);
  }
  err = sqrt_nr(e * (1.0 / NV));
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
    const double isk = err_ratio(scale[i], y[i], y1[i], scale[i], rtol, atol);
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
  err = fabs(h) * e5s * sqrt_nr(rcp_nr(NV * deno));
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
  const double h1 = (der12 <= 1e-15) ? fmax(1e-6, fabs(h) * 1e-3) : pow_fp64(0.01 / der12, iord_inv);
  h = fmin(fmin(100.0 * fabs(h), h1), hmax);
  return copysign(h, posneg);
}

// The step-size factors of the DOPRI5/DOP853 controller (Hairer's codes, as
// SciPy's dopri5/dop853 run them) in FP32: fac11 = err^expo1, the Lund
// stabilisation facold^-beta, the safety factor and the clamp; only the new
// step h * factor is formed in FP64. A factor needs a few digits, and FP32
// keeps its two logarithms, exponentials and quotients off the FP64 pipe.
struct StepFactorF32 {
  float inv_facold_beta;  // facold^-beta
  float fac11;            // err^expo1 of the last attempt
  __device__ __forceinline__ void reset(float beta) { inv_facold_beta = exp2f(-beta * __log2f(1e-4f)); }
  // err of an attempt -> the factor h_new / h after acceptance
  __device__ __forceinline__ float accept_factor(double err, float expo1, float safe, float facc1, float facc2) {
    fac11 = exp2f(expo1 * __log2f((float)fmax(err, 1e-30)));
    const float fac = fmaxf(facc2, fminf(facc1, fac11 * inv_facold_beta * __fdividef(1.f, safe)));
    return __fdividef(1.f, fac);
  }
  // DOPRI5 rejection: h_new / h = 1 / min(facc1, fac11 / safe)
  __device__ __forceinline__ float reject_factor(float safe, float facc1) const {
    return __fdividef(1.f, fminf(facc1, fac11 * __fdividef(1.f, safe)));
  }
  __device__ __forceinline__ void accepted(double err, float beta) {
    inv_facold_beta = exp2f(-beta * __log2f((float)fmax(err, 1e-4)));
  }
};

}  // namespace rapt
