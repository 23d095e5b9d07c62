// fp32_form.cuh -- the FP32 form: stages on the FP32 pipe, compensated.
//
// Stage arithmetic runs on FP32 hardware with compensated (float-float)
// arithmetic: the state, the stage derivatives, the tableau coefficients, the
// field at the stage point and the dominant terms of the equations of motion are
// hi + lo pairs of floats (df.cuh), so stage values keep ~48 bits. FP64 hardware
// is kept for time, the error norm and the step size. The guiding centres'
// finite-difference grad|B| and curl b are FP32 differences formed without
// cancellation for the dipole models, and the plain form's FP64 stencil (with
// db/dt) for the others.
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

// The dipole models' field for the guiding-centre equations: one routine gives
// the centre sample (|B| and b, float-float: the streaming term b v_par is the
// dominant slope) and the reference's central differences grad|B| and curl b
// (fields.py:111-131, 175-200): (|B|(x + d e_a) - |B|(x - d e_a)) / 2d and the
// same differences of b.
//
// The differences are FP32 and formed without cancellation. Subtracting two
// samples of |B| loses the digits they share (d / r is 2e-4 for the double
// dipole, 2e-7 for the Earth dipole), which is why the reference needs FP64
// samples. Here no step subtracts two samples. For each dipole term
// F(r) = P(r) s(r), P = (3 rz rx, 3 rz ry, 2 rz^2 - rx^2 - ry^2), s = |r|^-5:
//   s(r +- d e_A) = s0 (1 + g(x+-)),  x+- = (d^2 +- 2 r_A d) / |r|^2,
//   g(x) = (1 + x)^(-5/2) - 1 by its series (the direct form for |x| > 1e-2),
// so the sum and difference of the two samples of s come from g's even and odd
// parts, each to FP32's relative rounding; P's exact difference and sum give
//   2 (F+ - F-) = (P+ - P-)(s+ + s-) + (P+ + P-)(s+ - s-),
//   2 (F+ + F-) = (P+ + P-)(s+ + s-) + (P+ - P-)(s+ - s-),
// and then
//   |F+| - |F-| = (F+ - F-) . (F+ + F-) / (|F+| + |F-|),
//   f+ - f-     = (F+ - F-) / |F+| - F- (|F+| - |F-|) / (|F+| |F-|).
// The quotients are the reference's, with the same step d. s0 = |r|^-5 and
// |r|^2 come from the float-float centre sample, which computes them anyway
// (their rounding would scale every difference the same way). No step is
// biased: positions are scaled by a power of two (units of L = 2^22 m),
// reciprocal square roots are Newton-refined and divisions correctly rounded,
// and the constants (the model's coefficient, the second dipole's position and
// strength, the quotient 1 / 2d) enter as float-float. What remains is FP32
// rounding noise, ~1e-7 of the gradient, which averages out along a
// trajectory where a systematic error would not.
constexpr float kStencilLinv = 1.f / 4194304.f;  // 1 / L, L = 2^22 m

// 1 / sqrt(u) to within rounding: rsqrtf and one Newton step whose residual
// 1 - u y^2 is formed with an exact product.
__device__ __forceinline__ float rsqrt_nr(float u) {
  const float y = rsqrtf(u);
  const float t = u * y;
  const float tl = fmaf(u, y, -t);  // u y = t + tl
  const float r = fmaf(-tl, y, fmaf(-t, y, 1.f));
  return fmaf(0.5f * y, r, y);
}

// (1 + x)^(-5/2) - 1 for |x| <= 1e-2: the binomial series to x^6 (truncation
// below 1e-12 relative).
__device__ __forceinline__ float g52(float x) {
  float a = 15015.f / 1024.f;
  a = fmaf(a, x, -3003.f / 256.f);
  a = fmaf(a, x, 1155.f / 128.f);
  a = fmaf(a, x, -105.f / 16.f);
  a = fmaf(a, x, 35.f / 8.f);
  a = fmaf(a, x, -2.5f);
  return a * x;
}

// One dipole term at r +- d e_A: dF = 2 (F+ - F-), sF = 2 (F+ + F-); s0 = |r|^-5,
// r2 = |r|^2, ir2 = 1 / r2 (each rounded once from the float-float centre).
template <int A>
__device__ __forceinline__ void dipole_pm(float rx, float ry, float rz, float d, float s0, float r2, float ir2,
                                          float* dF, float* sF) {
  const float ra = A == 0 ? rx : (A == 1 ? ry : rz);
  const float a1 = 2.f * ra * d * ir2, a0 = d * d * ir2;
  float ss, ds;  // s+ + s-, s+ - s-
  if (fabsf(a1) <= 1e-2f) {
    const float gp = g52(a0 + a1), gm = g52(a0 - a1);
    ss = s0 * (2.f + (gp + gm));
    ds = s0 * (gp - gm);
  } else {  // within ~100 d of a dipole: s+ - s- = (ip - iq)(ip^4 + ip^3 iq + ... + iq^4)
    const float w = fmaf(d, d, r2), e = 2.f * ra * d;
    const float u = w + e, v = w - e;
    const float ip = rsqrt_nr(u), iq = rsqrt_nr(v);
    const float ip2 = ip * ip, iq2 = iq * iq, ab = ip * iq, s2 = ip2 + iq2;
    ss = fmaf(ip2 * ip2, ip, iq2 * iq2 * iq);
    ds = __fdiv_rn(-2.f * e * ab * fmaf(s2, s2 + ab, -ab * ab), fmaf(u, ip, v * iq));
  }
  const float q = 2.f * (2.f * rz * rz - rx * rx - ry * ry);
  float dP[3], sP[3];
  sP[0] = 6.f * rz * rx;
  sP[1] = 6.f * rz * ry;
  if (A == 0) { dP[0] = 6.f * rz * d; dP[1] = 0.f; dP[2] = -4.f * rx * d; sP[2] = q - 2.f * d * d; }
  if (A == 1) { dP[0] = 0.f; dP[1] = 6.f * rz * d; dP[2] = -4.f * ry * d; sP[2] = q - 2.f * d * d; }
  if (A == 2) { dP[0] = 6.f * rx * d; dP[1] = 6.f * ry * d; dP[2] = 8.f * rz * d; sP[2] = q + 4.f * d * d; }
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    dF[i] = fmaf(dP[i], ss, sP[i] * ds);
    sF[i] = fmaf(sP[i], ss, dP[i] * ds);
  }
}

// The float-float centre of one dipole term at r (units of L): F(r) and, for the
// stencil, s0 = |r|^-5, |r|^2 and 1 / |r|^2 rounded to FP32.
struct DipoleCentre {
  DF F0, F1, F2;
  float s0, r2, ir2;
};
__device__ __forceinline__ DipoleCentre dipole_centre(DF rx, DF ry, DF rz) {
  const DF x2 = rx * rx, y2 = ry * ry, z2 = rz * rz;
  const DF r2 = x2 + y2 + z2;
  const DF ip = df_rsqrt(r2), ip2 = ip * ip;
  const DF s0 = (ip2 * ip2) * ip;
  const DF tz = rz * 3.f;
  const DF q = (z2 * 2.f) - x2 - y2;
  return DipoleCentre{(tz * rx) * s0, (tz * ry) * s0, q * s0, df_f(s0), df_f(r2), df_f(ip2)};
}

struct DipoleSample {
  DF mag, u0, u1, u2;  // |B| and b at the centre
  float g0, g1, g2;    // grad|B|
  float c0, c1, c2;    // curl b
};

// Differences along axis A of the field with unit coefficient (the sign and
// size of the coefficient enter the quotients): dmag = |F+| - |F-|,
// db = f+ - f- (f = F / |F|).
template <int M, int A>
__device__ __forceinline__ void dipole_axis(const FieldP& f, float x, float y, float z, float xb,
                                            const DipoleCentre& ca, const DipoleCentre& cb, float& dmag,
                                            float* db) {
  float dF[3], sF[3];
  dipole_pm<A>(x, y, z, f.sd, ca.s0, ca.r2, ca.ir2, dF, sF);
  if constexpr (M == RAPT_DOUBLE_DIPOLE) {  // F(r) + k F(r - xb e_x)
    float dG[3], sG[3];
    dipole_pm<A>(xb, y, z, f.sd, cb.s0, cb.r2, cb.ir2, dG, sG);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      dF[i] = fmaf(f.skl, dG[i], fmaf(f.skh, dG[i], dF[i]));
      sF[i] = fmaf(f.skl, sG[i], fmaf(f.skh, sG[i], sF[i]));
    }
  }
  // with Fp = sF + dF = 4 F+ and Fm = sF - dF = 4 F-:
  //   |F+| - |F-| = (dF . sF) / (|Fp| + |Fm|),
  //   f+ - f-     = 2 dF / |Fp| - Fm 4 (|F+| - |F-|) / (|Fp| |Fm|)
  float Fp[3], Fm[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) { Fp[i] = sF[i] + dF[i]; Fm[i] = sF[i] - dF[i]; }
  const float np = fmaf(Fp[0], Fp[0], fmaf(Fp[1], Fp[1], Fp[2] * Fp[2]));
  const float nm = fmaf(Fm[0], Fm[0], fmaf(Fm[1], Fm[1], Fm[2] * Fm[2]));
  const float ip = rsqrt_nr(np), im = rsqrt_nr(nm);
  dmag = __fdiv_rn(fmaf(dF[0], sF[0], fmaf(dF[1], sF[1], dF[2] * sF[2])), fmaf(np, ip, nm * im));
  const float t = 4.f * dmag * ip * im;
#pragma unroll
  for (int i = 0; i < 3; ++i) db[i] = fmaf(2.f * dF[i], ip, -Fm[i] * t);
}

// Inlined into the right-hand side, its one caller, which is not inlined: one
// copy of the field code per kernel (the kernel's instruction fetch is a
// limit), and no call of its own (measured 2 % faster than a separate call).
template <int M>
__device__ __forceinline__ DipoleSample dipole_sample(const FieldP& f, DF X0, DF X1, DF X2) {
  const DF rx{X0.hi * kStencilLinv, X0.lo * kStencilLinv}, ry{X1.hi * kStencilLinv, X1.lo * kStencilLinv},
      rz{X2.hi * kStencilLinv, X2.lo * kStencilLinv};
  const DipoleCentre ca = dipole_centre(rx, ry, rz);
  DF F[3] = {ca.F0, ca.F1, ca.F2};
  DipoleCentre cb{};
  float xb = 0.f;
  if constexpr (M == RAPT_DOUBLE_DIPOLE) {
    const DF d = X0 - DF{f.sxh, f.sxl};
    const DF rxb{d.hi * kStencilLinv, d.lo * kStencilLinv};
    cb = dipole_centre(rxb, ry, rz);
    const DF k{f.skh, f.skl};
    F[0] = F[0] + cb.F0 * k; F[1] = F[1] + cb.F1 * k; F[2] = F[2] + cb.F2 * k;
    xb = rxb.hi;
  }
  // B = c F: |B| = |c| |F|, b = sign(c) F / |F|
  const DF s2 = F[0] * F[0] + F[1] * F[1] + F[2] * F[2];
  const DF iF = df_rsqrt(s2);
  const DF sc{f.sch < 0.f ? -1.f : 1.f, 0.f};
  const DF ui = iF * sc;
  DipoleSample o;
  o.mag = (s2 * iF) * DF{f.cah, f.cal};
  o.u0 = F[0] * ui; o.u1 = F[1] * ui; o.u2 = F[2] * ui;
  float d0, d1, d2, b0[3], b1[3], b2[3];
  dipole_axis<M, 0>(f, rx.hi, ry.hi, rz.hi, xb, ca, cb, d0, b0);
  dipole_axis<M, 1>(f, rx.hi, ry.hi, rz.hi, xb, ca, cb, d1, b1);
  dipole_axis<M, 2>(f, rx.hi, ry.hi, rz.hi, xb, ca, cb, d2, b2);
  // quotients |c| / (2 d) and sign(c) / (2 d) as float-float products
  auto qg = [&](float v) { return fmaf(v, f.sgl, v * f.sgh); };
  auto qc = [&](float v) { return fmaf(v, f.scl, v * f.sch); };
  o.g0 = qg(d0); o.g1 = qg(d1); o.g2 = qg(d2);
  // curl b = (d bz/dy - d by/dz, d bx/dz - d bz/dx, d by/dx - d bx/dy)
  o.c0 = qc(b1[2] - b2[1]);
  o.c1 = qc(b2[0] - b0[2]);
  o.c2 = qc(b0[1] - b1[0]);
  return o;
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
  // the stage time is read only by models without a float-float form (the dipole
  // models are static); the others skip its FP64 arithmetic
  static constexpr bool kTime = !FieldDF<M>::kDF;
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
    float gB[3], cb[3], db[3] = {0.f, 0.f, 0.f};
    DF Eg[3];  // Grid: E from the same cell search as B
    if constexpr (FieldDF<M>::kDF) {
      static_assert(!FieldDF<M>::kDF || Field<M>::kStatic, "float-float field models are static");
      // centre (float-float) and stencil differences (FP32) in one call, B = |B| b
      const DipoleSample c = dipole_sample<M>(f, Y[0], Y[1], Y[2]);
      Bmag = c.mag;
      ub[0] = c.u0; ub[1] = c.u1; ub[2] = c.u2;
      B[0] = ub[0] * Bmag; B[1] = ub[1] * Bmag; B[2] = ub[2] * Bmag;
      gB[0] = c.g0; gB[1] = c.g1; gB[2] = c.g2;
      cb[0] = c.c0; cb[1] = c.c1; cb[2] = c.c2;
    } else {
      double Ed[3] = {0.0, 0.0, 0.0};
      if constexpr (M == RAPT_GRID) {
        // B, E, the stencil and db/dt of the plain form from one cell search
        const GridFields g = grid_gc_fields(RAPT_GRID_PASS(f), f.gB, f.gE, t, df_to_double(Y[0]),
                                            df_to_double(Y[1]), df_to_double(Y[2]), f.gradstep, f.inv2d,
                                            f.timestep, !field_static<M>(f));
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          B[k] = dfd(g.B[k]); Ed[k] = g.E[k];
          gB[k] = (float)g.gB[k]; cb[k] = (float)g.cb[k]; db[k] = (float)g.db[k];
        }
      } else {
        FieldDF<M>::B(f, t, Y, B);
      }
      const DF b2 = B[0] * B[0] + B[1] * B[1] + B[2] * B[2];
      const DF ib = df_rsqrt(b2);
      Bmag = b2 * ib;
      ub[0] = B[0] * ib; ub[1] = B[1] * ib; ub[2] = B[2] * ib;
      if constexpr (M == RAPT_GRID) { Eg[0] = dfd(Ed[0]); Eg[1] = dfd(Ed[1]); Eg[2] = dfd(Ed[2]); }
    }
    if constexpr (!FieldDF<M>::kDF && M != RAPT_GRID) {
      const double Xd[3] = {df_to_double(Y[0]), df_to_double(Y[1]), df_to_double(Y[2])};
      double gBd[3], cbd[3], dbd[3];
      stencil_gradB_curlb<M>(f, t, Xd, gBd, cbd);
      dbdt<M>(f, t, Xd, dbd);
#pragma unroll
      for (int i = 0; i < 3; ++i) { gB[i] = (float)gBd[i]; cb[i] = (float)cbd[i]; db[i] = (float)dbd[i]; }
    }
    const DF rg = df_rsqrt(DF{1.f, 0.f} + kmu * Bmag + u * u);
    const DF pq = mcq * u;  // ppar / q
    const DF a = (u * rg) * DF(DFc(kC));
    DF Bs[3];
    if constexpr (FieldDF<M>::kDF) {
      // static field, no E. The curl-b term of B* (~rho / L of B) and E* =
      // -(mu / (gamma q)) grad|B| carry the FP32 stencil's relative noise, so
      // the curl-b term, E* x b and E* . B* are FP32 (the drift is ~1e-4..1e-2
      // of the velocity; FP32 rounding of these terms is below the stencil's
      // noise). The per-tracer constants q / (m c) and mu / q enter the mirror
      // force through float-float products: rounded to FP32 they would bias
      // every evaluation of a tracer the same way.
      const float pqf = df_f(pq);
#pragma unroll
      for (int i = 0; i < 3; ++i) Bs[i] = B[i] + pqf * cb[i];
      const DF iBsp = df_rcp(Bs[0] * ub[0] + Bs[1] * ub[1] + Bs[2] * ub[2]);
      const float mgf = df_f(muq * rg);
      const float Es[3] = {-mgf * gB[0], -mgf * gB[1], -mgf * gB[2]};
      const float u0 = df_f(ub[0]), u1 = df_f(ub[1]), u2 = df_f(ub[2]);
      const float Exb[3] = {Es[1] * u2 - Es[2] * u1, Es[2] * u0 - Es[0] * u2, Es[0] * u1 - Es[1] * u0};
#pragma unroll
      for (int i = 0; i < 3; ++i) o[i] = (a * Bs[i] + Exb[i]) * iBsp;
      const float EsBs = Es[0] * df_f(Bs[0]) + Es[1] * df_f(Bs[1]) + Es[2] * df_f(Bs[2]);
      o[3] = (qmc * EsBs) * iBsp;
    } else {
      const DF mg = muq * rg;
#pragma unroll
      for (int i = 0; i < 3; ++i) Bs[i] = B[i] + pq * cb[i];
      const DF iBsp = df_rcp(Bs[0] * ub[0] + Bs[1] * ub[1] + Bs[2] * ub[2]);
      DF E[3], Es[3];
      if constexpr (M == RAPT_GRID) { E[0] = Eg[0]; E[1] = Eg[1]; E[2] = Eg[2]; }
      else FieldDF<M>::E(f, t, Y, E);
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
// floor: a lower bound of the tolerance (0: the plain form's norm).
__device__ __forceinline__ double err_ratio(double e_si, DF y0, DF y1, double scale, double rtol, double atol,
                                           double floor = 0.0) {
  const float ym = fmaxf(fabsf(y0.hi), fabsf(y1.hi));
  return e_si * rcp_nr(fmax(fma(rtol * scale, (double)ym, atol), floor));
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
// cache at the high occupancy this form runs at.
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
    DF acc[NV];
    // only the slopes of row s (k1..k_s; the last row skips k2): warp-uniform
    // tests, and the skipped terms would add exact zeros
    {
      const DF a{A[0].hi, A[0].lo};
#pragma unroll
      for (int i = 0; i < NV; ++i) acc[i] = k1[i] * a;
    }
    if (s >= 2 && s <= 5) {
      const DF a{A[1].hi, A[1].lo};
#pragma unroll
      for (int i = 0; i < NV; ++i) acc[i] = acc[i] + k2[i] * a;
    }
    if (s >= 3) {
      const DF a{A[2].hi, A[2].lo};
#pragma unroll
      for (int i = 0; i < NV; ++i) acc[i] = acc[i] + k3[i] * a;
    }
    if (s >= 4) {
      const DF a{A[3].hi, A[3].lo};
#pragma unroll
      for (int i = 0; i < NV; ++i) acc[i] = acc[i] + k4[i] * a;
    }
    if (s >= 5) {
      const DF a{A[4].hi, A[4].lo};
#pragma unroll
      for (int i = 0; i < NV; ++i) acc[i] = acc[i] + k5[i] * a;
    }
    if (s == 6) {
      const DF a{A[5].hi, A[5].lo};
#pragma unroll
      for (int i = 0; i < NV; ++i) acc[i] = acc[i] + k6[i] * a;
    }
#pragma unroll
    for (int i = 0; i < NV; ++i) yt[i] = y[i] + hd * acc[i];
    f(F::kTime ? x + kDp5C[s] * h : x, yt, kt);
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
  // error estimate sum_j e_j k_j = sum_{j > 1} e_j (k_j - k1) (the e_j sum to
  // zero): the differences of nearby slopes are formed from the float-float
  // parts (nearly exact where they cancel) and summed in FP32 -- the estimate
  // is compared with the tolerance and needs a few digits, not 48 bits.
  // Position components (0..2, metres): the tolerance is floored at 3e-9 of the
  // step's displacement. The FP32 stencil differences put ~1e-7 relative noise
  // on the drift velocity (at most a few per cent of the speed), which the slopes
  // and so the estimate inherit: ~1e-9 of the displacement. Where the
  // reference's scalar tolerance atol + rtol |x| is tighter than that -- a
  // coordinate crossing zero slowly, where atol (1e-8 m) governs alone -- the
  // controller would shrink the step chasing the noise until the interval
  // exceeds nsteps. Elsewhere the floor (~5 mm on a 2e6 m step) is far below
  // the tolerance (~0.3 m) and changes nothing.
  float dp2 = 0.f;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const float d = (y1[i].hi - y[i].hi) + (y1[i].lo - y[i].lo);
    dp2 = fmaf(d, d, dp2);
  }
  const double pfloor = 3e-9 * (double)sqrtf(dp2);
  double e = 0.0;
#pragma unroll
  for (int i = 0; i < NV; ++i) {
    auto dk = [&](const DF& k) { return (k.hi - k1[i].hi) + (k.lo - k1[i].lo); };
    float ei = (float)e3 * dk(k3[i]);
    ei = fmaf((float)e4, dk(k4[i]), ei);
    ei = fmaf((float)e5, dk(k5[i]), ei);
    ei = fmaf((float)e6, dk(k6[i]), ei);
    ei = fmaf((float)e7, dk(k7[i]), ei);
    const double r = err_ratio((double)ei * (h * scale[i]), y[i], y1[i], scale[i], rtol, atol, i < 3 ? pfloor : 0.0);
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
