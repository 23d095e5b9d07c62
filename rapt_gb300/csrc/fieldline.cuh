// fieldline.cuh -- the guiding-centre bounce period on the device: the output
// cadence of GuidingCenter.advance when params["GCtimestep"] == 0
// (rapt/GuidingCenter.py:443-446: dt = bounceperiod() / bounceresolution).
//
// One thread computes one tracer's bounce period, once per advance() call
// (and per Adaptive guiding-centre segment), following
//   GuidingCenter.bounceperiod      rapt/GuidingCenter.py:593-606
//   flutils.halfbouncepath          rapt/flutils.py:254-316
//   Fieldline.trace with rkf        rapt/fieldline.py:13-107, rapt/rkf.py:13-143
// and the SciPy routines halfbouncepath calls, from their published methods:
// the quadratic interpolating B-spline of interp1d(kind='quadratic') and
// Brent's root finder (brentq defaults); the final integral (quad in the
// reference) is taken to convergence (see fl_bounce_integral). Products and
// sums are rounded separately (no FMA contraction), as the reference's numpy
// arithmetic is.
//
// The (s, |B|) samples of the trace live in a per-thread scratch buffer:
// the backward half written downwards from slot cap, the forward half upwards,
// so the joined curve is contiguous. The spline solve reuses the buffer.
#pragma once
#include <cfloat>

#include "fields.cuh"

namespace rapt {

__device__ __forceinline__ double dm(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double da(double a, double b) { return __dadd_rn(a, b); }
// numpy's 3-vector dot rounds as fma(a2, b2, fma(a1, b1, a0 b0))
__device__ __forceinline__ double ndot3(const double* a, const double* b) {
  return __fma_rn(a[2], b[2], __fma_rn(a[1], b[1], __dmul_rn(a[0], b[0])));
}

template <int M>
__device__ __forceinline__ double fl_magB(const FieldP& f, double t, double x, double y, double z) {
  double B[3];
  Field<M>::B(f, t, x, y, z, B);
  return sqrt(ndot3(B, B));
}

// _Field.curvature (fields.py:155-174) with _Field.gradB (fields.py:111-131);
// np.dot(gB, |B|) is elementwise there (kept).
template <int M>
__device__ double fl_curvature(const FieldP& f, double t, const double* X) {
  double Bv[3];
  Field<M>::B(f, t, X[0], X[1], X[2], Bv);
  const double B = sqrt(ndot3(Bv, Bv));
  const double d = f.gradstep;
  double gp[3];
#pragma unroll 1
  for (int i = 0; i < 3; ++i) {
    double xp[3] = {X[0], X[1], X[2]}, xm[3] = {X[0], X[1], X[2]};
    xp[i] = da(X[i], d);
    xm[i] = da(X[i], -d);
    const double g = (fl_magB<M>(f, t, xp[0], xp[1], xp[2]) - fl_magB<M>(f, t, xm[0], xm[1], xm[2])) / (2 * d);
    gp[i] = da(g, -dm(dm(g, B) / dm(B, B), Bv[i]));
  }
  return sqrt(ndot3(gp, gp)) / B;
}

// d[s,x,y,z]/ds = sign (1, b) (fieldline.py:39-51)
template <int M>
__device__ __forceinline__ void fl_deriv(const FieldP& f, double t, double sign, const double* Y, double* o) {
  double B[3];
  Field<M>::B(f, t, Y[1], Y[2], Y[3], B);
  const double m = sqrt(ndot3(B, B));
  o[0] = sign;
  o[1] = sign > 0 ? B[0] / m : -(B[0] / m);
  o[2] = sign > 0 ? B[1] / m : -(B[1] / m);
  o[3] = sign > 0 ? B[2] / m : -(B[2] / m);
}

// rkf(f, 0, b, x0, tol, hmax, hmin) (rkf.py:13-143). Accepted points go to
// slots idx, idx + dirn, ... (s and |B|); returns false where rkf raises (the
// trace then ends) and sets overflow when the buffer is full.
template <int M>
__device__ bool fl_rkf(const FieldP& f, double t0, double sign, double* x, double b, double tol, double hmax,
                       double hmin, double* S, double* Bs, int& idx, int dirn, int lo, int hi, bool& overflow) {
  constexpr double b21 = 2.500000000000000e-01, b31 = 9.375000000000000e-02, b32 = 2.812500000000000e-01,
                   b41 = 8.793809740555303e-01, b42 = -3.277196176604461e+00, b43 = 3.320892125625853e+00,
                   b51 = 2.032407407407407e+00, b52 = -8.000000000000000e+00, b53 = 7.173489278752436e+00,
                   b54 = -2.058966861598441e-01, b61 = -2.962962962962963e-01, b62 = 2.000000000000000e+00,
                   b63 = -1.381676413255361e+00, b64 = 4.529727095516569e-01, b65 = -2.750000000000000e-01;
  constexpr double r1 = 2.777777777777778e-03, r3 = -2.994152046783626e-02, r4 = -2.919989367357789e-02,
                   r5 = 2.000000000000000e-02, r6 = 3.636363636363636e-02;
  constexpr double c1 = 1.157407407407407e-01, c3 = 5.489278752436647e-01, c4 = 5.353313840155945e-01,
                   c5 = -2.000000000000000e-01;
  double t = 0.0, h = hmax;
  for (int guard = 0; guard < 100000 && t < b; ++guard) {
    if (da(t, h) > b) h = da(b, -t);
    double k1[4], k2[4], k3[4], k4[4], k5[4], k6[4], xt[4], fv[4];
    fl_deriv<M>(f, t0, sign, x, fv);
    for (int i = 0; i < 4; ++i) k1[i] = dm(h, fv[i]);
    for (int i = 0; i < 4; ++i) xt[i] = da(x[i], dm(b21, k1[i]));
    fl_deriv<M>(f, t0, sign, xt, fv);
    for (int i = 0; i < 4; ++i) k2[i] = dm(h, fv[i]);
    for (int i = 0; i < 4; ++i) xt[i] = da(da(x[i], dm(b31, k1[i])), dm(b32, k2[i]));
    fl_deriv<M>(f, t0, sign, xt, fv);
    for (int i = 0; i < 4; ++i) k3[i] = dm(h, fv[i]);
    for (int i = 0; i < 4; ++i) xt[i] = da(da(da(x[i], dm(b41, k1[i])), dm(b42, k2[i])), dm(b43, k3[i]));
    fl_deriv<M>(f, t0, sign, xt, fv);
    for (int i = 0; i < 4; ++i) k4[i] = dm(h, fv[i]);
    for (int i = 0; i < 4; ++i)
      xt[i] = da(da(da(da(x[i], dm(b51, k1[i])), dm(b52, k2[i])), dm(b53, k3[i])), dm(b54, k4[i]));
    fl_deriv<M>(f, t0, sign, xt, fv);
    for (int i = 0; i < 4; ++i) k5[i] = dm(h, fv[i]);
    for (int i = 0; i < 4; ++i)
      xt[i] = da(da(da(da(da(x[i], dm(b61, k1[i])), dm(b62, k2[i])), dm(b63, k3[i])), dm(b64, k4[i])),
                 dm(b65, k5[i]));
    fl_deriv<M>(f, t0, sign, xt, fv);
    for (int i = 0; i < 4; ++i) k6[i] = dm(h, fv[i]);
    double r = 0.0;
    for (int i = 0; i < 4; ++i) {
      const double e = da(da(da(da(dm(r1, k1[i]), dm(r3, k3[i])), dm(r4, k4[i])), dm(r5, k5[i])), dm(r6, k6[i]));
      const double ri = fabs(e) / h;
      if (i == 0 || ri > r) r = ri;
    }
    if (r <= tol) {
      t = da(t, h);
      for (int i = 0; i < 4; ++i) x[i] = da(da(da(da(x[i], dm(c1, k1[i])), dm(c3, k3[i])), dm(c4, k4[i])), dm(c5, k5[i]));
      idx += dirn;
      if (idx < lo || idx > hi) { overflow = true; return false; }
      S[idx] = x[0];
      Bs[idx] = fl_magB<M>(f, t0, x[1], x[2], x[3]);
    }
    h = dm(h, fmin(fmax(dm(0.84, pow(tol / r, 0.25)), 0.1), 4.0));
    if (h > hmax) h = hmax;
    else if (h < hmin) return false;
  }
  return true;
}

// ---------------------------------------------------------------- quadratic spline
// Interpolating B-spline of degree 2 on n points x[0..n-1] (knots x0 x0 x0,
// midpoints of (x1,x2) .. (x_{n-3},x_{n-2}), x_{n-1} x3); c[0..n-1] coefficients.
struct DSpline2 {
  const double* x;
  const double* c;
  int n;
  __device__ __forceinline__ double knot(int j) const {
    return j <= 2 ? x[0] : (j >= n ? x[n - 1] : (x[j - 2] + x[j - 1]) / 2.0);
  }
  __device__ __forceinline__ int find(double v) const {
    if (v >= knot(n)) return n - 1;
    int lo = 2, hi = n;
    while (hi - lo > 1) {
      const int mid = (lo + hi) / 2;
      if (v < knot(mid)) hi = mid; else lo = mid;
    }
    return lo;
  }
  __device__ __forceinline__ void basis(double v, int l, double* h) const {
    double hh[2];
    h[0] = 1.0;
    h[1] = h[2] = 0.0;
#pragma unroll
    for (int j = 1; j <= 2; ++j) {
      for (int i = 0; i < j; ++i) hh[i] = h[i];
      h[0] = 0.0;
      for (int m = 1; m <= j; ++m) {
        const double xb = knot(l + m), xa = knot(l + m - j);
        if (xb == xa) { h[m] = 0.0; continue; }
        const double w = hh[m - 1] / (xb - xa);
        h[m - 1] = da(h[m - 1], dm(w, xb - v));
        h[m] = dm(w, v - xa);
      }
    }
  }
  __device__ __forceinline__ double operator()(double v) const {
    const int l = find(v);
    double h[3];
    basis(v, l, h);
    double y = 0.0;
    for (int a = 0; a <= 2; ++a) y = da(y, dm(c[l + a - 2], h[a]));
    return y;
  }
};

// Collocation solve (tridiagonal: x_i lies in [t[i+1], t[i+2])), in place:
// yc holds the data on entry and the coefficients on exit; di, up scratch.
static __device__ __noinline__ void spline2_solve(const double* x, double* yc, double* di, double* up, int n) {
  DSpline2 sp{x, yc, n};
  // forward elimination row by row (the lower entry is formed when the row is built)
  for (int i = 0; i < n; ++i) {
    const int l = sp.find(x[i]);
    double h[3];
    sp.basis(x[i], l, h);
    double lo = 0.0, d = 0.0, u = 0.0;
    for (int a = 0; a <= 2; ++a) {
      const int j = l + a - 2;
      if (j == i - 1) lo = h[a];
      else if (j == i) d = h[a];
      else if (j == i + 1) u = h[a];
    }
    if (i > 0) {
      const double m = lo / di[i - 1];
      d = da(d, -dm(m, up[i - 1]));
      yc[i] = da(yc[i], -dm(m, yc[i - 1]));
    }
    di[i] = d;
    up[i] = u;
  }
  yc[n - 1] = yc[n - 1] / di[n - 1];
  for (int i = n - 2; i >= 0; --i) yc[i] = da(yc[i], -dm(up[i], yc[i + 1])) / di[i];
}

// ---------------------------------------------------------------- brentq
struct MirrorFn {
  DSpline2 sp;
  double Bm;
  __device__ __forceinline__ double operator()(double v) const { return da(sp(v), -Bm); }
};

static __device__ __noinline__ double fl_brentq(const MirrorFn& f, double xa, double xb) {
  const double xtol = 2e-12, rtol = 4 * DBL_EPSILON;
  double xpre = xa, xcur = xb, xblk = 0.0, fpre, fcur, fblk = 0.0, spre = 0.0, scur = 0.0, sbis;
  fpre = f(xpre);
  fcur = f(xcur);
  if (fpre == 0) return xpre;
  if (fcur == 0) return xcur;
  for (int i = 0; i < 100; ++i) {
    if (fpre != 0 && fcur != 0 && (signbit(fpre) != signbit(fcur))) {
      xblk = xpre;
      fblk = fpre;
      spre = scur = xcur - xpre;
    }
    if (fabs(fblk) < fabs(fcur)) {
      xpre = xcur; xcur = xblk; xblk = xpre;
      fpre = fcur; fcur = fblk; fblk = fpre;
    }
    const double delta = da(xtol, dm(rtol, fabs(xcur))) / 2;
    sbis = (xblk - xcur) / 2;
    if (fcur == 0 || fabs(sbis) < delta) return xcur;
    if (fabs(spre) > delta && fabs(fcur) < fabs(fpre)) {
      double stry;
      if (xpre == xblk) {
        stry = dm(-fcur, xcur - xpre) / (fcur - fpre);
      } else {
        const double dpre = (fpre - fcur) / (xpre - xcur);
        const double dblk = (fblk - fcur) / (xblk - xcur);
        stry = dm(-fcur, da(dm(fblk, dblk), -dm(fpre, dpre))) / dm(dm(dblk, dpre), fblk - fpre);
      }
      if (2 * fabs(stry) < fmin(fabs(spre), da(3 * fabs(sbis), -delta))) {
        spre = scur;
        scur = stry;
      } else {
        spre = sbis;
        scur = sbis;
      }
    } else {
      spre = sbis;
      scur = sbis;
    }
    xpre = xcur;
    fpre = fcur;
    if (fabs(scur) > delta) xcur = da(xcur, scur);
    else xcur = da(xcur, sbis > 0 ? delta : -delta);
    fcur = f(xcur);
  }
  return xcur;
}

// ---------------------------------------------------------------- half-bounce integral
// The reference integrates 1/sqrt(1 - B(s)/Bm) over [sm1, sm2] with QUADPACK
// QAGS at epsrel 1e-4; on these symmetric field lines the two mirror-point
// singularities give tied error estimates and QAGS's bisection order (and its
// result, to ~5e-6) depends on the last bit of the spline values. Here the
// same spline is integrated to convergence instead: s = c + h sin(theta)
// removes the singularities and an 8-point Gauss-Legendre rule runs on every
// panel between the images of the spline's knots.
__device__ __forceinline__ void gauss_legendre8(double* x, double* w) {
  const int n = 8;
  for (int i = 0; i < n / 2; ++i) {
    double z = cos(kPi * (i + 0.75) / (n + 0.5)), pp = 0.0;
    for (int it = 0; it < 100; ++it) {
      double p1 = 1.0, p2 = 0.0;
      for (int j = 1; j <= n; ++j) {
        const double p3 = p2;
        p2 = p1;
        p1 = da(dm(dm(2.0 * j - 1.0, z), p2), -dm(j - 1.0, p3)) / j;
      }
      pp = dm(n, da(dm(z, p1), -p2)) / da(dm(z, z), -1.0);
      const double z1 = z;
      z = da(z1, -(p1 / pp));
      if (fabs(z - z1) <= 1e-16) break;
    }
    x[i] = -z;
    x[n - 1 - i] = z;
    w[i] = w[n - 1 - i] = 2.0 / dm(dm(da(1.0, -dm(z, z)), pp), pp);
  }
}

// INV: integrand 1/sqrt(1 - B/Bm) (half-bounce path); otherwise sqrt(1 - B/Bm)
// (the second invariant I), which the substitution leaves smooth as well.
template <bool INV = true>
static __device__ __noinline__ double fl_bounce_integral(const DSpline2& sp, double sm1, double sm2, double Bm) {
  double gx[8], gw[8];
  gauss_legendre8(gx, gw);
  const double c = dm(0.5, da(sm1, sm2)), h = dm(0.5, da(sm2, -sm1));
  double sum = 0.0, ea = -kPi / 2;
  // panel edges: -pi/2, the knots inside (sm1, sm2) in order, pi/2
  for (int j = 3; j <= sp.n; ++j) {
    double eb;
    if (j < sp.n) {
      const double tj = sp.knot(j);
      if (!(tj > sm1 && tj < sm2)) continue;
      eb = asin((tj - c) / h);
    } else {
      eb = kPi / 2;
    }
    const double mid = dm(0.5, da(ea, eb)), half = dm(0.5, da(eb, -ea));
    double ps = 0.0;
    for (int k = 0; k < 8; ++k) {
      const double th = da(mid, dm(half, gx[k]));
      const double arg = da(1.0, -(sp(da(c, dm(h, sin(th)))) / Bm));
      if (arg > 0.0) ps = da(ps, dm(gw[k], INV ? dm(h, cos(th)) / sqrt(arg) : dm(dm(h, cos(th)), sqrt(arg))));
    }
    sum = da(sum, dm(half, ps));
    ea = eb;
  }
  return sum;
}

// ---------------------------------------------------------------- half-bounce path and bounce period
// flutils.halfbouncepath (flutils.py:254-316) at position X, time t, mirror
// field Bm. scratch: 4 * (2 * cap) doubles. Returns NaN where the trace
// overflows the buffer or the result is not finite.
// Fieldline(tpos, field, Bmax=Bm).trace() (fieldline.py:37-105) through X,
// both directions joined in S, Bs [first, first + n0); false where the trace
// overflows the buffer or the step is not finite.
template <int M>
__device__ bool fl_trace(const FieldP& f, double t, const double* X, double Bm, double flres, double* scratch,
                         int cap, int& first, int& n0) {
  double* S = scratch;                 // [2 cap] arc length of the joined curve
  double* Bs = scratch + 2 * cap;      // [2 cap] |B|
  const double ds = 1.0 / fl_curvature<M>(f, t, X) / flres;  // fieldline.py:31-35
  if (!(ds > 0) || !isfinite(ds)) return false;
  const int c0 = cap;  // slot of the start point
  S[c0] = 0.0;
  Bs[c0] = fl_magB<M>(f, t, X[0], X[1], X[2]);
  int ifw = c0, ibw = c0;
  bool overflow = false;
  for (int dir = 0; dir < 2; ++dir) {
    const double tol = dir == 0 ? 1e-3 : 1e-4;  // fieldline.py:67 and :92
    const double sign = dir == 0 ? 1.0 : -1.0;
    int& idx = dir == 0 ? ifw : ibw;
    double x[4] = {0.0, X[0], X[1], X[2]};
    for (int guard = 0; guard < 4 * cap; ++guard) {
      // x holds the last point of this direction; where rkf raises, the
      // reference keeps none of that call's points (fieldline.py:68-69)
      const int before = idx;
      if (!fl_rkf<M>(f, t, sign, x, ds, tol, ds, 1e-6, S, Bs, idx, dir == 0 ? 1 : -1, 0, 2 * cap - 1, overflow)) {
        idx = before;
        break;
      }
      if (Bs[idx] > Bm) break;
    }
    if (overflow) return false;
  }
  first = ibw;
  n0 = ifw - ibw + 1;  // joined curve: slots ibw .. ifw
  return true;
}

template <int M>
__device__ __noinline__ double fl_halfbouncepath(const FieldP& f, double t, const double* X, double Bm,
                                                 double flres, double* scratch, int cap) {
  double* S = scratch;                 // [2 cap] arc length of the joined curve
  double* Bs = scratch + 2 * cap;      // [2 cap] |B|, then the spline coefficients
  double* di = scratch + 4 * cap;      // [2 cap]
  double* up = scratch + 6 * cap;      // [2 cap]
  int first, n0;
  if (!fl_trace<M>(f, t, X, Bm, flres, scratch, cap, first, n0)) return nan("");
  int fin = -1, lin = -1;
  for (int i = 0; i < n0; ++i)
    if (Bs[first + i] <= Bm) {
      if (fin < 0) fin = i;
      lin = i;
    }
  int i1, i2;
  if (fin < 0) { i1 = (n0 - 3) / 2; i2 = (n0 + 1) / 2; }
  else { i1 = fin - 1; i2 = lin + 1; }
  const int lo = i1 < 0 ? 0 : i1, hi = i2 > n0 - 1 ? n0 - 1 : i2;
  const int n = hi - lo + 1;
  const double* s = S + first + lo;
  double* b = Bs + first + lo;
  if (n == 3) {  // equatorial (flutils.py:292-303)
    const double s12 = s[0] - s[1], s23 = s[1] - s[2], s13 = s[0] - s[2];
    const double B2s = 2 * da(da(dm(b[0], s23), -dm(b[1], s13)), dm(b[2], s12)) / dm(dm(s12, s13), s23);
    return dm(kPi, sqrt(2 * Bm / B2s));
  }
  if (n < 3) return nan("");
  spline2_solve(s, b, di, up, n);
  const DSpline2 sp{s, b, n};
  const MirrorFn g{sp, Bm};
  const double sm1 = fl_brentq(g, s[0], s[1]);
  const double sm2 = fl_brentq(g, s[n - 2], s[n - 1]);
  return fl_bounce_integral(sp, sm1, sm2, Bm);
}

// flutils.eye (flutils.py:65-151), the second invariant I at X for mirror field
// Bm, over the same trace: 0 where the line's minimum |B| exceeds Bm or equals
// it (equatorial); the points with B < Bm plus one beyond each end; the
// quadratic spline, brentq mirror points and the integral of sqrt(1 - B/Bm)
// to convergence. The reference takes this spline branch at equatorial pitch
// angles of 70 degrees and above; below, its Simpson branch calls an undefined
// name and raises, and here the spline branch serves every pitch angle. NaN
// where the trace overflows or the trimmed line fails the reference's assert.
template <int M>
__device__ __noinline__ double fl_eye(const FieldP& f, double t, const double* X, double Bm, double flres,
                                     double* scratch, int cap) {
  double* S = scratch;
  double* Bs = scratch + 2 * cap;
  double* di = scratch + 4 * cap;
  double* up = scratch + 6 * cap;
  int first, n0;
  if (!fl_trace<M>(f, t, X, Bm, flres, scratch, cap, first, n0) || n0 < 1) return nan("");
  double Bmin = Bs[first];
  for (int i = 1; i < n0; ++i) Bmin = fmin(Bmin, Bs[first + i]);
  if (Bmin > Bm) return 0.0;
  if (fabs(Bmin - Bm) / Bm < 1e-12) return 0.0;
  int fin = -1, lin = -1;
  for (int i = 0; i < n0; ++i)
    if (Bs[first + i] < Bm) {
      if (fin < 0) fin = i;
      lin = i;
    }
  const int lo = fin - 1 < 0 ? 0 : fin - 1, hi = lin + 1 > n0 - 1 ? n0 - 1 : lin + 1;
  const int n = hi - lo + 1;
  const double* s = S + first + lo;
  double* b = Bs + first + lo;
  if (!(n >= 3 && b[0] > Bm && b[1] < Bm && b[n - 2] < Bm && b[n - 1] > Bm)) return nan("");
  spline2_solve(s, b, di, up, n);
  const DSpline2 sp{s, b, n};
  const MirrorFn g{sp, Bm};
  const double sm1 = fl_brentq(g, s[0], s[1]);
  const double sm2 = sp(s[n - 2]) == Bm ? s[n - 2] : fl_brentq(g, s[n - 2], s[n - 1]);
  return fl_bounce_integral<false>(sp, sm1, sm2, Bm);
}

// flutils.gradI (flutils.py:153-229): central differences of I over d in the
// two directions perpendicular to b built from (x, y, 0); one-sided where one
// end has I = 0.
template <int M>
__device__ void fl_gradI(const FieldP& f, double t, const double* X, double Bm, double d, double flres,
                         double* scratch, int cap, double* out) {
  const double sc = fmax(fabs(X[0]), fabs(X[1]));
  double r[3] = {X[0] / sc, X[1] / sc, 0.0 / sc};
  double b[3], mag;
  unit_and_mag<M>(f, t, X[0], X[1], X[2], b, mag);
  const double rb = ndot3(r, b);
  for (int i = 0; i < 3; ++i) r[i] = da(r[i], -dm(rb, b[i]));
  const double rn = sqrt(ndot3(r, r));
  for (int i = 0; i < 3; ++i) r[i] = r[i] / rn;
  const double v2[3] = {da(dm(b[1], r[2]), -dm(b[2], r[1])), da(dm(b[2], r[0]), -dm(b[0], r[2])),
                        da(dm(b[0], r[1]), -dm(b[1], r[0]))};
  double dI[2];
  for (int k = 0; k < 2; ++k) {
    const double* v = k == 0 ? r : v2;
    const double xp[3] = {da(X[0], dm(d, v[0])), da(X[1], dm(d, v[1])), da(X[2], dm(d, v[2]))};
    const double xm[3] = {da(X[0], -dm(d, v[0])), da(X[1], -dm(d, v[1])), da(X[2], -dm(d, v[2]))};
    const double I1 = fl_eye<M>(f, t, xp, Bm, flres, scratch, cap);
    const double I2 = fl_eye<M>(f, t, xm, Bm, flres, scratch, cap);
    if (I1 == 0.0) dI[k] = da(fl_eye<M>(f, t, X, Bm, flres, scratch, cap), -I2) / d;
    else if (I2 == 0.0) dI[k] = da(I1, -fl_eye<M>(f, t, X, Bm, flres, scratch, cap)) / d;
    else dI[k] = da(I1, -I2) / (2.0 * d);
  }
  for (int i = 0; i < 3; ++i) out[i] = da(dm(dI[0], r[i]), dm(dI[1], v2[i]));
}

// GuidingCenter.bounceperiod (GuidingCenter.py:593-606) at state (x, y, z, ppar).
template <int M>
__device__ double gc_bounceperiod(const FieldP& f, double t, const double* y, double mu, double m, double flres,
                                  double* scratch, int cap) {
  const double Bmag = fl_magB<M>(f, t, y[0], y[1], y[2]);
  const double ppar = y[3];
  const double gamma = sqrt(da(da(1.0, dm(2.0, dm(mu, Bmag)) / dm(m, dm(kC, kC))), dm(ppar / (m * kC), ppar / (m * kC))));
  double p, v, Bmirror;
  if (gamma - 1 < 1e-6) {
    p = sqrt(da(dm(dm(2.0, m), dm(mu, Bmag)), dm(ppar, ppar)));
    v = p / m;
    Bmirror = dm(p, p) / dm(dm(2.0, m), mu);
  } else {
    p = dm(dm(m, kC), sqrt(dm(gamma + 1, gamma - 1)));
    Bmirror = dm(dm(p, p) / dm(p - ppar, p + ppar), Bmag);
    v = p / m / gamma;
  }
  return dm(2.0 / v, fl_halfbouncepath<M>(f, t, y, Bmirror, flres, scratch, cap));
}

}  // namespace rapt
