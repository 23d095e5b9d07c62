// fieldline_oracle.cpp -- CPU restatement of the guiding-centre bounce period
// (test infrastructure: the oracle of the device code in csrc/fieldline.cuh).
//
// Follows, in order:
//   GuidingCenter.bounceperiod      rapt/GuidingCenter.py:593-606
//   flutils.bounceperiod            rapt/flutils.py:232-252
//   flutils.halfbouncepath          rapt/flutils.py:254-316
//   Fieldline.__init__/_estimate_step/trace   rapt/fieldline.py:13-107, getB :123-127
//   rkf (Runge-Kutta-Fehlberg 4(5), Burden & Faires)   rapt/rkf.py:13-143
// and the SciPy routines halfbouncepath calls, restated from their published
// methods: interp1d(kind='quadratic') = quadratic interpolating B-spline with
// knots at the midpoints of the interior data (de Boor); brentq = Brent's
// root finder with SciPy's defaults (xtol 2e-12, rtol 4 eps, 100 iterations);
// quad = QUADPACK QAGS (21-point Gauss-Kronrod, bisection, Wynn's epsilon
// algorithm; Piessens et al. 1983) with epsabs 1.49e-8, epsrel 1e-4, limit 50.
#include <cfloat>
#include <cmath>
#include <cstring>
#include <vector>

#include "rapt_oracle.h"

namespace {

constexpr double kPiF = 3.141592653589793;

// ---------------------------------------------------------------- rkf.py
const double ra2 = 2.500000000000000e-01, ra3 = 3.750000000000000e-01, ra4 = 9.230769230769231e-01,
             ra6 = 5.000000000000000e-01;
const double rb21 = 2.500000000000000e-01, rb31 = 9.375000000000000e-02, rb32 = 2.812500000000000e-01,
             rb41 = 8.793809740555303e-01, rb42 = -3.277196176604461e+00, rb43 = 3.320892125625853e+00,
             rb51 = 2.032407407407407e+00, rb52 = -8.000000000000000e+00, rb53 = 7.173489278752436e+00,
             rb54 = -2.058966861598441e-01, rb61 = -2.962962962962963e-01, rb62 = 2.000000000000000e+00,
             rb63 = -1.381676413255361e+00, rb64 = 4.529727095516569e-01, rb65 = -2.750000000000000e-01;
const double rr1 = 2.777777777777778e-03, rr3 = -2.994152046783626e-02, rr4 = -2.919989367357789e-02,
             rr5 = 2.000000000000000e-02, rr6 = 3.636363636363636e-02;
const double rc1 = 1.157407407407407e-01, rc3 = 5.489278752436647e-01, rc4 = 5.353313840155945e-01,
             rc5 = -2.000000000000000e-01;

// d[s,x,y,z]/ds = sign * (1, b)
void fl_deriv(const orc_field* f, double time, double sign, const double* Y, double* o) {
  const double tpos[4] = {time, Y[1], Y[2], Y[3]};
  double b[3];
  orc_unitb(f, tpos, b);
  o[0] = sign * 1.0;
  o[1] = sign > 0 ? b[0] : -b[0];
  o[2] = sign > 0 ? b[1] : -b[1];
  o[3] = sign > 0 ? b[2] : -b[2];
}

// rkf(f, 0, b, x0, tol, hmax, hmin): appends the accepted points (after x0) to
// pts; returns false where rkf raises (step below hmin).
bool rkf_segment(const orc_field* f, double time, double sign, const double* x0, double b, double tol, double hmax,
                 double hmin, std::vector<double>& pts) {
  double t = 0.0, h = hmax, x[4];
  std::memcpy(x, x0, sizeof(x));
  while (t < b) {
    if (t + h > b) h = b - t;
    double k1[4], k2[4], k3[4], k4[4], k5[4], k6[4], xt[4], fv[4];
    fl_deriv(f, time, sign, x, fv);
    for (int i = 0; i < 4; ++i) k1[i] = h * fv[i];
    for (int i = 0; i < 4; ++i) xt[i] = x[i] + rb21 * k1[i];
    fl_deriv(f, time, sign, xt, fv);
    for (int i = 0; i < 4; ++i) k2[i] = h * fv[i];
    for (int i = 0; i < 4; ++i) xt[i] = x[i] + rb31 * k1[i] + rb32 * k2[i];
    fl_deriv(f, time, sign, xt, fv);
    for (int i = 0; i < 4; ++i) k3[i] = h * fv[i];
    for (int i = 0; i < 4; ++i) xt[i] = x[i] + rb41 * k1[i] + rb42 * k2[i] + rb43 * k3[i];
    fl_deriv(f, time, sign, xt, fv);
    for (int i = 0; i < 4; ++i) k4[i] = h * fv[i];
    for (int i = 0; i < 4; ++i) xt[i] = x[i] + rb51 * k1[i] + rb52 * k2[i] + rb53 * k3[i] + rb54 * k4[i];
    fl_deriv(f, time, sign, xt, fv);
    for (int i = 0; i < 4; ++i) k5[i] = h * fv[i];
    for (int i = 0; i < 4; ++i)
      xt[i] = x[i] + rb61 * k1[i] + rb62 * k2[i] + rb63 * k3[i] + rb64 * k4[i] + rb65 * k5[i];
    fl_deriv(f, time, sign, xt, fv);
    for (int i = 0; i < 4; ++i) k6[i] = h * fv[i];
    double r = 0.0;
    for (int i = 0; i < 4; ++i) {
      const double ri = std::fabs(rr1 * k1[i] + rr3 * k3[i] + rr4 * k4[i] + rr5 * k5[i] + rr6 * k6[i]) / h;
      if (i == 0 || ri > r) r = ri;  // numpy max (no NaN expected)
    }
    (void)ra2; (void)ra3; (void)ra4; (void)ra6;  // f does not depend on s
    if (r <= tol) {
      t = t + h;
      for (int i = 0; i < 4; ++i) x[i] = x[i] + rc1 * k1[i] + rc3 * k3[i] + rc4 * k4[i] + rc5 * k5[i];
      pts.insert(pts.end(), x, x + 4);
    }
    const double q = 0.84 * std::pow(tol / r, 0.25);
    h = h * std::fmin(std::fmax(q, 0.1), 4.0);
    if (h > hmax) h = hmax;
    else if (h < hmin) return false;
  }
  return true;
}

// Fieldline(tpos, field, Bmax=Bm).trace(): the (s, |B|) samples of the curve,
// backward part reversed, then the forward part.
void trace_sB(const orc_field* f, const double* tpos, double Bm, double flres, std::vector<double>& s,
              std::vector<double>& B) {
  const double ds = 1.0 / orc_curvature(f, tpos) / flres;  // fieldline.py:31-35
  s.clear();
  B.clear();
  if (!(ds > 0) || !std::isfinite(ds)) return;  // a non-finite start (the device's trace gives up too)
  const double init[4] = {0.0, tpos[1], tpos[2], tpos[3]};
  std::vector<double> fw(init, init + 4), bw(init, init + 4);
  for (int dir = 0; dir < 2; ++dir) {
    std::vector<double>& c = dir == 0 ? fw : bw;
    const double tol = dir == 0 ? 1e-3 : 1e-4;  // fieldline.py:67 and :92
    const double sign = dir == 0 ? 1.0 : -1.0;
    for (long guard = 0; guard < 10000000; ++guard) {
      const double last[4] = {c[c.size() - 4], c[c.size() - 3], c[c.size() - 2], c[c.size() - 1]};
      // rkf raising: the reference keeps none of that call's points (fieldline.py:68-69)
      const size_t before = c.size();
      if (!rkf_segment(f, tpos[0], sign, last, ds, tol, ds, 1e-6, c)) { c.resize(before); break; }
      const double tp[4] = {tpos[0], c[c.size() - 3], c[c.size() - 2], c[c.size() - 1]};
      if (orc_magB(f, tp) > Bm) break;
    }
  }
  const size_t nb = bw.size() / 4, nf = fw.size() / 4;
  s.clear();
  B.clear();
  for (size_t i = nb - 1; i >= 1; --i) {
    s.push_back(bw[4 * i]);
    const double tp[4] = {tpos[0], bw[4 * i + 1], bw[4 * i + 2], bw[4 * i + 3]};
    B.push_back(orc_magB(f, tp));
  }
  for (size_t i = 0; i < nf; ++i) {
    s.push_back(fw[4 * i]);
    const double tp[4] = {tpos[0], fw[4 * i + 1], fw[4 * i + 2], fw[4 * i + 3]};
    B.push_back(orc_magB(f, tp));
  }
}

// ---------------------------------------------------------------- quadratic spline
// Interpolating B-spline of degree 2 (scipy make_interp_spline, k = 2): knots
// x0 x0 x0, midpoints of (x1,x2) ... (x_{n-3},x_{n-2}), x_{n-1} x3.
struct Spline2 {
  std::vector<double> t, c;
  int n = 0;
  int find(double x) const {  // t[l] <= x < t[l+1], l in [2, n-1]
    int lo = 2, hi = n;          // t[n] is the last data point
    if (x >= t[n]) return n - 1;
    while (hi - lo > 1) {
      const int mid = (lo + hi) / 2;
      if (x < t[mid]) hi = mid; else lo = mid;
    }
    return lo;
  }
  void basis(double x, int l, double* h) const {  // Cox-de Boor, scipy _deBoor_D (nu = 0)
    double hh[3];
    h[0] = 1.0;
    for (int j = 1; j <= 2; ++j) {
      for (int i = 0; i < j; ++i) hh[i] = h[i];
      h[0] = 0.0;
      for (int m = 1; m <= j; ++m) {
        const int ind = l + m;
        const double xb = t[ind], xa = t[ind - j];
        if (xb == xa) { h[m] = 0.0; continue; }
        const double w = hh[m - 1] / (xb - xa);
        h[m - 1] += w * (xb - x);
        h[m] = w * (x - xa);
      }
    }
  }
  double operator()(double x) const {
    const int l = find(x);
    double h[3];
    basis(x, l, h);
    double y = 0.0;
    for (int a = 0; a <= 2; ++a) y += c[l + a - 2] * h[a];
    return y;
  }
  void build(const double* x, const double* y, int nn) {
    n = nn;
    t.assign(n + 3, 0.0);
    t[0] = t[1] = t[2] = x[0];
    for (int i = 1; i <= n - 3; ++i) t[2 + i] = (x[i] + x[i + 1]) / 2.0;
    t[n] = t[n + 1] = t[n + 2] = x[n - 1];
    // collocation rows: the basis functions j = l-2..l at x_i; with these knots
    // x_i lies in [t[i+1], t[i+2]), so row i couples coefficients i-1, i, i+1
    // (the first and last rows are unit rows): a tridiagonal system, solved
    // by elimination without pivoting (the matrix is diagonally dominant).
    std::vector<double> lo(n, 0.0), di(n, 0.0), up(n, 0.0);
    for (int i = 0; i < n; ++i) {
      const int l = find(x[i]);
      double h[3];
      basis(x[i], l, h);
      for (int a = 0; a <= 2; ++a) {
        const int j = l + a - 2;
        if (j == i - 1) lo[i] = h[a];
        else if (j == i) di[i] = h[a];
        else if (j == i + 1) up[i] = h[a];
      }
    }
    c.assign(y, y + n);
    for (int i = 1; i < n; ++i) {
      const double m = lo[i] / di[i - 1];
      di[i] -= m * up[i - 1];
      c[i] -= m * c[i - 1];
    }
    c[n - 1] /= di[n - 1];
    for (int i = n - 2; i >= 0; --i) c[i] = (c[i] - up[i] * c[i + 1]) / di[i];
  }
};

// ---------------------------------------------------------------- brentq (SciPy Zeros/brentq.c)
template <class F>
double brentq(F&& f, double xa, double xb, double xtol, double rtol, int iter) {
  double xpre = xa, xcur = xb, xblk = 0.0, fpre, fcur, fblk = 0.0, spre = 0.0, scur = 0.0, sbis;
  fpre = f(xpre);
  fcur = f(xcur);
  if (fpre == 0) return xpre;
  if (fcur == 0) return xcur;
  for (int i = 0; i < iter; ++i) {
    if (fpre != 0 && fcur != 0 && (std::signbit(fpre) != std::signbit(fcur))) {
      xblk = xpre;
      fblk = fpre;
      spre = scur = xcur - xpre;
    }
    if (std::fabs(fblk) < std::fabs(fcur)) {
      xpre = xcur; xcur = xblk; xblk = xpre;
      fpre = fcur; fcur = fblk; fblk = fpre;
    }
    const double delta = (xtol + rtol * std::fabs(xcur)) / 2;
    sbis = (xblk - xcur) / 2;
    if (fcur == 0 || std::fabs(sbis) < delta) return xcur;
    if (std::fabs(spre) > delta && std::fabs(fcur) < std::fabs(fpre)) {
      double stry;
      if (xpre == xblk) {
        stry = -fcur * (xcur - xpre) / (fcur - fpre);
      } else {
        const double dpre = (fpre - fcur) / (xpre - xcur);
        const double dblk = (fblk - fcur) / (xblk - xcur);
        stry = -fcur * (fblk * dblk - fpre * dpre) / (dblk * dpre * (fblk - fpre));
      }
      if (2 * std::fabs(stry) < std::fmin(std::fabs(spre), 3 * std::fabs(sbis) - delta)) {
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
    if (std::fabs(scur) > delta) xcur += scur;
    else xcur += (sbis > 0 ? delta : -delta);
    fcur = f(xcur);
  }
  return xcur;
}

// ---------------------------------------------------------------- QUADPACK QAGS
const double xgk[11] = {0.995657163025808080735527280689003, 0.973906528517171720077964012084452,
                        0.930157491355708226001207180059508, 0.865063366688984510732096688423493,
                        0.780817726586416897063717578345042, 0.679409568299024406234327365114874,
                        0.562757134668604683339000099272694, 0.433395394129247190799265943165784,
                        0.294392862701460198131126603103866, 0.148874338981631210884826001129720, 0.0};
const double wgk[11] = {0.011694638867371874278064396062192, 0.032558162307964727478818972459390,
                        0.054755896574351996031381300244580, 0.075039674810919952767043140916190,
                        0.093125454583697605535065465083366, 0.109387158802297641899210590325805,
                        0.123491976262065851077958109831074, 0.134709217311473325928054001771707,
                        0.142775938577060080797094273138717, 0.147739104901338491374841515972068,
                        0.149445554002916905664936468389821};
const double wg[5] = {0.066671344308688137593568809893332, 0.149451349150580593145776339657697,
                      0.219086362515982043995534934228163, 0.269266719309996355091226921569469,
                      0.295524224714752870173892994651338};

template <class F>
void qk21(F&& f, double a, double b, double& result, double& abserr, double& resabs, double& resasc) {
  const double epmach = DBL_EPSILON, uflow = DBL_MIN;
  const double centr = 0.5 * (a + b), hlgth = 0.5 * (b - a), dhlgth = std::fabs(hlgth);
  double resg = 0.0, fv1[10], fv2[10];
  const double fc = f(centr);
  double resk = wgk[10] * fc;
  resabs = std::fabs(resk);
  for (int j = 1; j <= 5; ++j) {
    const int jtw = 2 * j;  // Fortran index
    const double absc = hlgth * xgk[jtw - 1];
    const double fval1 = f(centr - absc), fval2 = f(centr + absc);
    fv1[jtw - 1] = fval1;
    fv2[jtw - 1] = fval2;
    const double fsum = fval1 + fval2;
    resg = resg + wg[j - 1] * fsum;
    resk = resk + wgk[jtw - 1] * fsum;
    resabs = resabs + wgk[jtw - 1] * (std::fabs(fval1) + std::fabs(fval2));
  }
  for (int j = 1; j <= 5; ++j) {
    const int jtwm1 = 2 * j - 1;
    const double absc = hlgth * xgk[jtwm1 - 1];
    const double fval1 = f(centr - absc), fval2 = f(centr + absc);
    fv1[jtwm1 - 1] = fval1;
    fv2[jtwm1 - 1] = fval2;
    const double fsum = fval1 + fval2;
    resk = resk + wgk[jtwm1 - 1] * fsum;
    resabs = resabs + wgk[jtwm1 - 1] * (std::fabs(fval1) + std::fabs(fval2));
  }
  const double reskh = resk * 0.5;
  resasc = wgk[10] * std::fabs(fc - reskh);
  for (int j = 0; j < 10; ++j) resasc = resasc + wgk[j] * (std::fabs(fv1[j] - reskh) + std::fabs(fv2[j] - reskh));
  result = resk * hlgth;
  resabs = resabs * dhlgth;
  resasc = resasc * dhlgth;
  abserr = std::fabs((resk - resg) * hlgth);
  if (resasc != 0.0 && abserr != 0.0) abserr = resasc * std::fmin(1.0, std::pow(200.0 * abserr / resasc, 1.5));
  if (resabs > uflow / (50.0 * epmach)) abserr = std::fmax((epmach * 50.0) * resabs, abserr);
}

void qpsrt(int limit, int last, int& maxerr, double& ermax, const double* elist, int* iord, int& nrmax) {
  // 1-based arrays emulated with index - 1
  auto E = [&](int i) { return elist[i - 1]; };
  auto I = [&](int i) -> int& { return iord[i - 1]; };
  int i = 0, k, isucc;
  if (last <= 2) {
    I(1) = 1;
    I(2) = 2;
    goto L90;
  }
  {
    const double errmax = E(maxerr);
    if (nrmax != 1) {
      const int ido = nrmax - 1;
      for (int ii = 1; ii <= ido; ++ii) {
        isucc = I(nrmax - 1);
        if (errmax <= E(isucc)) break;
        I(nrmax) = isucc;
        nrmax = nrmax - 1;
      }
    }
    int jupbn = last;
    if (last > (limit / 2 + 2)) jupbn = limit + 3 - last;
    const double errmin = E(last);
    const int jbnd = jupbn - 1;
    const int ibeg = nrmax + 1;
    bool found = false;
    if (ibeg <= jbnd) {
      for (i = ibeg; i <= jbnd; ++i) {
        isucc = I(i);
        if (errmax >= E(isucc)) { found = true; break; }
        I(i - 1) = isucc;
      }
    }
    if (!found) {
      I(jbnd) = maxerr;
      I(jupbn) = last;
      goto L90;
    }
    I(i - 1) = maxerr;
    k = jbnd;
    for (int j = i; j <= jbnd; ++j) {
      isucc = I(k);
      if (errmin < E(isucc)) {
        I(k + 1) = last;
        goto L90;
      }
      I(k + 1) = isucc;
      k = k - 1;
    }
    I(i) = last;
  }
L90:
  maxerr = I(nrmax);
  ermax = E(maxerr);
}

void qelg(int& n, double* epstab, double& result, double& abserr, double* res3la, int& nres) {
  // epstab[1..52], res3la[1..3] (1-based views)
  const double epmach = DBL_EPSILON, oflow = DBL_MAX;
  auto T = [&](int i) -> double& { return epstab[i - 1]; };
  auto R = [&](int i) -> double& { return res3la[i - 1]; };
  nres = nres + 1;
  abserr = oflow;
  result = T(n);
  if (n < 3) goto L100;
  {
    const int limexp = 50;
    T(n + 2) = T(n);
    const int newelm = (n - 1) / 2;
    T(n) = oflow;
    const int num = n;
    int k1 = n;
    bool shifted = false;
    for (int i = 1; i <= newelm; ++i) {
      const int k2 = k1 - 1, k3 = k1 - 2;
      double res = T(k1 + 2);
      const double e0 = T(k3), e1 = T(k2), e2 = res;
      const double e1abs = std::fabs(e1);
      const double delta2 = e2 - e1, err2 = std::fabs(delta2);
      const double tol2 = std::fmax(std::fabs(e2), e1abs) * epmach;
      const double delta3 = e1 - e0, err3 = std::fabs(delta3);
      const double tol3 = std::fmax(e1abs, std::fabs(e0)) * epmach;
      if (!(err2 > tol2 || err3 > tol3)) {
        result = res;
        abserr = err2 + err3;
        goto L100;
      }
      const double e3 = T(k1);
      T(k1) = e1;
      const double delta1 = e1 - e3, err1 = std::fabs(delta1);
      const double tol1 = std::fmax(e1abs, std::fabs(e3)) * epmach;
      if (err1 <= tol1 || err2 <= tol2 || err3 <= tol3) {
        n = i + i - 1;
        shifted = true;
        break;
      }
      const double ss = 1.0 / delta1 + 1.0 / delta2 - 1.0 / delta3;
      const double epsinf = std::fabs(ss * e1);
      if (!(epsinf > 1.0e-4)) {
        n = i + i - 1;
        shifted = true;
        break;
      }
      res = e1 + 1.0 / ss;
      T(k1) = res;
      k1 = k1 - 2;
      const double error = err2 + std::fabs(res - e2) + err3;
      if (!(error > abserr)) {
        abserr = error;
        result = res;
      }
    }
    (void)shifted;
    if (n == limexp) n = 2 * (limexp / 2) - 1;
    int ib = ((num / 2) * 2 == num) ? 2 : 1;
    const int ie = newelm + 1;
    for (int i = 1; i <= ie; ++i) {
      const int ib2 = ib + 2;
      T(ib) = T(ib2);
      ib = ib2;
    }
    if (num != n) {
      int indx = num - n + 1;
      for (int i = 1; i <= n; ++i) {
        T(i) = T(indx);
        indx = indx + 1;
      }
    }
    if (nres < 4) {
      R(nres) = result;
      abserr = oflow;
      goto L100;
    }
    abserr = std::fabs(result - R(3)) + std::fabs(result - R(2)) + std::fabs(result - R(1));
    R(1) = R(2);
    R(2) = R(3);
    R(3) = result;
  }
L100:
  abserr = std::fmax(abserr, 5.0 * epmach * std::fabs(result));
}

template <class F>
double qags(F&& f, double a, double b, double epsabs, double epsrel, int limit, int& ier) {
  const double epmach = DBL_EPSILON, uflow = DBL_MIN, oflow = DBL_MAX;
  std::vector<double> alist(limit + 1), blist(limit + 1), rlist(limit + 1), elist(limit + 1);
  std::vector<int> iord(limit + 1);
  double rlist2[52], res3la[3];
  auto AL = [&](int i) -> double& { return alist[i - 1]; };
  auto BL = [&](int i) -> double& { return blist[i - 1]; };
  auto RL = [&](int i) -> double& { return rlist[i - 1]; };
  auto EL = [&](int i) -> double& { return elist[i - 1]; };
  auto IO = [&](int i) -> int& { return iord[i - 1]; };
  auto R2 = [&](int i) -> double& { return rlist2[i - 1]; };
  ier = 0;
  int last = 0;
  double result = 0.0, abserr = 0.0;
  AL(1) = a;
  BL(1) = b;
  RL(1) = 0.0;
  EL(1) = 0.0;
  double defabs, resabs, area, errsum, errmax, erlarg = 0, ertest = 0, small = 0, correc = 0, erlast, area1,
         area2, error1, error2, defab1, defab2, area12, erro12, a1, a2, b1, b2, reseps, abseps, dres, errbnd;
  int maxerr, nrmax, nres, numrl2, ktmin, ierro, iroff1, iroff2, iroff3, ksgn;
  bool extrap, noext;
  ierro = 0;
  qk21(f, a, b, result, abserr, defabs, resabs);
  dres = std::fabs(result);
  errbnd = std::fmax(epsabs, epsrel * dres);
  last = 1;
  RL(1) = result;
  EL(1) = abserr;
  IO(1) = 1;
  if (abserr <= 100.0 * epmach * defabs && abserr > errbnd) ier = 2;
  if (limit == 1) ier = 1;
  if (ier != 0 || (abserr <= errbnd && abserr != resabs) || abserr == 0.0) goto L140;
  R2(1) = result;
  errmax = abserr;
  maxerr = 1;
  area = result;
  errsum = abserr;
  abserr = oflow;
  nrmax = 1;
  nres = 0;
  numrl2 = 2;
  ktmin = 0;
  extrap = false;
  noext = false;
  iroff1 = iroff2 = iroff3 = 0;
  ksgn = -1;
  if (dres >= (1.0 - 50.0 * epmach) * defabs) ksgn = 1;
  for (last = 2; last <= limit; ++last) {
    a1 = AL(maxerr);
    b1 = 0.5 * (AL(maxerr) + BL(maxerr));
    a2 = b1;
    b2 = BL(maxerr);
    erlast = errmax;
    qk21(f, a1, b1, area1, error1, resabs, defab1);
    qk21(f, a2, b2, area2, error2, resabs, defab2);
    area12 = area1 + area2;
    erro12 = error1 + error2;
    errsum = errsum + erro12 - errmax;
    area = area + area12 - RL(maxerr);
    if (defab1 != error1 && defab2 != error2) {
      if (std::fabs(RL(maxerr) - area12) <= 1.0e-5 * std::fabs(area12) && erro12 >= 0.99 * errmax) {
        if (extrap) iroff2 = iroff2 + 1;
        else iroff1 = iroff1 + 1;
      }
      if (last > 10 && erro12 > errmax) iroff3 = iroff3 + 1;
    }
    RL(maxerr) = area1;
    RL(last) = area2;
    errbnd = std::fmax(epsabs, epsrel * std::fabs(area));
    if (iroff1 + iroff2 >= 10 || iroff3 >= 20) ier = 2;
    if (iroff2 >= 5) ierro = 3;
    if (last == limit) ier = 1;
    if (std::fmax(std::fabs(a1), std::fabs(b2)) <= (1.0 + 100.0 * epmach) * (std::fabs(a2) + 1000.0 * uflow)) ier = 4;
    if (error2 > error1) {
      AL(maxerr) = a2;
      AL(last) = a1;
      BL(last) = b1;
      RL(maxerr) = area2;
      RL(last) = area1;
      EL(maxerr) = error2;
      EL(last) = error1;
    } else {
      AL(last) = a2;
      BL(maxerr) = b1;
      BL(last) = b2;
      EL(maxerr) = error1;
      EL(last) = error2;
    }
    qpsrt(limit, last, maxerr, errmax, elist.data(), iord.data(), nrmax);
    if (errsum <= errbnd) goto L115;
    if (ier != 0) goto L100;
    if (last == 2) {
      small = std::fabs(b - a) * 0.375;
      erlarg = errsum;
      ertest = errbnd;
      R2(2) = area;
      continue;
    }
    if (noext) continue;
    erlarg = erlarg - erlast;
    if (std::fabs(b1 - a1) > small) erlarg = erlarg + erro12;
    if (!extrap) {
      if (std::fabs(BL(maxerr) - AL(maxerr)) > small) continue;
      extrap = true;
      nrmax = 2;
    }
    {
      bool go_extrap = true;
      if (ierro != 3 && erlarg > ertest) {
        const int id = nrmax;
        int jupbnd = last;
        if (last > (2 + limit / 2)) jupbnd = limit + 3 - last;
        for (int k = id; k <= jupbnd; ++k) {
          maxerr = IO(nrmax);
          errmax = EL(maxerr);
          if (std::fabs(BL(maxerr) - AL(maxerr)) > small) { go_extrap = false; break; }
          nrmax = nrmax + 1;
        }
      }
      if (!go_extrap) continue;
    }
    numrl2 = numrl2 + 1;
    R2(numrl2) = area;
    qelg(numrl2, rlist2, reseps, abseps, res3la, nres);
    ktmin = ktmin + 1;
    if (ktmin > 5 && abserr < 1.0e-3 * errsum) ier = 5;
    if (abseps < abserr) {
      ktmin = 0;
      abserr = abseps;
      result = reseps;
      correc = erlarg;
      ertest = std::fmax(epsabs, epsrel * std::fabs(reseps));
      if (abserr <= ertest) goto L100;
    }
    if (numrl2 == 1) noext = true;
    if (ier == 5) goto L100;
    maxerr = IO(1);
    errmax = EL(maxerr);
    nrmax = 1;
    extrap = false;
    small = small * 0.5;
    erlarg = errsum;
  }
L100:
  if (abserr == oflow) goto L115;
  if (ier + ierro != 0) {
    if (ierro == 3) abserr = abserr + correc;
    if (ier == 0) ier = 3;
    if (result != 0.0 && area != 0.0) {
      if (abserr / std::fabs(result) > errsum / std::fabs(area)) goto L115;
    } else if (abserr > errsum) {
      goto L115;
    } else if (area == 0.0) {
      goto L130;
    }
  }
  if (!(ksgn == -1 && std::fmax(std::fabs(result), std::fabs(area)) <= defabs * 0.01)) {
    if (0.01 > (result / area) || (result / area) > 100.0 || errsum > std::fabs(area)) ier = 6;
  }
  goto L130;
L115:
  result = 0.0;
  for (int k = 1; k <= last; ++k) result = result + RL(k);
  abserr = errsum;
L130:
  if (ier > 2) ier = ier - 1;
L140:
  (void)abserr;
  return result;
}

// Gauss-Legendre nodes and weights of order 8 by Newton's method on P_8.
void gauss_legendre8(double* x, double* w) {
  const int n = 8;
  for (int i = 0; i < n / 2; ++i) {
    double z = std::cos(kPiF * (i + 0.75) / (n + 0.5)), pp = 0.0;
    for (int it = 0; it < 100; ++it) {
      double p1 = 1.0, p2 = 0.0;
      for (int j = 1; j <= n; ++j) {
        const double p3 = p2;
        p2 = p1;
        p1 = ((2.0 * j - 1.0) * z * p2 - (j - 1.0) * p3) / j;
      }
      pp = n * (z * p1 - p2) / (z * z - 1.0);
      const double z1 = z;
      z = z1 - p1 / pp;
      if (std::fabs(z - z1) <= 1e-16) break;
    }
    x[i] = -z;
    x[n - 1 - i] = z;
    w[i] = w[n - 1 - i] = 2.0 / ((1.0 - z * z) * pp * pp);
  }
}

// The half-bounce integral of the spline to convergence (the device's method):
// s = c + h sin(theta) removes the inverse-square-root singularities at the
// mirror points, and an 8-point Gauss-Legendre rule runs on every panel between
// the images of the spline's knots (each panel a smooth polynomial piece).
// The same rule for the second invariant's integrand sqrt(1 - B(s)/Bm), which
// the substitution leaves smooth as well.
double eye_integral_converged(const Spline2& sp, double sm1, double sm2, double Bm) {
  double gx[8], gw[8];
  gauss_legendre8(gx, gw);
  const double c = 0.5 * (sm1 + sm2), h = 0.5 * (sm2 - sm1);
  double sum = 0.0, ea = -kPiF / 2;
  for (int j = 3; j <= sp.n; ++j) {
    double eb;
    if (j < sp.n) {
      const double tj = sp.t[j];
      if (!(tj > sm1 && tj < sm2)) continue;
      eb = std::asin((tj - c) / h);
    } else {
      eb = kPiF / 2;
    }
    const double mid = 0.5 * (ea + eb), half = 0.5 * (eb - ea);
    double ps = 0.0;
    for (int k = 0; k < 8; ++k) {
      const double th = mid + half * gx[k];
      const double arg = 1.0 - sp(c + h * std::sin(th)) / Bm;
      if (arg > 0.0) ps += gw[k] * (h * std::cos(th) * std::sqrt(arg));
    }
    sum += half * ps;
    ea = eb;
  }
  return sum;
}

double bounce_integral_converged(const Spline2& sp, double sm1, double sm2, double Bm) {
  double gx[8], gw[8];
  gauss_legendre8(gx, gw);
  const double c = 0.5 * (sm1 + sm2), h = 0.5 * (sm2 - sm1);
  double sum = 0.0, ea = -kPiF / 2;
  for (int j = 3; j <= sp.n; ++j) {
    double eb;
    if (j < sp.n) {
      const double tj = sp.t[j];
      if (!(tj > sm1 && tj < sm2)) continue;
      eb = std::asin((tj - c) / h);
    } else {
      eb = kPiF / 2;
    }
    const double mid = 0.5 * (ea + eb), half = 0.5 * (eb - ea);
    double ps = 0.0;
    for (int k = 0; k < 8; ++k) {
      const double th = mid + half * gx[k];
      const double arg = 1.0 - sp(c + h * std::sin(th)) / Bm;
      if (arg > 0.0) ps += gw[k] * (h * std::cos(th) / std::sqrt(arg));
    }
    sum += half * ps;
    ea = eb;
  }
  return sum;
}

}  // namespace

extern "C" {

double orc_qags_test(int which, double a, double b, double epsabs, double epsrel, int limit, int* ier) {
  // test integrands for pinning qags against scipy.integrate.quad
  auto f = [which](double x) -> double {
    switch (which) {
      case 0: return 1.0 / std::sqrt(x);                   // endpoint singularity on [0, b]
      case 1: return std::log(x) * std::sqrt(x);           // smooth-ish
      case 2: return 1.0 / std::sqrt(1.0 - x * x);         // both endpoints singular on [-1, 1]
      case 3: return std::cos(50.0 * x) * std::exp(-x);    // oscillatory
      default: return std::exp(-x * x);
    }
  };
  int e = 0;
  const double r = qags(f, a, b, epsabs, epsrel, limit, e);
  if (ier) *ier = e;
  return r;
}

int orc_fieldline_sB(const orc_field* f, const double* tpos, double Bm, double flres, double* s, double* B,
                     int cap) {
  std::vector<double> sv, bv;
  trace_sB(f, tpos, Bm, flres, sv, bv);
  const int n = (int)sv.size();
  for (int i = 0; i < n && i < cap; ++i) { s[i] = sv[i]; B[i] = bv[i]; }
  return n;
}

double orc_halfbouncepath(const orc_field* f, const double* tpos, double Bm, double flres, int quad, int* npts) {
  // flutils.halfbouncepath, rapt/flutils.py:254-316
  std::vector<double> s, b;
  trace_sB(f, tpos, Bm, flres, s, b);
  int n = (int)b.size();
  int first = -1, lastin = -1;
  for (int i = 0; i < n; ++i)
    if (b[i] <= Bm) {
      if (first < 0) first = i;
      lastin = i;
    }
  int i1, i2;
  if (first < 0) {
    i1 = (n - 3) / 2;
    i2 = (n + 1) / 2;
  } else {
    i1 = first - 1;
    i2 = lastin + 1;
  }
  // np.delete(range(0, i1) + range(i2 + 1, n)): keep max(i1, 0) .. min(i2, n - 1)
  const int lo = i1 < 0 ? 0 : i1, hi = i2 > n - 1 ? n - 1 : i2;
  std::vector<double> ss(s.begin() + lo, s.begin() + hi + 1), bb(b.begin() + lo, b.begin() + hi + 1);
  n = (int)bb.size();
  if (npts) *npts = n;
  if (n == 3) {  // equatorial: pi sqrt(2 Bm / B''), B'' by the quadratic through the three points
    const double s1 = ss[0], s2 = ss[1], s3 = ss[2], B1 = bb[0], B2 = bb[1], B3 = bb[2];
    const double s12 = s1 - s2, s23 = s2 - s3, s13 = s1 - s3;
    const double B2s = 2 * (B1 * s23 - B2 * s13 + B3 * s12) / (s12 * s13 * s23);
    return kPiF * std::sqrt(2 * Bm / B2s);
  }
  Spline2 sp;
  sp.build(ss.data(), bb.data(), n);
  auto g = [&](double x) { return sp(x) - Bm; };
  const double xtol = 2e-12, rtol = 4 * DBL_EPSILON;
  const double sm1 = brentq(g, ss[0], ss[1], xtol, rtol, 100);
  const double sm2 = brentq(g, ss[n - 2], ss[n - 1], xtol, rtol, 100);
  if (quad == 1) return bounce_integral_converged(sp, sm1, sm2, Bm);
  int ier = 0;
  return qags([&](double x) { return 1 / std::sqrt(1 - sp(x) / Bm); }, sm1, sm2, 1.49e-8, 1e-4, 50, ier);
}

double orc_eye(const orc_field* f, const double* tpos, double Bm, double flres, int quad) {
  // flutils.eye, rapt/flutils.py:65-151 (usedipole False). quad 0: as the
  // reference -- equatorial pitch angles below 70 degrees take its Simpson
  // branch, which calls the undefined name simps (flutils.py:18, :130) and
  // raises NameError: NaN here; 70 and above: quadratic spline, brentq mirror
  // points, QAGS at epsrel 1e-4. quad 1: the spline branch at every pitch angle,
  // integrated to convergence (the device's method).
  std::vector<double> s, b;
  trace_sB(f, tpos, Bm, flres, s, b);
  const int n0 = (int)b.size();
  if (n0 == 0) return NAN;
  double Bmin = b[0];
  for (int i = 1; i < n0; ++i) Bmin = std::min(Bmin, b[i]);
  if (Bmin > Bm) return 0.0;
  if (std::fabs(Bmin - Bm) / Bm < 1e-12) return 0.0;  // equatorial particle
  int first = -1, last = -1;
  for (int i = 0; i < n0; ++i)
    if (b[i] < Bm) {
      if (first < 0) first = i;
      last = i;
    }
  // np.delete of range(0, first - 1) and range(last + 2, n): keep first-1 .. last+1
  const int lo = std::max(first - 1, 0), hi = std::min(last + 1, n0 - 1);
  std::vector<double> ss(s.begin() + lo, s.begin() + hi + 1), bb(b.begin() + lo, b.begin() + hi + 1);
  const int n = (int)bb.size();
  if (!(n >= 3 && bb[0] > Bm && bb[1] < Bm && bb[n - 2] < Bm && bb[n - 1] > Bm)) return NAN;  // AssertionError
  const double eqpa = std::asin(std::sqrt(Bmin / Bm)) * 180 / kPiF;
  if (quad == 0 && eqpa < 70) return NAN;  // NameError in the reference
  Spline2 sp;
  sp.build(ss.data(), bb.data(), n);
  auto g = [&](double x) { return sp(x) - Bm; };
  const double xtol = 2e-12, rtol = 4 * DBL_EPSILON;
  const double sm1 = brentq(g, ss[0], ss[1], xtol, rtol, 100);
  const double sm2 = sp(ss[n - 2]) == Bm ? ss[n - 2] : brentq(g, ss[n - 2], ss[n - 1], xtol, rtol, 100);
  if (quad == 1) return eye_integral_converged(sp, sm1, sm2, Bm);
  int ier = 0;
  return qags([&](double x) { return std::sqrt(1 - sp(x) / Bm); }, sm1, sm2, 1.49e-8, 1e-4, 50, ier);
}

void orc_gradI(const orc_field* f, const double* tpos, double Bm, double d, double flres, int quad, double* out) {
  // flutils.gradI, rapt/flutils.py:153-229 (usedipole False): central differences
  // of I over d in two directions perpendicular to b, one-sided where an end
  // has I = 0
  const double x = tpos[1], y = tpos[2];
  const double sc = std::max(std::fabs(x), std::fabs(y));
  double r[3] = {x / sc, y / sc, 0.0 / sc};
  double b[3];
  orc_unitb(f, tpos, b);
  const double rb = r[0] * b[0] + r[1] * b[1] + r[2] * b[2];
  for (int i = 0; i < 3; ++i) r[i] = r[i] - rb * b[i];
  const double rn = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
  for (int i = 0; i < 3; ++i) r[i] = r[i] / rn;
  const double v2[3] = {b[1] * r[2] - b[2] * r[1], b[2] * r[0] - b[0] * r[2], b[0] * r[1] - b[1] * r[0]};
  const double* dirs[2] = {r, v2};
  double dI[2];
  for (int k = 0; k < 2; ++k) {
    const double* v = dirs[k];
    double tp[4] = {tpos[0], tpos[1] + d * v[0], tpos[2] + d * v[1], tpos[3] + d * v[2]};
    double tm[4] = {tpos[0], tpos[1] - d * v[0], tpos[2] - d * v[1], tpos[3] - d * v[2]};
    const double I1 = orc_eye(f, tp, Bm, flres, quad), I2 = orc_eye(f, tm, Bm, flres, quad);
    if (I1 == 0) dI[k] = (orc_eye(f, tpos, Bm, flres, quad) - I2) / d;
    else if (I2 == 0) dI[k] = (I1 - orc_eye(f, tpos, Bm, flres, quad)) / d;
    else dI[k] = (I1 - I2) / (2 * d);
  }
  for (int i = 0; i < 3; ++i) out[i] = dI[0] * r[i] + dI[1] * v2[i];
}

double orc_gc_bounceperiod(const orc_field* f, const orc_tracer* g, double flres, int quad) {
  // GuidingCenter.bounceperiod, rapt/GuidingCenter.py:593-606 (state = trajectory[-1])
  const double c = 299792458.0;
  const double tpos[4] = {g->t, g->s[0], g->s[1], g->s[2]};
  const double ppar = g->s[3], m = g->mass, mu = g->mu;
  const double Bmag = orc_magB(f, tpos);
  const double gamma = std::sqrt(1 + 2 * mu * Bmag / (m * c * c) + (ppar / (m * c)) * (ppar / (m * c)));
  double p, v, Bmirror;
  if (gamma - 1 < 1e-6) {
    p = std::sqrt(2 * m * mu * Bmag + ppar * ppar);
    v = p / m;
    Bmirror = (p * p) / (2 * m * mu);
  } else {
    p = m * c * std::sqrt((gamma + 1) * (gamma - 1));
    Bmirror = p * p / ((p - ppar) * (p + ppar)) * Bmag;
    v = p / m / gamma;
  }
  return (2 / v) * orc_halfbouncepath(f, tpos, Bmirror, flres, quad, nullptr);
}

}  // extern "C"
