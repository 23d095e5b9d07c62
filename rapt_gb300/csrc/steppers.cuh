// steppers.cuh -- one embedded Runge-Kutta step per call, in registers.
//
// The methods are the published Dormand-Prince pairs with the controller of
// Hairer's DOPRI5/DOP853 codes that SciPy's `ode` dopri5/dop853 integrators
// wrap (Hairer, Norsett & Wanner, Solving ODEs I, Sec. II.4-II.5, II.10), and
// Fehlberg's 4(5) pair as restated from rapt/rkf.py:48-87. The tableau values
// are the published coefficients; they have to be the same numbers.
#pragma once
#include "common.cuh"

namespace rapt {

namespace dp5 {
constexpr double c2 = 0.2, c3 = 0.3, c4 = 0.8, c5 = 8.0 / 9.0;
constexpr double a21 = 0.2, a31 = 3.0 / 40.0, a32 = 9.0 / 40.0;
constexpr double a41 = 44.0 / 45.0, a42 = -56.0 / 15.0, a43 = 32.0 / 9.0;
constexpr double a51 = 19372.0 / 6561.0, a52 = -25360.0 / 2187.0, a53 = 64448.0 / 6561.0, a54 = -212.0 / 729.0;
constexpr double a61 = 9017.0 / 3168.0, a62 = -355.0 / 33.0, a63 = 46732.0 / 5247.0, a64 = 49.0 / 176.0,
                 a65 = -5103.0 / 18656.0;
constexpr double a71 = 35.0 / 384.0, a73 = 500.0 / 1113.0, a74 = 125.0 / 192.0, a75 = -2187.0 / 6784.0,
                 a76 = 11.0 / 84.0;
constexpr double e1 = 71.0 / 57600.0, e3 = -71.0 / 16695.0, e4 = 71.0 / 1920.0, e5 = -17253.0 / 339200.0,
                 e6 = 22.0 / 525.0, e7 = -1.0 / 40.0;
// continuous extension of order 4 (Hairer, Norsett & Wanner, Solving ODEs I, II.6;
// the coefficients of the DOPRI5 code's dense output)
constexpr double d1 = -12715105075.0 / 11282082432.0, d3 = 87487479700.0 / 32700410799.0,
                 d4 = -10690763975.0 / 1880347072.0, d5 = 701980252875.0 / 199316789632.0,
                 d6 = -1453857185.0 / 822651844.0, d7 = 69997945.0 / 29380423.0;
}  // namespace dp5

namespace dp8 {
constexpr double c2 = 0.526001519587677318785587544488e-01, c3 = 0.789002279381515978178381316732e-01,
                 c4 = 0.118350341907227396726757197510e+00, c5 = 0.281649658092772603273242802490e+00,
                 c6 = 0.333333333333333333333333333333e+00, c7 = 0.25e+00,
                 c8 = 0.307692307692307692307692307692e+00, c9 = 0.651282051282051282051282051282e+00,
                 c10 = 0.6e+00, c11 = 0.857142857142857142857142857142e+00;
constexpr double b1 = 5.42937341165687622380535766363e-2, b6 = 4.45031289275240888144113950566e0,
                 b7 = 1.89151789931450038304281599044e0, b8 = -5.8012039600105847814672114227e0,
                 b9 = 3.1116436695781989440891606237e-1, b10 = -1.52160949662516078556178806805e-1,
                 b11 = 2.01365400804030348374776537501e-1, b12 = 4.47106157277725905176885569043e-2;
constexpr double bhh1 = 0.244094488188976377952755905512e+00, bhh2 = 0.733846688281611857341361741547e+00,
                 bhh3 = 0.220588235294117647058823529412e-01;
constexpr double er1 = 0.1312004499419488073250102996e-01, er6 = -0.1225156446376204440720569753e+01,
                 er7 = -0.4957589496572501915214079952e+00, er8 = 0.1664377182454986536961530415e+01,
                 er9 = -0.3503288487499736816886487290e+00, er10 = 0.3341791187130174790297318841e+00,
                 er11 = 0.8192320648511571246570742613e-01, er12 = -0.2235530786388629525884427845e-01;
constexpr double a21 = 5.26001519587677318785587544488e-2, a31 = 1.97250569845378994544595329183e-2,
                 a32 = 5.91751709536136983633785987549e-2, a41 = 2.95875854768068491816892993775e-2,
                 a43 = 8.87627564304205475450678981324e-2, a51 = 2.41365134159266685502369798665e-1,
                 a53 = -8.84549479328286085344864962717e-1, a54 = 9.24834003261792003115737966543e-1,
                 a61 = 3.7037037037037037037037037037e-2, a64 = 1.70828608729473871279604482173e-1,
                 a65 = 1.25467687566822425016691814123e-1, a71 = 3.7109375e-2,
                 a74 = 1.70252211019544039314978060272e-1, a75 = 6.02165389804559606850219397283e-2,
                 a76 = -1.7578125e-2, a81 = 3.70920001185047927108779319836e-2,
                 a84 = 1.70383925712239993810214054705e-1, a85 = 1.07262030446373284651809199168e-1,
                 a86 = -1.53194377486244017527936158236e-2, a87 = 8.27378916381402288758473766002e-3,
                 a91 = 6.24110958716075717114429577812e-1, a94 = -3.36089262944694129406857109825e0,
                 a95 = -8.68219346841726006818189891453e-1, a96 = 2.75920996994467083049415600797e1,
                 a97 = 2.01540675504778934086186788979e1, a98 = -4.34898841810699588477366255144e1,
                 a101 = 4.77662536438264365890433908527e-1, a104 = -2.48811461997166764192642586468e0,
                 a105 = -5.90290826836842996371446475743e-1, a106 = 2.12300514481811942347288949897e1,
                 a107 = 1.52792336328824235832596922938e1, a108 = -3.32882109689848629194453265587e1,
                 a109 = -2.03312017085086261358222928593e-2, a111 = -9.3714243008598732571704021658e-1,
                 a114 = 5.18637242884406370830023853209e0, a115 = 1.09143734899672957818500254654e0,
                 a116 = -8.14978701074692612513997267357e0, a117 = -1.85200656599969598641566180701e1,
                 a118 = 2.27394870993505042818970056734e1, a119 = 2.49360555267965238987089396762e0,
                 a1110 = -3.0467644718982195003823669022e0, a121 = 2.27331014751653820792359768449e0,
                 a124 = -1.05344954667372501984066689879e1, a125 = -2.00087205822486249909675718444e0,
                 a126 = -1.79589318631187989172765950534e1, a127 = 2.79488845294199600508499808837e1,
                 a128 = -2.85899827713502369474065508674e0, a129 = -8.87285693353062954433549289258e0,
                 a1210 = 1.23605671757943030647266201528e1, a1211 = 6.43392746015763530355970484046e-1;
}  // namespace dp8

// Automatic initial step size (Hairer's HINIT): an explicit Euler step probes
// the second derivative; h0 such that h^iord * max(|f|, |f'|) = 0.01.
// f0 = f(x, y) is supplied (FSAL); one RHS evaluation.
template <int NV, class F>
__device__ __forceinline__ double hinit(const F& f, double x, const double* y, const double* f0, double posneg,
                                        double iord_inv, double hmax, double rtol, double atol) {
  double dnf = 0.0, dny = 0.0, isk[NV];
#pragma unroll
  for (int i = 0; i < NV; ++i) {
    isk[i] = 1.0 / (atol + rtol * fabs(y[i]));
    const double a = f0[i] * isk[i], b = y[i] * isk[i];
    dnf += a * a;
    dny += b * b;
  }
  double h = (dnf <= 1e-10 || dny <= 1e-10) ? 1e-6 : sqrt(dny / dnf) * 0.01;
  h = fmin(h, hmax);
  h = copysign(h, posneg);
  double y1[NV], f1[NV];
#pragma unroll
  for (int i = 0; i < NV; ++i) y1[i] = y[i] + h * f0[i];
  f(x + h, y1, f1);
  double der2 = 0.0;
#pragma unroll
  for (int i = 0; i < NV; ++i) {
    const double a = (f1[i] - f0[i]) * isk[i];
    der2 += a * a;
  }
  der2 = sqrt(der2) / h;
  const double der12 = fmax(fabs(der2), sqrt(dnf));
  const double h1 = (der12 <= 1e-15) ? fmax(1e-6, fabs(h) * 1e-3) : pow_fp64(0.01 / der12, iord_inv);
  h = fmin(fmin(100.0 * fabs(h), h1), hmax);
  return copysign(h, posneg);
}

// One DOPRI5 attempt from (x, y) with step h and FSAL slope k1.
// Outputs the 5th-order solution y1, its slope k7 = f(x+h, y1) and the scaled
// error norm err = sqrt(mean((e_i / sk_i)^2)).
template <int NV, class F>
__device__ __forceinline__ void dopri5_attempt(const F& f, double x, const double* y, const double* k1, double h,
                                               double rtol, double atol, double* y1, double* k7, double& err) {
  using namespace dp5;
  double k2[NV], k3[NV], k4[NV], k5[NV], k6[NV], yt[NV];
#pragma unroll
  for (int i = 0; i < NV; ++i) yt[i] = y[i] + h * (a21 * k1[i]);
  f(x + c2 * h, yt, k2);
#pragma unroll
  for (int i = 0; i < NV; ++i) yt[i] = y[i] + h * (a31 * k1[i] + a32 * k2[i]);
  f(x + c3 * h, yt, k3);
#pragma unroll
  for (int i = 0; i < NV; ++i) yt[i] = y[i] + h * (a41 * k1[i] + a42 * k2[i] + a43 * k3[i]);
  f(x + c4 * h, yt, k4);
#pragma unroll
  for (int i = 0; i < NV; ++i) yt[i] = y[i] + h * (a51 * k1[i] + a52 * k2[i] + a53 * k3[i] + a54 * k4[i]);
  f(x + c5 * h, yt, k5);
#pragma unroll
  for (int i = 0; i < NV; ++i)
    yt[i] = y[i] + h * (a61 * k1[i] + a62 * k2[i] + a63 * k3[i] + a64 * k4[i] + a65 * k5[i]);
  const double xph = x + h;
  f(xph, yt, k6);
#pragma unroll
  for (int i = 0; i < NV; ++i)
    y1[i] = y[i] + h * (a71 * k1[i] + a73 * k3[i] + a74 * k4[i] + a75 * k5[i] + a76 * k6[i]);
  f(xph, y1, k7);
  double e = 0.0;
#pragma unroll
  for (int i = 0; i < NV; ++i) {
    const double ei = (e1 * k1[i] + e3 * k3[i] + e4 * k4[i] + e5 * k5[i] + e6 * k6[i] + e7 * k7[i]) * h;
    const double sk = atol + rtol * fmax(fabs(y[i]), fabs(y1[i]));
    const double r = ei / sk;
    e += r * r;
  }
  err = sqrt(e * (1.0 / NV));
}

// DOPRI5 coefficient table for the rolled stage loop: row s (1..6) gives the
// stage input y + h sum_j A[s][j] k_{j+1} and its time offset C[s].
static __constant__ double kDp5A[7][6] = {
    {0, 0, 0, 0, 0, 0},
    {dp5::a21, 0, 0, 0, 0, 0},
    {dp5::a31, dp5::a32, 0, 0, 0, 0},
    {dp5::a41, dp5::a42, dp5::a43, 0, 0, 0},
    {dp5::a51, dp5::a52, dp5::a53, dp5::a54, 0, 0},
    {dp5::a61, dp5::a62, dp5::a63, dp5::a64, dp5::a65, 0},
    {dp5::a71, 0, dp5::a73, dp5::a74, dp5::a75, dp5::a76}};
static __constant__ double kDp5C[7] = {0, dp5::c2, dp5::c3, dp5::c4, dp5::c5, 1.0, 1.0};

// The same DOPRI5 attempt with the six right-hand sides in one rolled loop, so
// that an expensive right-hand side (the guiding-centre stencil) is emitted once
// rather than six times. A stage sum takes only the slopes its tableau row uses
// (row s uses k1..k_s, the last row all but k2): the tests on s are the same for
// every lane of a warp, and the terms they skip would add exact zeros.
template <int NV, class F, bool DENSE = false>
__device__ __forceinline__ void dopri5_attempt_rolled(const F& f, double x, const double* y, const double* k1,
                                                      double h, double rtol, double atol, double* y1, double* k7,
                                                      double& err, double* dd = nullptr) {
  using namespace dp5;
  double k2[NV], k3[NV], k4[NV], k5[NV], k6[NV], yt[NV], kt[NV];
#pragma unroll
  for (int i = 0; i < NV; ++i) { k2[i] = k3[i] = k4[i] = k5[i] = k6[i] = 0.0; }
#pragma unroll 1
  for (int s = 1; s <= 6; ++s) {
    const double* A = kDp5A[s];
    double acc[NV];
#pragma unroll
    for (int i = 0; i < NV; ++i) acc[i] = A[0] * k1[i];
    if (s >= 2 && s <= 5) {
#pragma unroll
      for (int i = 0; i < NV; ++i) acc[i] = fma(A[1], k2[i], acc[i]);
    }
    if (s >= 3) {
#pragma unroll
      for (int i = 0; i < NV; ++i) acc[i] = fma(A[2], k3[i], acc[i]);
    }
    if (s >= 4) {
#pragma unroll
      for (int i = 0; i < NV; ++i) acc[i] = fma(A[3], k4[i], acc[i]);
    }
    if (s >= 5) {
#pragma unroll
      for (int i = 0; i < NV; ++i) acc[i] = fma(A[4], k5[i], acc[i]);
    }
    if (s == 6) {
#pragma unroll
      for (int i = 0; i < NV; ++i) acc[i] = fma(A[5], k6[i], acc[i]);
    }
#pragma unroll
    for (int i = 0; i < NV; ++i) yt[i] = fma(h, acc[i], y[i]);
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
    const double ei = (e1 * k1[i] + e3 * k3[i] + e4 * k4[i] + e5 * k5[i] + e6 * k6[i] + e7 * k7[i]) * h;
    const double sk = atol + rtol * fmax(fabs(y[i]), fabs(y1[i]));
    const double r = ei / sk;
    e += r * r;
    if (DENSE) dd[i] = h * (d1 * k1[i] + d3 * k3[i] + d4 * k4[i] + d5 * k5[i] + d6 * k6[i] + d7 * k7[i]);
  }
  err = sqrt(e * (1.0 / NV));
}

// DOPRI5 continuous extension at theta in [0, 1] of an accepted step from y0
// (slope k1) to y1 (slope k7): the Hermite-like form of Hairer's CONTD5 with
// the fifth coefficient dd from the attempt.
template <int NV>
__device__ __forceinline__ void dopri5_dense(const double* y0, const double* y1, const double* k1, const double* k7,
                                             const double* dd, double h, double theta, double* out) {
  const double th1 = 1.0 - theta;
#pragma unroll
  for (int i = 0; i < NV; ++i) {
    const double ydiff = y1[i] - y0[i];
    const double bspl = h * k1[i] - ydiff;
    const double r4 = ydiff - h * k7[i] - bspl;
    out[i] = y0[i] + theta * (ydiff + th1 * (bspl + theta * (r4 + th1 * dd[i])));
  }
}

// One DOP853 attempt: 11 new stages; the 5th- and 3rd-order error estimates
// combined as in DOP853. Outputs the 8th-order solution y1 and err.
template <int NV, class F>
__device__ __forceinline__ void dop853_attempt(const F& f, double x, const double* y, const double* k1, double h,
                                               double rtol, double atol, double* y1, double& err) {
  using namespace dp8;
  double k2[NV], k3[NV], k4[NV], k5[NV], k6[NV], k7[NV], k8[NV], k9[NV], k10[NV], yt[NV];
#pragma unroll
  for (int i = 0; i < NV; ++i) yt[i] = y[i] + h * a21 * k1[i];
  f(x + c2 * h, yt, k2);
#pragma unroll
  for (int i = 0; i < NV; ++i) yt[i] = y[i] + h * (a31 * k1[i] + a32 * k2[i]);
  f(x + c3 * h, yt, k3);
#pragma unroll
  for (int i = 0; i < NV; ++i) yt[i] = y[i] + h * (a41 * k1[i] + a43 * k3[i]);
  f(x + c4 * h, yt, k4);
#pragma unroll
  for (int i = 0; i < NV; ++i) yt[i] = y[i] + h * (a51 * k1[i] + a53 * k3[i] + a54 * k4[i]);
  f(x + c5 * h, yt, k5);
#pragma unroll
  for (int i = 0; i < NV; ++i) yt[i] = y[i] + h * (a61 * k1[i] + a64 * k4[i] + a65 * k5[i]);
  f(x + c6 * h, yt, k6);
#pragma unroll
  for (int i = 0; i < NV; ++i) yt[i] = y[i] + h * (a71 * k1[i] + a74 * k4[i] + a75 * k5[i] + a76 * k6[i]);
  f(x + c7 * h, yt, k7);
#pragma unroll
  for (int i = 0; i < NV; ++i)
    yt[i] = y[i] + h * (a81 * k1[i] + a84 * k4[i] + a85 * k5[i] + a86 * k6[i] + a87 * k7[i]);
  f(x + c8 * h, yt, k8);
#pragma unroll
  for (int i = 0; i < NV; ++i)
    yt[i] = y[i] + h * (a91 * k1[i] + a94 * k4[i] + a95 * k5[i] + a96 * k6[i] + a97 * k7[i] + a98 * k8[i]);
  f(x + c9 * h, yt, k9);
#pragma unroll
  for (int i = 0; i < NV; ++i)
    yt[i] = y[i] + h * (a101 * k1[i] + a104 * k4[i] + a105 * k5[i] + a106 * k6[i] + a107 * k7[i] +
                        a108 * k8[i] + a109 * k9[i]);
  f(x + c10 * h, yt, k10);
#pragma unroll
  for (int i = 0; i < NV; ++i)
    yt[i] = y[i] + h * (a111 * k1[i] + a114 * k4[i] + a115 * k5[i] + a116 * k6[i] + a117 * k7[i] +
                        a118 * k8[i] + a119 * k9[i] + a1110 * k10[i]);
  f(x + c11 * h, yt, k2);  // stage 11 reuses k2
  const double xph = x + h;
#pragma unroll
  for (int i = 0; i < NV; ++i)
    yt[i] = y[i] + h * (a121 * k1[i] + a124 * k4[i] + a125 * k5[i] + a126 * k6[i] + a127 * k7[i] +
                        a128 * k8[i] + a129 * k9[i] + a1210 * k10[i] + a1211 * k2[i]);
  f(xph, yt, k3);  // stage 12 reuses k3
  double e5 = 0.0, e3 = 0.0;
#pragma unroll
  for (int i = 0; i < NV; ++i) {
    const double bs = b1 * k1[i] + b6 * k6[i] + b7 * k7[i] + b8 * k8[i] + b9 * k9[i] + b10 * k10[i] +
                      b11 * k2[i] + b12 * k3[i];
    y1[i] = y[i] + h * bs;
    const double isk = 1.0 / (atol + rtol * fmax(fabs(y[i]), fabs(y1[i])));
    const double r3 = (bs - bhh1 * k1[i] - bhh2 * k9[i] - bhh3 * k3[i]) * isk;
    const double r5 = (er1 * k1[i] + er6 * k6[i] + er7 * k7[i] + er8 * k8[i] + er9 * k9[i] + er10 * k10[i] +
                       er11 * k2[i] + er12 * k3[i]) * isk;
    e3 += r3 * r3;
    e5 += r5 * r5;
  }
  double deno = e5 + 0.01 * e3;
  if (deno <= 0.0) deno = 1.0;
  err = fabs(h) * e5 * sqrt(1.0 / (NV * deno));
}

// One RKF45 attempt as restated from rapt/rkf.py:101-124 (coefficients
// rkf.py:48-87): k_i = h f(...),
// error r = max_i |sum r_j k_j| / h, 4th-order solution y1. NANPROP: r is NaN
// when any term is (a Grid stage outside the grid), which fmax alone would drop.
template <int NV, bool NANPROP = false, class F>
__device__ __forceinline__ void rkf45_attempt(const F& f, double t, const double* x, double h, double* y1,
                                              double& r) {
  // the decimal coefficients of rkf.py:48-87 (several differ from the exact
  // fractions in the last bit)
  constexpr double a2 = 2.500000000000000e-01, a3 = 3.750000000000000e-01, a4 = 9.230769230769231e-01, a5 = 1.0,
                   a6 = 5.000000000000000e-01;
  constexpr double b21 = 2.500000000000000e-01, b31 = 9.375000000000000e-02, b32 = 2.812500000000000e-01,
                   b41 = 8.793809740555303e-01, b42 = -3.277196176604461e+00, b43 = 3.320892125625853e+00,
                   b51 = 2.032407407407407e+00, b52 = -8.000000000000000e+00, b53 = 7.173489278752436e+00,
                   b54 = -2.058966861598441e-01, b61 = -2.962962962962963e-01, b62 = 2.000000000000000e+00,
                   b63 = -1.381676413255361e+00, b64 = 4.529727095516569e-01, b65 = -2.750000000000000e-01;
  constexpr double r1 = 2.777777777777778e-03, r3 = -2.994152046783626e-02, r4 = -2.919989367357789e-02,
                   r5 = 2.000000000000000e-02, r6 = 3.636363636363636e-02;
  constexpr double c1 = 1.157407407407407e-01, c3 = 5.489278752436647e-01, c4 = 5.353313840155945e-01,
                   c5 = -2.000000000000000e-01;
  double k1[NV], k2[NV], k3[NV], k4[NV], k5[NV], k6[NV], xt[NV];
  f(t, x, k1);
#pragma unroll
  for (int i = 0; i < NV; ++i) { k1[i] *= h; xt[i] = x[i] + b21 * k1[i]; }
  f(t + a2 * h, xt, k2);
#pragma unroll
  for (int i = 0; i < NV; ++i) { k2[i] *= h; xt[i] = x[i] + b31 * k1[i] + b32 * k2[i]; }
  f(t + a3 * h, xt, k3);
#pragma unroll
  for (int i = 0; i < NV; ++i) { k3[i] *= h; xt[i] = x[i] + b41 * k1[i] + b42 * k2[i] + b43 * k3[i]; }
  f(t + a4 * h, xt, k4);
#pragma unroll
  for (int i = 0; i < NV; ++i) { k4[i] *= h; xt[i] = x[i] + b51 * k1[i] + b52 * k2[i] + b53 * k3[i] + b54 * k4[i]; }
  f(t + a5 * h, xt, k5);
#pragma unroll
  for (int i = 0; i < NV; ++i) {
    k5[i] *= h;
    xt[i] = x[i] + b61 * k1[i] + b62 * k2[i] + b63 * k3[i] + b64 * k4[i] + b65 * k5[i];
  }
  f(t + a6 * h, xt, k6);
  r = 0.0;
  bool nan_term = false;
#pragma unroll
  for (int i = 0; i < NV; ++i) {
    k6[i] *= h;
    const double ri = fabs(r1 * k1[i] + r3 * k3[i] + r4 * k4[i] + r5 * k5[i] + r6 * k6[i]) / h;
    r = fmax(r, ri);
    if (NANPROP) nan_term = nan_term || isnan(ri);
    y1[i] = x[i] + c1 * k1[i] + c3 * k3[i] + c4 * k4[i] + c5 * k5[i];
  }
  if (NANPROP && nan_term) r = __longlong_as_double(0x7ff8000000000000LL);
}

}  // namespace rapt
