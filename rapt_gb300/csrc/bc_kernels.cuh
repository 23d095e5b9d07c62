// bc_kernels.cuh -- BounceCenter (rapt/BounceCenter.py) on the device: the
// bounce-averaged drift of a guiding centre in a static magnetic field,
//   dx/dt = gamma m v^2 / (q S_b |B|^2) (grad I x B)        BounceCenter.py:236-245
// with S_b the half-bounce path (flutils.halfbouncepath) and grad I the
// gradient of the second invariant (flutils.gradI): five field-line traces per
// right-hand side, each thread tracing its own lines in a private scratch slot.
// advance(delta) (BounceCenter.py:214-252) outputs every BCtimestep x the
// bounce period at the start, restarting DOPRI5 (SciPy's dopri5 defaults) per
// row; the host launches one interval of every tracer per kernel.
//
// The reference's isequatorial branch (BounceCenter.py:238-239) hands the
// 3-vector state to _v_grad as (t, x, y, z) and fails; it is not built.
#pragma once
#include "fieldline.cuh"
#include "steppers.cuh"
#include "tracer_kernels.cuh"

namespace rapt {

template <int M>
struct BcRHS {
  FieldP f;
  double Bm, kdrift, d, flres;  // kdrift = gamma m v^2 / q
  double* scratch;
  int cap;
  int32_t* flag;  // set where a value is not finite (the host reruns the tracer with full trace slots)
  __device__ void operator()(double t, const double* Y, double* o) const {
    double B[3], gI[3];
    Field<M>::B(f, t, Y[0], Y[1], Y[2], B);
    const double magBsq = ndot3(B, B);
    const double Sb = fl_halfbouncepath<M>(f, t, Y, Bm, flres, scratch, cap);
    fl_gradI<M>(f, t, Y, Bm, d, flres, scratch, cap, gI);
    if (flag && !(isfinite(Sb) && isfinite(gI[0]) && isfinite(gI[1]) && isfinite(gI[2]))) *flag = 1;
    const double k = kdrift / dm(Sb, magBsq);
    o[0] = dm(k, da(dm(gI[1], B[2]), -dm(gI[2], B[1])));
    o[1] = dm(k, da(dm(gI[2], B[0]), -dm(gI[0], B[2])));
    o[2] = dm(k, da(dm(gI[0], B[1]), -dm(gI[1], B[0])));
  }
};

__device__ __forceinline__ double bc_gamma(double v) { return 1.0 / sqrt(1.0 - (v / kC) * (v / kC)); }

// Start of advance(delta): mirror field, cadence and row count per tracer.
// st[5] = (t, x, y, z, tcur); plan[4] = (Bm, dt, K, arange step).
template <int M>
__global__ void k_bc_start(FieldP f, double flres, int64_t n, const double* st, const double* cst, double delta,
                           double bctimestep, double* plan, int32_t* status, int32_t* flag, double* scratch,
                           long long stride, int cap) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const double* s = st + 5 * k;
  const double v = cst[4 * k], mu = cst[4 * k + 1], mass = cst[4 * k + 2];
  const double gamma = bc_gamma(v);
  const double Bm = dm(dm(mass, dm(gamma, gamma)), dm(v, v)) / dm(2.0, mu);
  const double X[3] = {s[1], s[2], s[3]};
  const double bp = dm(2.0 / v, fl_halfbouncepath<M>(f, s[0], X, Bm, flres, scratch + (size_t)k * stride, cap));
  const double dt = dm(bctimestep, bp);
  double* p = plan + 4 * k;
  p[0] = Bm;
  p[1] = dt;
  if (!(dt > 0.0) || !isfinite(dt)) {
    status[k] = RAPT_ST_FIELDLINE;
    if (flag) flag[k] = 1;
    p[2] = 0.0;
    return;
  }
  const double tcur = s[4];
  p[2] = ceil(da(da(tcur, delta), -tcur) / dt);  // len(np.arange(tcur, tcur + delta, dt))
  p[3] = da(da(tcur, dt), -tcur);                 // numpy's fill step for i >= 2
  status[k] = RAPT_ST_OK;
}

// Interval j of every tracer with j < K: one SciPy-dopri5 integrate() call from
// the integrator time (state t) over dt, then the row stamped with the
// interval's start, np.arange's j-th value.
template <int M>
__global__ void __launch_bounds__(64) k_bc_interval(FieldP f, KParams P, int64_t n, double* st, const double* cst,
                                                    const double* plan, double d, int64_t j, double* rows,
                                                    int max_rows, int32_t* nrows, int32_t* status, int64_t* counters,
                                                    int32_t* flag, double* scratch, long long stride, int cap) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const double* p = plan + 4 * k;
  if (status[k] != RAPT_ST_OK || (double)j >= p[2]) return;
  double* s = st + 5 * k;
  const double v = cst[4 * k], mass = cst[4 * k + 2], charge = cst[4 * k + 3];
  const double gamma = bc_gamma(v);
  const BcRHS<M> rhs{f, p[0], dm(dm(dm(gamma, mass), v), v) / charge, d, P.flres, scratch + (size_t)k * stride, cap,
                     flag ? flag + k : nullptr};
  const double dt = p[1];
  double rt = s[0];
  double y[3] = {s[1], s[2], s[3]}, k1[3];
  const double xend = da(rt, dt);
  // SciPy dopri5 (Hairer's DOPRI5, beta 0.04) over [rt, xend], restarted
  constexpr double beta = 0.04, safe = 0.9;
  constexpr double expo1 = 0.2 - beta * 0.75, facc1 = 1.0 / 0.2, facc2 = 1.0 / 10.0;
  const double hmax = fabs(xend - rt), posneg = copysign(1.0, xend - rt);
  rhs(rt, y, k1);
  double h = hinit<3>(rhs, rt, y, k1, posneg, 1.0 / 5.0, hmax, P.rtol, P.atol);
  long long nfcn = 2, nstep = 0, nacc = 0, nrej = 0;
  double facold = 1e-4;
  bool reject = false, last = false;
  int fail = 0;
  for (;;) {
    if (nstep > P.nsteps) { fail = RAPT_ST_MAXSTEPS; break; }
    if (0.1 * fabs(h) <= fabs(rt) * kUround) { fail = RAPT_ST_HMIN; break; }
    if ((rt + 1.01 * h - xend) * posneg > 0.0) { h = xend - rt; last = true; }
    ++nstep;
    double y1[3], k7[3], err;
    dopri5_attempt_rolled<3>(rhs, rt, y, k1, h, P.rtol, P.atol, y1, k7, err);
    nfcn += 6;
    const double fac11 = pow_fp64(err, expo1);
    double fac = fac11 / pow_fp64(facold, beta);
    fac = fmax(facc2, fmin(facc1, fac / safe));
    double hnew = h / fac;
    if (err <= 1.0) {
      facold = fmax(err, 1.0e-4);
      ++nacc;
      for (int i = 0; i < 3; ++i) { k1[i] = k7[i]; y[i] = y1[i]; }
      rt = rt + h;
      if (last) break;
      if (fabs(hnew) > hmax) hnew = posneg * hmax;
      if (reject) hnew = posneg * fmin(fabs(hnew), fabs(h));
      reject = false;
    } else {
      hnew = h / fmin(facc1, fac11 / safe);
      reject = true;
      if (nacc >= 1) ++nrej;
      last = false;
    }
    h = hnew;
  }
  if (fail) status[k] = fail;
  if (!(isfinite(y[0]) && isfinite(y[1]) && isfinite(y[2]))) status[k] = RAPT_ST_NONFINITE;
  const double tcur0 = s[4];
  const double tj = j == 0 ? tcur0 : (j == 1 ? da(tcur0, dt) : da(tcur0, dm((double)j, p[3])));
  if (nrows[k] < max_rows) {
    double* r = rows + ((size_t)k * (size_t)max_rows + (size_t)nrows[k]) * 4;
    r[0] = tj; r[1] = y[0]; r[2] = y[1]; r[3] = y[2];
  }
  nrows[k] += 1;
  s[0] = tj;  // trajectory[-1] = (t_j, x, y, z); the integrator restarts from it
  s[1] = y[0]; s[2] = y[1]; s[3] = y[2];
  if (j + 1 >= (int64_t)p[2] || status[k] != RAPT_ST_OK) s[4] = tj;  // tcur = trajectory[-1, 0]
  if (counters) {
    int64_t* c = counters + 4 * k;
    c[0] += nfcn; c[1] += nstep; c[2] += nacc; c[3] += nrej;
  }
}

// what 0 the second invariant I, 1 grad I (3 values), 2 the drift velocity
// (3 values), 3 the half-bounce path, at tpos[n][4] with mirror fields Bm[n]
// (what 2: cst[n][4]).
template <int M>
__global__ void k_bc_eval(FieldP f, double flres, int what, int64_t n, const double* tpos, const double* Bm, double d,
                          const double* cst, double* out, double* scratch, long long stride, int cap) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const double* tp = tpos + 4 * k;
  const double X[3] = {tp[1], tp[2], tp[3]};
  double* scr = scratch + (size_t)k * stride;
  double* o = out + 3 * k;
  if (what == 0 || what == 3) {
    o[0] = what == 0 ? fl_eye<M>(f, tp[0], X, Bm[k], flres, scr, cap)
                     : fl_halfbouncepath<M>(f, tp[0], X, Bm[k], flres, scr, cap);
    o[1] = o[2] = 0.0;
  } else if (what == 1) {
    fl_gradI<M>(f, tp[0], X, Bm[k], d, flres, scr, cap, o);
  } else {
    const double v = cst[4 * k], mass = cst[4 * k + 2], charge = cst[4 * k + 3];
    const double gamma = bc_gamma(v);
    const BcRHS<M> rhs{f, Bm[k], dm(dm(dm(gamma, mass), v), v) / charge, d, flres, scr, cap, nullptr};
    rhs(tp[0], X, o);
  }
}

}  // namespace rapt
