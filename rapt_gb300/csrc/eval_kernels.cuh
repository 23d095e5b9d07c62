// eval_kernels.cuh -- single-point field and right-hand-side evaluation, and
// the Adaptive constructor's mode pick, used by checks and by rapt_adaptive_init.
#pragma once
#include "tracer_kernels.cuh"

namespace rapt {

// what: 0 B, 1 E, 2 gradB, 3 curlb, 4 magB, 5 unitb, 6 lengthscale, 7 dbdt,
// 8 jacobianB (row-major dB_i/dx_j), 9 dBdt, 10 timescale (NaN when static).
template <int M>
__global__ void k_field_eval(FieldP f, int what, int64_t n, const double* tpos, double* out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double t = tpos[4 * i];
  const double X[3] = {tpos[4 * i + 1], tpos[4 * i + 2], tpos[4 * i + 3]};
  double* o = out + 9 * i;
  double r[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  switch (what) {
    case 0: Field<M>::B(f, t, X[0], X[1], X[2], r); break;
    case 1: Field<M>::E(f, t, X[0], X[1], X[2], r); break;
    case 2: { double cb[3]; stencil_gradB_curlb<M>(f, t, X, r, cb); } break;
    case 3: { double gb[3]; stencil_gradB_curlb<M>(f, t, X, gb, r); } break;
    case 4: { double u[3]; unit_and_mag<M>(f, t, X[0], X[1], X[2], u, r[0]); } break;
    case 5: { double m; unit_and_mag<M>(f, t, X[0], X[1], X[2], r, m); } break;
    case 6: r[0] = lengthscale<M>(f, t, X); break;
    case 7: dbdt<M>(f, t, X, r); break;
    case 8:
      for (int a = 0; a < 3; ++a) {
        double xp[3] = {X[0], X[1], X[2]}, xm[3] = {X[0], X[1], X[2]};
        xp[a] = X[a] + f.gradstep;
        xm[a] = X[a] - f.gradstep;
        double bp[3], bm[3];
        Field<M>::B(f, t, xp[0], xp[1], xp[2], bp);
        Field<M>::B(f, t, xm[0], xm[1], xm[2], bm);
        for (int c = 0; c < 3; ++c) r[3 * c + a] = (bp[c] - bm[c]) * f.inv2d;
      }
      break;
    case 9: r[0] = dBdt<M>(f, t, X); break;
    case 10: {
      if (field_static<M>(f)) { r[0] = nan(""); break; }
      double u[3], m;
      unit_and_mag<M>(f, t, X[0], X[1], X[2], u, m);
      r[0] = m / fabs(dBdt<M>(f, t, X));
    } break;
    default: break;
  }
  for (int k = 0; k < 9; ++k) o[k] = r[k];
}

// state[i] = (t, y0..y5, gm | mu); mode 0 particle (gm frozen), 1 GC.
template <int M>
__global__ void k_rhs_eval(KParams P, int mode, int64_t n, const double* state, const double* mass,
                           const double* charge, const double* v, double* out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double* s = state + 8 * i;
  double o[6] = {0, 0, 0, 0, 0, 0};
  if (mode == 0) {
    const ParticleRHS<M> rhs{P.f, charge[i], mass[i] * mass[i], 1.0 / s[7], P.enforce_eq != 0};
    rhs(s[0], s + 1, o);
  } else {
    const double m = mass[i], q = charge[i], mu = s[7], vs = v[i];
    const double gv = 1.0 / sqrt(1.0 - (vs / kC) * (vs / kC));
    const GcRHS<M> rhs{P.f, q, 1.0 / q, mu, 1.0 / m, 2.0 * mu / (m * kC * kC), 1.0 / (m * kC), 1.0 / gv,
                       gv * m, gv * m * vs * vs, P.gc_eom, P.enforce_eq != 0};
    rhs(s[0], s + 1, o);
  }
  for (int k = 0; k < 6; ++k) out[6 * i + k] = o[k];
}

// Adaptive.__init__ (rapt/Adaptive.py:70-104): a particle that is adiabatic at
// its start is replaced by its guiding centre (GuidingCenter.init(Particle)).
template <int M>
__global__ void k_adaptive_init(DevEnsemble E, KParams P) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= E.n || E.mode[k] != RAPT_MODE_PARTICLE) return;
  double s[6];
  for (int i = 0; i < 6; ++i) s[i] = E.s[i][k];
  const double t = E.t_row[k];
  if (!particle_isadiabatic<M>(P, t, s, E.mass[k], E.charge[k])) return;
  double g[6], mu, vs;
  if (!particle_to_gc<M>(P.f, t, s, E.mass[k], E.charge[k], g, mu, vs)) {
    E.status[k] = RAPT_ST_GC_NOCONV;
    return;
  }
  for (int i = 0; i < 6; ++i) E.s[i][k] = g[i];
  E.mu[k] = mu;
  E.v[k] = vs;
  E.mode[k] = RAPT_MODE_GC;
}

// GuidingCenter.bounceperiod (GuidingCenter.py:593-606) for n states
// (t, x, y, z, ppar, mu, mass); one thread each, fl_stride doubles of scratch
// per thread. NaN where the trace does not fit the buffer.
template <int M>
__global__ void k_bounce_period(FieldP f, double flres, int64_t n, const double* in, double* out, double* scratch,
                                long long stride, int cap) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const double* r = in + 7 * k;
  const double y[4] = {r[1], r[2], r[3], r[4]};
  out[k] = gc_bounceperiod<M>(f, r[0], y, r[5], r[6], flres, scratch + (size_t)k * (size_t)stride, cap);
}

}  // namespace rapt
