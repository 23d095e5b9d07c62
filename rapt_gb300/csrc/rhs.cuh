// rhs.cuh -- equations of motion on the device.
#pragma once
#include "fields.cuh"

namespace rapt {

// Newton-Lorentz equation, the eom closure of Particle.advance
// (rapt/Particle.py:284-298): dx/dt = p / (gamma m), dp/dt = q (E + p x B / (gamma m)).
// gamma m is frozen at the start of the advance() call when the field is
// static and recomputed from the stage momentum otherwise, as in the reference.
template <int M>
struct ParticleRHS {
  FieldP f;
  double charge, mass2, inv_gm_frozen;
  bool eq;
  __device__ __forceinline__ void operator()(double t, const double* Y, double* o) const {
    double igm = inv_gm_frozen;
    if (!field_static<M>(f)) igm = rsqrt(mass2 + (Y[3] * Y[3] + Y[4] * Y[4] + Y[5] * Y[5]) * (1.0 / (kC * kC)));
    double B[3], E[3];
    field_BE<M>(f, t, Y[0], Y[1], Y[2], B, E);
    o[0] = Y[3] * igm;
    o[1] = Y[4] * igm;
    o[2] = Y[5] * igm;
    const double qg = charge * igm;
    o[3] = charge * E[0] + qg * (Y[4] * B[2] - Y[5] * B[1]);
    o[4] = charge * E[1] + qg * (Y[5] * B[0] - Y[3] * B[2]);
    o[5] = charge * E[2] + qg * (Y[3] * B[1] - Y[4] * B[0]);
    if (eq) { o[2] = 0.0; o[5] = 0.0; }
  }
};

// Guiding-centre equations (rapt/GuidingCenter.py:329-395).
//   eom 0: Tao-Chan-Brizard   (GuidingCenter.py:329-355)
//   eom 1: Brizard-Chan       (GuidingCenter.py:357-379)
//   eom 2: Northrop-Teller    (GuidingCenter.py:381-395)
// grad|B| and curl b use the reference's central differences with the field's
// gradientstepsize, evaluated on the 6-point stencil once (7 B evaluations per
// call for static fields instead of the reference's 13; same values).
template <int M>
struct GcRHS {
  FieldP f;
  double charge, qinv, mu, minv, k_mu, inv_mc;  // k_mu = 2 mu/(m c^2), inv_mc = 1/(m c)
  double inv_gamma_v, gm_v, gm_v_v2;             // BC/NT: 1/gamma(v), gamma(v) m, gamma m v^2
  int eom;
  bool eq;
  __device__ __forceinline__ void operator()(double t, const double* Y, double* o) const {
    const double ppar = Y[3];
    double ub[3], Bmag;
    double B[3], gB[3], cb[3], Eg[3], dbg[3];
    if constexpr (M == RAPT_GRID) {
      // B, E, the stencil and db/dt from one cell search (grid_gc_fields)
      const GridFields g = grid_gc_fields(RAPT_GRID_PASS(f), f.gB, eom == 0 ? f.gE : nullptr, t, Y[0], Y[1], Y[2],
                                          f.gradstep, f.inv2d, f.timestep, eom == 0 && !field_static<M>(f));
#pragma unroll
      for (int k = 0; k < 3; ++k) { B[k] = g.B[k]; Eg[k] = g.E[k]; gB[k] = g.gB[k]; cb[k] = g.cb[k]; dbg[k] = g.db[k]; }
    } else {
      Field<M>::B(f, t, Y[0], Y[1], Y[2], B);
    }
    {
      const double b2 = dot3(B, B);
      const double ib = rsqrt(b2);
      Bmag = b2 * ib;
      ub[0] = B[0] * ib; ub[1] = B[1] * ib; ub[2] = B[2] * ib;
    }
    if constexpr (M != RAPT_GRID) stencil_gradB_curlb<M>(f, t, Y, gB, cb);
    if (eom == 0) {
      const double pm = ppar * inv_mc;
      const double g2 = 1.0 + k_mu * Bmag + pm * pm;
      const double rg = rsqrt(g2);
      double E[3], db[3];
      if constexpr (M == RAPT_GRID) {
#pragma unroll
        for (int k = 0; k < 3; ++k) { E[k] = Eg[k]; db[k] = dbg[k]; }
      } else {
        Field<M>::E(f, t, Y[0], Y[1], Y[2], E);
        dbdt<M>(f, t, Y, db);
      }
      const double pq = ppar * qinv;
      double Bs[3] = {B[0] + pq * cb[0], B[1] + pq * cb[1], B[2] + pq * cb[2]};
      const double iBsp = 1.0 / dot3(Bs, ub);
      const double mg = mu * rg;
      double Es[3];
#pragma unroll
      for (int i = 0; i < 3; ++i) Es[i] = E[i] - (ppar * db[i] + mg * gB[i]) * qinv;
      double Exb[3];
      cross3(Es, ub, Exb);
      const double a = ppar * rg * minv;
#pragma unroll
      for (int i = 0; i < 3; ++i) o[i] = (a * Bs[i] + Exb[i]) * iBsp;
      o[3] = charge * dot3(Es, Bs) * iBsp;
    } else if (eom == 1) {
      const double pq = ppar * qinv;
      double Bs[3] = {B[0] + pq * cb[0], B[1] + pq * cb[1], B[2] + pq * cb[2]};
      const double iBsp = 1.0 / dot3(Bs, ub);
      double bxg[3];
      cross3(ub, gB, bxg);
      const double a = ppar * inv_gamma_v * minv;
      const double c = mu * qinv * inv_gamma_v;
#pragma unroll
      for (int i = 0; i < 3; ++i) o[i] = (a * Bs[i] + c * bxg[i]) * iBsp;
      o[3] = -mu * dot3(Bs, gB) * inv_gamma_v * iBsp;
    } else {
      double bxg[3];
      cross3(ub, gB, bxg);
      const double s = (gm_v_v2 + ppar * ppar / gm_v) / (2.0 * charge * Bmag * Bmag);
      const double a = ppar / gm_v;
#pragma unroll
      for (int i = 0; i < 3; ++i) o[i] = s * bxg[i] + a * ub[i];
      o[3] = -mu * dot3(ub, gB) * inv_gamma_v;
    }
    if (eq) { o[2] = 0.0; o[3] = 0.0; }
  }
};

}  // namespace rapt
