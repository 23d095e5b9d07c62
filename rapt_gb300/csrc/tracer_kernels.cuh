// tracer_kernels.cuh -- persistent one-thread-per-tracer kernels, one per mode.
//
// Each thread owns one tracer at a time and runs it as a state machine that
// performs exactly one Runge-Kutta step attempt per loop iteration, so a warp
// keeps stepping in lockstep while its lanes sit at different points of their
// output intervals. When a lane's tracer finishes its advance() call, switches
// mode (Adaptive) or runs out of this launch's step budget, the warp refills
// all such lanes at once: __ballot_sync collects the idle lanes, one lane takes
// that many indices from the global work queue with a single atomicAdd, and
// each idle lane picks its index by the popcount of the lanes below it.
//
// Semantics follow the reference tracer loops:
//   Particle.advance       rapt/Particle.py:230-309
//   GuidingCenter.advance  rapt/GuidingCenter.py:397-458
//   Adaptive.advance       rapt/Adaptive.py:187-222
// including the per-interval restart of the integrator with an automatic
// initial step (every SciPy integrate() call), the row time r.t+dt and the
// one-dt-ahead tcur of Particle.advance, and the adiabaticity checks after
// each output row. Every loop is bounded: nsteps per interval, the per-launch
// step budget, 20 guiding-centre iterations, and the Adaptive segment cap.
#pragma once
#include "fieldline.cuh"
#include "mlp.cuh"
#include "rhs.cuh"
#include "steppers.cuh"

namespace rapt {

constexpr double kUround = 2.3e-16;  // Hairer's default UROUND

template <int N>
__device__ __forceinline__ bool all_finite(const double* y) {
  bool ok = true;
#pragma unroll
  for (int i = 0; i < N; ++i) ok = ok && isfinite(y[i]);
  return ok;
}

// ---------------------------------------------------------------- physics helpers
// utils.cyclotron_period (rapt/utils.py:62-66) from position and velocity.
template <int M>
__device__ double cyc_period_vel(const FieldP& f, double t, const double* pos, const double* vel, double mass,
                                 double charge) {
  const double gamma = 1.0 / sqrt(1.0 - dot3(vel, vel) / (kC * kC));
  double ub[3], B;
  unit_and_mag<M>(f, t, pos[0], pos[1], pos[2], ub, B);
  return 2.0 * kPi * gamma * mass / B / fabs(charge);
}

// Particle.isadiabatic, rapt/Particle.py:345-384.
template <int M>
__device__ bool particle_isadiabatic(const KParams& P, double t, const double* s, double mass, double charge) {
  const FieldP& f = P.f;
  const double* mom = s + 3;
  const double gm = sqrt(mass * mass + dot3(mom, mom) / (kC * kC));
  const double v[3] = {mom[0] / gm, mom[1] / gm, mom[2] / gm};
  const double vsq = dot3(v, v);
  const double gamma = 1.0 / sqrt(1.0 - vsq / (kC * kC));
  double B[3];
  Field<M>::B(f, t, s[0], s[1], s[2], B);
  const double Bmag = sqrt(dot3(B, B));
  const double vpar = dot3(v, B) / Bmag;
  const double vperp = sqrt(vsq - vpar * vpar);
  const double cycrad = gamma * mass * vperp / (fabs(charge) * Bmag);
  const bool sp = cycrad / lengthscale<M>(f, t, s) < P.epss;
  if (field_static<M>(f)) return sp;
  if (!sp) return false;
  const double cycper = cyc_period_vel<M>(f, t, s, v, mass, charge);
  const double ts = Bmag / fabs(dBdt<M>(f, t, s));
  return cycper / ts < P.epst;
}

// GuidingCenter.isadiabatic, rapt/GuidingCenter.py:287-327 (cycrad :517-530,
// cycper :532-541 whose gamma squares ppar without dividing by m c -- kept).
template <int M>
__device__ bool gc_isadiabatic(const KParams& P, double t, const double* s, double mu, double mass,
                               double charge) {
  const FieldP& f = P.f;
  const double pp = s[3], m = mass;
  double B[3];
  Field<M>::B(f, t, s[0], s[1], s[2], B);
  const double Bmag = sqrt(dot3(B, B));
  const double gamma = sqrt(1.0 + 2.0 * mu * Bmag / (m * kC * kC) + (pp / m / kC) * (pp / m / kC));
  double vp, v;
  if (gamma - 1.0 < 1e-6) { vp = pp / m; v = sqrt(2.0 * mu * Bmag / m + vp * vp); }
  else { vp = pp / m / gamma; v = kC * sqrt(1.0 - 1.0 / (gamma * gamma)); }
  const double g2 = 1.0 / sqrt(1.0 - (v / kC) * (v / kC));
  const double cycrad = g2 * m * sqrt((v - vp) * (v + vp)) / (fabs(charge) * Bmag);
  const bool sp = cycrad / lengthscale<M>(f, t, s) < P.epss;
  if (field_static<M>(f)) return sp;
  if (!sp) return false;
  const double gq = sqrt(1.0 + 2.0 * mu * Bmag / (m * kC * kC) + pp * pp);
  double v2;
  if (gq - 1.0 < 1e-6) { const double vp2 = pp / m; v2 = sqrt(2.0 * mu * Bmag / m + vp2 * vp2); }
  else v2 = kC * sqrt(1.0 - 1.0 / (gq * gq));
  const double g3 = 1.0 / sqrt(1.0 - (v2 / kC) * (v2 / kC));
  const double cycper = 2.0 * kPi * g3 * m / Bmag / fabs(charge);
  const double ts = Bmag / fabs(dBdt<M>(f, t, s));
  return cycper / ts < P.epst;
}

// utils.guidingcenter fixed point R = r - rho(R), tol 1e-3, <= 20 iterations
// (rapt/utils.py:251-326) followed by GuidingCenter.__init__ with ppar given
// (GuidingCenter.py:108-133), as GuidingCenter.init(Particle) does (:168-187).
// Writes g = (x, y, z, ppar), mu and the speed; false if the iteration fails.
template <int M>
__device__ bool particle_to_gc(const FieldP& f, double t, const double* s, double mass, double charge, double* g,
                               double& mu, double& vspeed) {
  const double* mom = s + 3;
  const double gm = sqrt(mass * mass + dot3(mom, mom) / (kC * kC));
  const double v[3] = {mom[0] / gm, mom[1] / gm, mom[2] / gm};
  const double vsq = dot3(v, v);
  const double gam = 1.0 / sqrt(1.0 - vsq / (kC * kC));
  double gv[3], old[3], cur[3];
  auto gyro = [&](const double* r) {
    double B[3];
    Field<M>::B(f, t, r[0], r[1], r[2], B);
    const double sc = gam * mass / (charge * dot3(B, B));
    double bxv[3];
    cross3(B, v, bxv);
    gv[0] = sc * bxv[0]; gv[1] = sc * bxv[1]; gv[2] = sc * bxv[2];
  };
  gyro(s);
  for (int i = 0; i < 3; ++i) old[i] = s[i] - gv[i];
  for (int it = 1; it <= 20; ++it) {
    gyro(old);
    for (int i = 0; i < 3; ++i) cur[i] = s[i] - gv[i];
    const double d[3] = {cur[0] - old[0], cur[1] - old[1], cur[2] - old[2]};
    if (sqrt(dot3(d, d)) / sqrt(dot3(cur, cur)) < 1e-3) {
      double B[3];
      Field<M>::B(f, t, cur[0], cur[1], cur[2], B);
      const double vp = dot3(v, B) / sqrt(dot3(B, B));
      const double sp = sqrt(vsq);
      const double gamma = 1.0 / sqrt(1.0 - (sp / kC) * (sp / kC));
      const double ppar = mass * gamma * vp;
      // utils.magnetic_moment, rapt/utils.py:214-216
      const double vpar = ppar / (mass * gamma);
      double ub[3], Bm;
      unit_and_mag<M>(f, t, cur[0], cur[1], cur[2], ub, Bm);
      mu = gamma * gamma * mass * (sp - vpar) * (sp + vpar) / (2.0 * Bm);
      vspeed = sp;
      g[0] = cur[0]; g[1] = cur[1]; g[2] = cur[2]; g[3] = ppar; g[4] = 0.0; g[5] = 0.0;
      return true;
    }
    for (int i = 0; i < 3; ++i) old[i] = cur[i];
  }
  return false;
}

// Particle.init(GuidingCenter) (rapt/Particle.py:149-164): speed and parallel
// speed from mu, |B| and ppar at the GC's time t_gc, then utils.GCtoFP with
// gyrophase 0 (utils.py:376-433). GCtoFP is called with the new Particle's
// tcur, which is 0 for a freshly constructed Particle (quirk kept), then
// Particle.__init__ sets p = gamma m v (Particle.py:105-109).
template <int M>
__device__ void gc_to_particle(const FieldP& f, double t_gc, const double* g, double mu, double mass,
                               double charge, double* s) {
  const double ppar = g[3];
  double ub[3], Bm;
  unit_and_mag<M>(f, t_gc, g[0], g[1], g[2], ub, Bm);
  const double gammasq = 1.0 + 2.0 * mu * Bm / (mass * kC * kC) + (ppar / mass / kC) * (ppar / mass / kC);
  double v;
  if (sqrt(gammasq) - 1.0 < 1e-6) v = sqrt(2.0 * mu * Bm / mass + (ppar / mass) * (ppar / mass));
  else v = kC * sqrt(1.0 - 1.0 / gammasq);
  const double vpar = ppar / mass / sqrt(gammasq);
  // GCtoFP at t = 0
  double B[3];
  Field<M>::B(f, 0.0, g[0], g[1], g[2], B);
  const double bn = sqrt(dot3(B, B));
  const double b[3] = {B[0] / bn, B[1] / bn, B[2] / bn};
  const double pa = acos(vpar / v);
  const double gamma = 1.0 / sqrt(1.0 - (v / kC) * (v / kC));
  const double rc = gamma * mass * sqrt((v - vpar) * (v + vpar)) / (fabs(charge) * bn);
  double u[3];
  if (B[0] == 0.0) { u[0] = 1.0; u[1] = 0.0; u[2] = 0.0; }       // utils.getperp, utils.py:328-374
  else if (B[1] == 0.0) { u[0] = 0.0; u[1] = 1.0; u[2] = 0.0; }
  else if (B[2] == 0.0) { u[0] = 0.0; u[1] = 0.0; u[2] = 1.0; }
  else {
    const double cc = -1.0 * (B[0] + B[1]) / B[2];
    const double nn = sqrt(2.0 + cc * cc);
    u[0] = 1.0 / nn; u[1] = 1.0 / nn; u[2] = cc / nn;
  }
  const double un = sqrt(dot3(u, u));
  u[0] /= un; u[1] /= un; u[2] /= un;
  double w[3];
  cross3(b, u, w);
  const double sq = (charge > 0.0) ? 1.0 : ((charge < 0.0) ? -1.0 : 0.0);
  const double cp = cos(pa), sp = sin(pa);
  double pos[3], vel[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    pos[i] = g[i] + rc * (1.0 * u[i] + 0.0 * w[i]);
    vel[i] = v * (cp * b[i] + sq * sp * 0.0 * u[i] - sq * sp * 1.0 * w[i]);
  }
  const double gv = 1.0 / sqrt(1.0 - dot3(vel, vel) / (kC * kC));
#pragma unroll
  for (int i = 0; i < 3; ++i) { s[i] = pos[i]; s[3 + i] = mass * gv * vel[i]; }
}

// ---------------------------------------------------------------- shared lane logic
__device__ __forceinline__ unsigned long long warp_sum(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}

struct LaneStats {
  unsigned long long acc = 0, rej = 0, rhs = 0, sw = 0, done = 0, fail = 0, pend = 0;
  __device__ void flush(Scratch* S) {
    const unsigned long long a = warp_sum(acc), r = warp_sum(rej), h = warp_sum(rhs), s = warp_sum(sw),
                             d = warp_sum(done), f = warp_sum(fail), p = warp_sum(pend);
    if ((threadIdx.x & 31) == 0) {
      if (a) atomicAdd(&S->accepted, a);
      if (r) atomicAdd(&S->rejected, r);
      if (h) atomicAdd(&S->rhs, h);
      if (s) atomicAdd(&S->switches, s);
      if (d) atomicAdd(&S->done, d);
      if (f) atomicAdd(&S->failed, f);
      if (p) atomicAdd(&S->pending, p);
    }
  }
};

// Warp-wide refill: every lane without a tracer takes the next queue index
// until it holds a tracer of this kernel's mode or the queue is exhausted.
// The queue runs over positions 0..n-1; E.order maps a position to a tracer
// (longest expected work first, so that the lanes that finish last at the end
// of a launch hold the shortest tracers). Must be called by all 32 lanes.
template <class LoadFn>
__device__ __forceinline__ void warp_refill(unsigned long long* queue, const DevEnsemble& E, int mode, int64_t& idx,
                                            bool& exhausted, LoadFn&& load) {
  const int lane = threadIdx.x & 31;
  for (;;) {
    const bool need = (idx < 0) && !exhausted;
    const unsigned m = __ballot_sync(kFull, need);
    if (m == 0u) break;
    const int leader = __ffs(m) - 1;
    unsigned long long base = 0ull;
    if (lane == leader) base = atomicAdd(queue, (unsigned long long)__popc(m));
    base = __shfl_sync(kFull, base, leader);
    if (need) {
      const unsigned long long q = base + (unsigned long long)__popc(m & ((1u << lane) - 1u));
      if (q >= (unsigned long long)E.n) {
        exhausted = true;
      } else {
        const int64_t k = E.order ? (int64_t)E.order[q] : (int64_t)q;
        if (E.mode[k] == mode && !(E.flags[k] & RAPT_FLAG_DONE) && E.status[k] != RAPT_ST_ROWS_FULL) {
          idx = k;
          load(idx);
        }
      }
    }
  }
}

__device__ __forceinline__ void put_row(const DevEnsemble& E, const KParams& P, int64_t idx, int& nrows, double t,
                                        const double* s, int ns, int mode) {
  double* r = E.rows + ((size_t)idx * (size_t)P.max_rows + (size_t)nrows) * 7;
  r[0] = t;
#pragma unroll
  for (int i = 0; i < 6; ++i) r[1 + i] = (i < ns) ? s[i] : 0.0;
  E.row_mode[(size_t)idx * (size_t)P.max_rows + (size_t)nrows] = (int8_t)mode;
  ++nrows;
}

// ---------------------------------------------------------------- particle kernel
// TAB 0: DOP853 with beta 0.1 (Particle.py:300); TAB 1: RKF45 (rkf.py).
template <int M, int TAB>
__global__ void __launch_bounds__(128) k_particle(DevEnsemble E, KParams P, Scratch* S) {
  int64_t idx = -1;
  bool exhausted = false;
  long long budget = P.budget;
  LaneStats st;

  double y[6] = {0, 0, 0, 0, 0, 0}, k1[6] = {0, 0, 0, 0, 0, 0};
  double rt = 0, t_row = 0, tcur = 0, dt = 0, stop = 0, igm = 0, mass = 0, mass2 = 0, charge = 0, delta = 0,
         rowt = 0;
  long long nacc = 0, nrej = 0, nfcn = 0;
  int status = 0, flags = 0, nrows = 0, nsw = 0, nseg = 0, nswitch = 0;
  bool k1_valid = false, seg_ok = true, in_interval = false;
  double xend = 0, h = 0, facold = 1e-4, hmax = 0, posneg = 1;
  bool reject = false, last = false;
  int nst = 0, nacc_int = 0;

  // DOP853 controller constants as SciPy passes them (dfactor 0.3, ifactor 6).
  constexpr double beta = 0.1, safe = 0.9;
  constexpr double expo1 = 1.0 / 8.0 - beta * 0.2, facc1 = 1.0 / 0.3, facc2 = 1.0 / 6.0;

  auto begin_segment = [&](double seg_delta) {
    // Particle.advance start: t0 = trajectory[-1,0], gm from the momentum,
    // dt = cyclotron_period / cyclotronresolution (Particle.py:271-282).
    rt = t_row;
    const double gm = sqrt(mass * mass + (y[3] * y[3] + y[4] * y[4] + y[5] * y[5]) / (kC * kC));
    igm = 1.0 / gm;
    const double vel[3] = {y[3] / gm, y[4] / gm, y[5] / gm};
    dt = cyc_period_vel<M>(P.f, t_row, y, vel, mass, charge) / P.cycres;
    stop = t_row + seg_delta;
    seg_ok = true;
    k1_valid = false;
    in_interval = false;
  };

  auto load = [&](int64_t k) {
#pragma unroll
    for (int i = 0; i < 6; ++i) y[i] = E.s[i][k];
    rt = E.t_int[k]; t_row = E.t_row[k]; tcur = E.tcur[k];
    mass = E.mass[k]; charge = E.charge[k]; delta = E.delta[k];
    mass2 = mass * mass;
    nacc = E.naccept[k]; nrej = E.nreject[k]; nfcn = E.nfcn[k];
    status = E.status[k]; flags = E.flags[k]; nrows = E.nrows[k]; nswitch = E.nswitch[k];
    nseg = E.nseg[k];
    nsw = nswitch;
    in_interval = false;
    k1_valid = false;
    seg_ok = true;
    if (E.seg_active[k]) {
      stop = E.seg_stop[k]; dt = E.seg_dt[k]; igm = E.seg_gm[k];
    } else {
      begin_segment((P.kind == RAPT_KIND_ADAPTIVE && nseg > 0) ? delta - tcur : delta);
    }
  };

  auto store = [&](int64_t k, bool active) {
#pragma unroll
    for (int i = 0; i < 6; ++i) E.s[i][k] = y[i];
    E.t_int[k] = rt; E.t_row[k] = t_row; E.tcur[k] = tcur;
    E.naccept[k] = nacc; E.nreject[k] = nrej; E.nfcn[k] = nfcn;
    E.status[k] = status; E.flags[k] = flags; E.nrows[k] = nrows; E.nswitch[k] = nswitch; E.nseg[k] = nseg;
    E.seg_active[k] = active ? 1 : 0;
    E.seg_stop[k] = stop; E.seg_dt[k] = dt; E.seg_gm[k] = igm;
  };

  for (;;) {
    warp_refill(&S->queue[0], E, RAPT_MODE_PARTICLE, idx, exhausted, load);
    if (__all_sync(kFull, idx < 0)) break;
    if (idx < 0) continue;

    const ParticleRHS<M> rhs{P.f, charge, mass2, igm, P.enforce_eq != 0};
    bool release = false;

    if (!in_interval) {
      if (!(seg_ok && rt < stop)) {
        // end of this Particle.advance() call
        bool more = false;
        if (P.kind == RAPT_KIND_ADAPTIVE && status != RAPT_ST_NONFINITE && status != RAPT_ST_OUT_OF_GRID && status != RAPT_ST_RKF_HMIN &&
            tcur < delta) {
          if (nseg + 1 >= P.max_segments) {
            status = RAPT_ST_ADAPTIVE_LIMIT;
          } else {
            more = true;
            ++nseg;
            begin_segment(delta - tcur);
          }
        }
        if (!more) {
          flags |= RAPT_FLAG_DONE;
          st.done++;
          if (status != RAPT_ST_OK) st.fail++;
          store(idx, false);
          idx = -1;
          continue;
        }
      }
      if (budget <= 0) {
        store(idx, true);
        idx = -1;
        exhausted = true;
        st.pend++;
        continue;
      }
      if (nrows + 2 > P.max_rows) {
        status = RAPT_ST_ROWS_FULL;
        store(idx, true);
        idx = -1;
        continue;
      }
      // start of one SciPy integrate(r.t + dt) call
      xend = rt + dt;
      rowt = rt + dt;
      hmax = fabs(xend - rt);
      posneg = copysign(1.0, xend - rt);
      nst = 0;
      nacc_int = 0;
      if (TAB == 0) {
        if (!k1_valid) { rhs(rt, y, k1); k1_valid = true; st.rhs++; }
        h = hinit<6>(rhs, rt, y, k1, posneg, 1.0 / 8.0, hmax, P.rtol, P.atol);
        st.rhs++;
        nfcn += 2;
        facold = 1e-4;
        reject = false;
        last = false;
      } else {
        h = hmax;
      }
      in_interval = true;
    }

    bool ended = false;
    int fail = 0;
    if (TAB == 0) {
      if (nst > P.nsteps) { ended = true; fail = RAPT_ST_MAXSTEPS; }
      else if (0.1 * fabs(h) <= fabs(rt) * kUround) { ended = true; fail = RAPT_ST_HMIN; }
      else {
        if ((rt + 1.01 * h - xend) * posneg > 0.0) { h = xend - rt; last = true; }
        ++nst;
        --budget;
        double y1[6], err;
        dop853_attempt<6>(rhs, rt, y, k1, h, P.rtol, P.atol, y1, err);
        nfcn += 11;
        st.rhs += 11;
        const double fac11 = pow_fp64(err, expo1);
        double fac = fac11 / pow_fp64(facold, beta);
        fac = fmax(facc2, fmin(facc1, fac / safe));
        double hnew = h / fac;
        if (left_grid<M>(err)) {
          ended = true;
          fail = RAPT_ST_OUT_OF_GRID;
        } else if (err <= 1.0) {
          facold = fmax(err, 1.0e-4);
          ++nacc; ++nacc_int; st.acc++;
          const double xph = rt + h;
          rhs(xph, y1, k1);
          nfcn += 1;
          st.rhs++;
#pragma unroll
          for (int i = 0; i < 6; ++i) y[i] = y1[i];
          rt = xph;
          if (last) {
            h = hnew;
            ended = true;
          } else {
            if (fabs(hnew) > hmax) hnew = posneg * hmax;
            if (reject) hnew = posneg * fmin(fabs(hnew), fabs(h));
            reject = false;
            h = hnew;
          }
        } else {
          // a rejected DOP853 step shrinks by dfactor (h * 0.3), as SciPy's dop853 does
          hnew = h / facc1;
          reject = true;
          if (nacc_int >= 1) { ++nrej; st.rej++; }
          last = false;
          h = hnew;
        }
      }
    } else {
      if (!(rt < xend)) { ended = true; }
      else if (nst > 1000000) { ended = true; fail = RAPT_ST_MAXSTEPS; }
      else {
        if (rt + h > xend) h = xend - rt;
        double y1[6], r;
        rkf45_attempt<6, M == RAPT_GRID>(rhs, rt, y, h, y1, r);
        ++nst;
        --budget;
        nfcn += 6;
        st.rhs += 6;
        if (left_grid<M>(r)) {
          ended = true;
          fail = RAPT_ST_OUT_OF_GRID;
        } else {
          if (r <= P.rkf_tol) {
            rt = rt + h;
#pragma unroll
            for (int i = 0; i < 6; ++i) y[i] = y1[i];
            ++nacc; st.acc++;
          } else {
            ++nrej; st.rej++;
          }
          h = h * fmin(fmax(0.84 * pow_fp64(P.rkf_tol / r, 0.25), 0.1), 4.0);
          if (h > hmax) h = hmax;
          else if (h < P.rkf_hmin) { ended = true; fail = RAPT_ST_RKF_HMIN; }
          if (!ended && !(rt < xend)) ended = true;
        }
      }
    }

    if (ended) {
      in_interval = false;
      if (fail) { seg_ok = false; status = fail; }
      if (!all_finite<6>(y)) { seg_ok = false; status = RAPT_ST_NONFINITE; }
      // a Grid step outside the grid (ValueError) or an RKF45 step below hmin
      // (RuntimeError): the reference raises inside the interval, adding no row
      const bool row = !(M == RAPT_GRID && status == RAPT_ST_OUT_OF_GRID) && status != RAPT_ST_RKF_HMIN;
      if (row) {
        t_row = rowt;
        tcur = rt + dt;  // Particle.py:306
        put_row(E, P, idx, nrows, rowt, y, 6, RAPT_MODE_PARTICLE);
      }
      if (row && (flags & RAPT_FLAG_CHECK_ADIABATICITY) && status != RAPT_ST_NONFINITE &&
          particle_isadiabatic<M>(P, t_row, y, mass, charge)) {
        if (P.kind == RAPT_KIND_ADAPTIVE) {
          double g[6], mu, vs;
          if (particle_to_gc<M>(P.f, t_row, y, mass, charge, g, mu, vs)) {
#pragma unroll
            for (int i = 0; i < 6; ++i) y[i] = g[i];
            E.mu[idx] = mu;
            E.v[idx] = vs;
            E.mode[idx] = RAPT_MODE_GC;
            tcur = t_row;
            rt = t_row;
            ++nseg;
            if (nsw < P.max_sw) {
              E.sw_time[(size_t)idx * P.max_sw + nsw] = tcur;
              E.sw_mode[(size_t)idx * P.max_sw + nsw] = RAPT_MODE_GC;
            }
            ++nsw;
            nswitch = nsw;
            // the first row of a guiding-centre segment carries its mu and v in
            // the two columns a guiding-centre row does not use
            const double first[6] = {g[0], g[1], g[2], g[3], mu, vs};
            put_row(E, P, idx, nrows, t_row, first, 6, RAPT_MODE_GC);
            st.sw++;
            st.pend++;
          } else {
            status = RAPT_ST_GC_NOCONV;
            flags |= RAPT_FLAG_DONE;
            st.done++;
            st.fail++;
          }
        } else {
          flags |= RAPT_FLAG_RAISED | RAPT_FLAG_DONE;
          st.done++;
        }
        release = true;
      }
    }
    if (release) {
      store(idx, false);
      idx = -1;
    }
  }
  st.flush(S);
}

// ---------------------------------------------------------------- guiding-centre kernel
// TAB 0: DOPRI5 (GuidingCenter.py:450, SciPy defaults; beta 0 -> 0.04); TAB 1: RKF45.
// LRN (DOPRI5 only): 0 plain, 1 training-sample collection, 2 MLP step proposals
// (a proposal replaces the controller's next step after an accepted step and
// HINIT at the next interval; a rejected proposal falls back to the controller).
template <int M, int TAB, int LRN = 0>
__global__ void __launch_bounds__(128) k_gc(DevEnsemble E, KParams P, Scratch* S) {
  static_assert(LRN == 0 || TAB == 0, "the step learner drives the DOPRI5 controller");
  int64_t idx = -1;
  bool exhausted = false;
  long long budget = P.budget;
  LaneStats st;
  StepLearner<LRN> lr;
  lr.init(P);

  double y[4] = {0, 0, 0, 0}, k1[4] = {0, 0, 0, 0};
  double rt = 0, t_row = 0, tcur = 0, dt = 0, stop = 0, mass = 0, charge = 0, delta = 0, mu = 0, vs = 0;
  double qinv = 0, minv = 0, kmu = 0, inv_mc = 0, igv = 0, gmv = 0, gmv2 = 0;
  long long nacc = 0, nrej = 0, nfcn = 0;
  int status = 0, flags = 0, nrows = 0, nsw = 0, nseg = 0, nswitch = 0;
  bool k1_valid = false, seg_ok = true, in_interval = false;
  double xend = 0, h = 0, facold = 1e-4, hmax = 0, posneg = 1;
  bool reject = false, last = false;
  int nst = 0, nacc_int = 0;

  constexpr double beta = 0.04, safe = 0.9;
  constexpr double expo1 = 0.2 - beta * 0.75, facc1 = 1.0 / 0.2, facc2 = 1.0 / 10.0;

  auto begin_segment = [&](double seg_delta) {
    // GuidingCenter.advance start (GuidingCenter.py:443-451)
    rt = t_row;
    dt = P.gctimestep;
    stop = t_row + seg_delta;
    seg_ok = true;
    if (dt == 0.0 && P.fl_scratch) {  // bounce-period cadence
      double* scr = P.fl_scratch + (size_t)(blockIdx.x * blockDim.x + threadIdx.x) * (size_t)P.fl_stride;
      dt = gc_bounceperiod<M>(P.f, t_row, y, mu, mass, P.flres, scr, P.fl_cap) / P.bounceres;
      if (!(dt > 0.0) || !isfinite(dt)) { seg_ok = false; status = RAPT_ST_FIELDLINE; dt = 0.0; }
    }
    if (!(dt > 0.0) && status != RAPT_ST_FIELDLINE) { seg_ok = false; status = RAPT_ST_BAD_INPUT; }
    k1_valid = false;
    in_interval = false;
  };

  auto load = [&](int64_t k) {
#pragma unroll
    for (int i = 0; i < 4; ++i) y[i] = E.s[i][k];
    rt = E.t_int[k]; t_row = E.t_row[k]; tcur = E.tcur[k];
    mass = E.mass[k]; charge = E.charge[k]; delta = E.delta[k];
    mu = E.mu[k]; vs = E.v[k];
    {
      // per-tracer constants of the guiding-centre equations
      const double gv = 1.0 / sqrt(1.0 - (vs / kC) * (vs / kC));
      qinv = 1.0 / charge; minv = 1.0 / mass; kmu = 2.0 * mu / (mass * kC * kC); inv_mc = 1.0 / (mass * kC);
      igv = 1.0 / gv; gmv = gv * mass; gmv2 = gv * mass * vs * vs;
    }
    nacc = E.naccept[k]; nrej = E.nreject[k]; nfcn = E.nfcn[k];
    status = E.status[k]; flags = E.flags[k]; nrows = E.nrows[k]; nswitch = E.nswitch[k];
    nseg = E.nseg[k];
    nsw = nswitch;
    in_interval = false;
    k1_valid = false;
    seg_ok = true;
    if (E.seg_active[k]) {
      stop = E.seg_stop[k]; dt = E.seg_dt[k];
    } else {
      begin_segment((P.kind == RAPT_KIND_ADAPTIVE && nseg > 0) ? delta - tcur : delta);
    }
    lr.load(mass, charge, vs, 1.0);
  };

  auto store = [&](int64_t k, bool active) {
#pragma unroll
    for (int i = 0; i < 4; ++i) E.s[i][k] = y[i];
    E.s[4][k] = 0.0;
    E.s[5][k] = 0.0;
    E.t_int[k] = rt; E.t_row[k] = t_row; E.tcur[k] = tcur;
    E.naccept[k] = nacc; E.nreject[k] = nrej; E.nfcn[k] = nfcn;
    E.status[k] = status; E.flags[k] = flags; E.nrows[k] = nrows; E.nswitch[k] = nswitch; E.nseg[k] = nseg;
    E.seg_active[k] = active ? 1 : 0;
    E.seg_stop[k] = stop; E.seg_dt[k] = dt;
  };

  for (;;) {
    warp_refill(&S->queue[1], E, RAPT_MODE_GC, idx, exhausted, load);
    if (__all_sync(kFull, idx < 0)) break;
    lr.infer(P, h);
    if (idx < 0) continue;

    const GcRHS<M> rhs{P.f, charge, qinv, mu, minv, kmu, inv_mc, igv, gmv, gmv2, P.gc_eom, P.enforce_eq != 0};
    bool release = false;

    if (!in_interval) {
      if (!(seg_ok && rt < stop)) {
        bool more = false;
        if (P.kind == RAPT_KIND_ADAPTIVE && status != RAPT_ST_NONFINITE && status != RAPT_ST_BAD_INPUT &&
            status != RAPT_ST_OUT_OF_GRID && status != RAPT_ST_RKF_HMIN && tcur < delta) {
          if (nseg + 1 >= P.max_segments) {
            status = RAPT_ST_ADAPTIVE_LIMIT;
          } else {
            more = true;
            ++nseg;
            begin_segment(delta - tcur);
          }
        }
        if (!more) {
          flags |= RAPT_FLAG_DONE;
          st.done++;
          if (status != RAPT_ST_OK) st.fail++;
          store(idx, false);
          idx = -1;
          continue;
        }
      }
      if (budget <= 0) {
        store(idx, true);
        idx = -1;
        exhausted = true;
        st.pend++;
        continue;
      }
      if (nrows + 2 > P.max_rows) {
        status = RAPT_ST_ROWS_FULL;
        store(idx, true);
        idx = -1;
        continue;
      }
      xend = rt + dt;
      hmax = fabs(xend - rt);
      posneg = copysign(1.0, xend - rt);
      nst = 0;
      nacc_int = 0;
      if (TAB == 0) {
        if (!k1_valid) { rhs(rt, y, k1); k1_valid = true; st.rhs++; }
        if (LRN == 2 && lr.have_prop) {
          // learned first step of the interval instead of HINIT
          h = posneg * fmin(fabs(h), hmax);
          lr.have_prop = false;
          nfcn += 1;
        } else {
          h = hinit<4>(rhs, rt, y, k1, posneg, 1.0 / 5.0, hmax, P.rtol, P.atol);
          st.rhs++;
          nfcn += 2;
        }
        facold = 1e-4;
        reject = false;
        last = false;
      } else {
        h = hmax;
      }
      in_interval = true;
    }

    bool ended = false;
    int fail = 0;
    if (TAB == 0) {
      if (nst > P.nsteps) { ended = true; fail = RAPT_ST_MAXSTEPS; }
      else if (0.1 * fabs(h) <= fabs(rt) * kUround) { ended = true; fail = RAPT_ST_HMIN; }
      else {
        if ((rt + 1.01 * h - xend) * posneg > 0.0) { lr.before_clip(h); h = xend - rt; last = true; }
        ++nst;
        --budget;
        double y1[4], k7[4], err;
        dopri5_attempt_rolled<4>(rhs, rt, y, k1, h, P.rtol, P.atol, y1, k7, err);
        nfcn += 6;
        st.rhs += 6;
        lr.on_attempt(P, h, err, last);
        const double fac11 = pow_fp64(err, expo1);
        double fac = fac11 / pow_fp64(facold, beta);
        fac = fmax(facc2, fmin(facc1, fac / safe));
        double hnew = h / fac;
        if (left_grid<M>(err)) {
          ended = true;
          fail = RAPT_ST_OUT_OF_GRID;
        } else if (err <= 1.0) {
          const double errprev = facold;
          const bool rej_before = reject;
          const double hstep = h;
          facold = fmax(err, 1.0e-4);
          ++nacc; ++nacc_int; st.acc++;
#pragma unroll
          for (int i = 0; i < 4; ++i) { k1[i] = k7[i]; y[i] = y1[i]; }
          rt = rt + h;
          const bool was_last = last;
          if (last) {
            h = hnew;
            ended = true;
          } else {
            if (fabs(hnew) > hmax) hnew = posneg * hmax;
            if (reject) hnew = posneg * fmin(fabs(hnew), fabs(h));
            reject = false;
            h = hnew;
          }
          lr.on_accept(P, idx, nacc, hstep, err, errprev, h, hmax, was_last, rej_before, nst - nacc_int <= 8,
                     (flags & RAPT_FLAG_CHECK_ADIABATICITY) != 0,
                     (float)y[0], (float)y[1],
                       (float)y[2], (float)y[3], vs, interval_progress(xend, rt, hmax));
        } else {
          hnew = h / fmin(facc1, fac11 / safe);
          reject = true;
          if (nacc_int >= 1) { ++nrej; st.rej++; }
          last = false;
          h = hnew;
        }
      }
    } else {
      if (!(rt < xend)) { ended = true; }
      else if (nst > 1000000) { ended = true; fail = RAPT_ST_MAXSTEPS; }
      else {
        if (rt + h > xend) h = xend - rt;
        double y1[4], r;
        rkf45_attempt<4, M == RAPT_GRID>(rhs, rt, y, h, y1, r);
        ++nst;
        --budget;
        nfcn += 6;
        st.rhs += 6;
        if (left_grid<M>(r)) {
          ended = true;
          fail = RAPT_ST_OUT_OF_GRID;
        } else {
          if (r <= P.rkf_tol) {
            rt = rt + h;
#pragma unroll
            for (int i = 0; i < 4; ++i) y[i] = y1[i];
            ++nacc; st.acc++;
          } else {
            ++nrej; st.rej++;
          }
          h = h * fmin(fmax(0.84 * pow_fp64(P.rkf_tol / r, 0.25), 0.1), 4.0);
          if (h > hmax) h = hmax;
          else if (h < P.rkf_hmin) { ended = true; fail = RAPT_ST_RKF_HMIN; }
          if (!ended && !(rt < xend)) ended = true;
        }
      }
    }

    if (ended) {
      in_interval = false;
      if (fail) { seg_ok = false; status = fail; }
      if (!all_finite<4>(y)) { seg_ok = false; status = RAPT_ST_NONFINITE; }
      // a Grid step outside the grid (ValueError) or an RKF45 step below hmin
      // (RuntimeError): the reference raises inside the interval, adding no row
      const bool row = !(M == RAPT_GRID && status == RAPT_ST_OUT_OF_GRID) && status != RAPT_ST_RKF_HMIN;
      if (row) {
        t_row = rt;
        tcur = rt;
        put_row(E, P, idx, nrows, rt, y, 4, RAPT_MODE_GC);
      }
      const bool row_chk = row && (flags & RAPT_FLAG_CHECK_ADIABATICITY) && status != RAPT_ST_NONFINITE;
      const bool nonadi = row_chk && !gc_isadiabatic<M>(P, t_row, y, mu, mass, charge);
      if (row_chk) lr.on_row(P, nonadi);
      if (nonadi) {
        if (P.kind == RAPT_KIND_ADAPTIVE) {
          double s6[6];
          gc_to_particle<M>(P.f, t_row, y, mu, mass, charge, s6);
          // the particle state is written directly; this kernel releases the tracer
#pragma unroll
          for (int i = 0; i < 6; ++i) E.s[i][idx] = s6[i];
          E.mode[idx] = RAPT_MODE_PARTICLE;
          tcur = t_row;
          rt = t_row;
          ++nseg;
          if (nsw < P.max_sw) {
            E.sw_time[(size_t)idx * P.max_sw + nsw] = tcur;
            E.sw_mode[(size_t)idx * P.max_sw + nsw] = RAPT_MODE_PARTICLE;
          }
          ++nsw;
          nswitch = nsw;
          put_row(E, P, idx, nrows, t_row, s6, 6, RAPT_MODE_PARTICLE);
          st.sw++;
          st.pend++;
          // store() below must not overwrite the particle state with the GC state
          E.t_int[idx] = rt; E.t_row[idx] = t_row; E.tcur[idx] = tcur;
          E.naccept[idx] = nacc; E.nreject[idx] = nrej; E.nfcn[idx] = nfcn;
          E.status[idx] = status; E.flags[idx] = flags; E.nrows[idx] = nrows; E.nswitch[idx] = nswitch;
          E.nseg[idx] = nseg; E.seg_active[idx] = 0;
          idx = -1;
          continue;
        } else {
          flags |= RAPT_FLAG_RAISED | RAPT_FLAG_DONE;
          st.done++;
        }
        release = true;
      }
    }
    if (release) {
      store(idx, false);
      idx = -1;
    }
  }
  st.flush(S);
}

}  // namespace rapt
