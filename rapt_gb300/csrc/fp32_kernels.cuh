// fp32_kernels.cuh -- persistent kernels of the FP32-stage form.
//
// Same work distribution, output-interval loop, Adaptive segments and status
// handling as tracer_kernels.cuh (Particle.py:230-309, GuidingCenter.py:397-458,
// Adaptive.py:187-222); the RK stages use the float-float arithmetic of fp32_form.cuh. Adiabaticity tests and
// the particle <-> guiding-centre conversions run in FP64 on the SI state.
#pragma once
#include "fp32_form.cuh"

namespace rapt {

template <int M>
// 2 blocks per SM (255 registers): measured best for the 12-stage DOP853
// float-float kernel (262,144 protons and electrons in the Earth dipole, 50
// gyro-periods each: 2 blocks/SM 1.37e8 accepted steps/s, 3: 1.26e8,
// 4: 1.18e8, 6: 1.05e8, 8: 1.02e8).
__global__ void __launch_bounds__(128, 2) k_particle32(DevEnsemble E, const __grid_constant__ KParams P,
                                                       Scratch* S) {
  int64_t idx = -1;
  bool exhausted = false;
  long long budget = P.budget;
  LaneStats st;

  DF y[6];
  DF k1[6];
  double scale[6] = {1, 1, 1, 1, 1, 1};
  double rt = 0, t_row = 0, tcur = 0, dt = 0, stop = 0, mass = 0, charge = 0, delta = 0, rowt = 0;
  DF qmc{0.f, 0.f}, qm{0.f, 0.f}, igam{0.f, 0.f};
  long long nacc = 0, nrej = 0, nfcn = 0;
  int status = 0, flags = 0, nrows = 0, nsw = 0, nseg = 0, nswitch = 0;
  bool k1_valid = false, seg_ok = true, in_interval = false;
  double xend = 0, h = 0, hmax = 0, posneg = 1;
  StepFactorF32 ctl{1.f, 1.f};
  bool reject = false, last = false;
  int nst = 0, nacc_int = 0;

  constexpr float beta = 0.1f, safe = 0.9f;
  constexpr float expo1 = 1.0f / 8.0f - beta * 0.2f, facc1 = 1.0f / 0.3f, facc2 = 1.0f / 6.0f;

  auto state_si = [&](double* s) {
    for (int i = 0; i < 6; ++i) s[i] = df_to_double(y[i]) * scale[i];
  };
  auto begin_segment = [&](double seg_delta) {
    rt = t_row;
    double s[6];
    state_si(s);
    const double gm = sqrt(mass * mass + (s[3] * s[3] + s[4] * s[4] + s[5] * s[5]) / (kC * kC));
    igam = df_from_double(mass / gm);
    const double vel[3] = {s[3] / gm, s[4] / gm, s[5] / gm};
    dt = cyc_period_vel<M>(P.f, t_row, s, vel, mass, charge) / P.cycres;
    stop = t_row + seg_delta;
    seg_ok = true;
    k1_valid = false;
    in_interval = false;
  };
  auto load = [&](int64_t k) {
    mass = E.mass[k]; charge = E.charge[k]; delta = E.delta[k];
    const double mc = mass * kC;
    for (int i = 0; i < 3; ++i) { scale[i] = 1.0; scale[3 + i] = mc; }
    for (int i = 0; i < 6; ++i) y[i] = df_from_double(E.s[i][k] / scale[i]);
    qmc = df_from_double(charge / mc);
    qm = df_from_double(charge / mass);
    rt = E.t_int[k]; t_row = E.t_row[k]; tcur = E.tcur[k];
    nacc = E.naccept[k]; nrej = E.nreject[k]; nfcn = E.nfcn[k];
    status = E.status[k]; flags = E.flags[k]; nrows = E.nrows[k]; nswitch = E.nswitch[k];
    nseg = E.nseg[k];
    nsw = nswitch;
    in_interval = false;
    k1_valid = false;
    seg_ok = true;
    if (E.seg_active[k]) {
      stop = E.seg_stop[k]; dt = E.seg_dt[k]; igam = df_from_double(mass * E.seg_gm[k]);
    } else {
      begin_segment((P.kind == RAPT_KIND_ADAPTIVE && nseg > 0) ? delta - tcur : delta);
    }
  };
  auto store = [&](int64_t k, bool active) {
    double s[6];
    state_si(s);
    for (int i = 0; i < 6; ++i) E.s[i][k] = s[i];
    E.t_int[k] = rt; E.t_row[k] = t_row; E.tcur[k] = tcur;
    E.naccept[k] = nacc; E.nreject[k] = nrej; E.nfcn[k] = nfcn;
    E.status[k] = status; E.flags[k] = flags; E.nrows[k] = nrows; E.nswitch[k] = nswitch; E.nseg[k] = nseg;
    E.seg_active[k] = active ? 1 : 0;
    E.seg_stop[k] = stop; E.seg_dt[k] = dt; E.seg_gm[k] = df_to_double(igam) / mass;
  };

  for (;;) {
    warp_refill(&S->queue[0], E, RAPT_MODE_PARTICLE, idx, exhausted, load);
    if (__all_sync(kFull, idx < 0)) break;
    if (idx < 0) continue;

    const ParticleRHSdf<M> rhs{P.f, qmc, qm, igam, P.enforce_eq != 0};
    bool release = false;

    if (!in_interval) {
      if (!(seg_ok && rt < stop)) {
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
      if (budget <= 0) { store(idx, true); idx = -1; exhausted = true; st.pend++; continue; }
      if (nrows + 2 > P.max_rows) { status = RAPT_ST_ROWS_FULL; store(idx, true); idx = -1; continue; }
      xend = rt + dt;
      rowt = rt + dt;
      hmax = fabs(xend - rt);
      posneg = copysign(1.0, xend - rt);
      nst = 0;
      nacc_int = 0;
      if (!k1_valid) {
        rhs(rt, y, k1);
        k1_valid = true;
        st.rhs++;
      }
      h = hinit_df<6>(rhs, rt, y, k1, scale, posneg, 1.0 / 8.0, hmax, P.rtol, P.atol);
      st.rhs++;
      nfcn += 2;
      ctl.reset(beta);
      reject = false;
      last = false;
      in_interval = true;
    }

    bool ended = false;
    int fail = 0;
    if (nst > P.nsteps) { ended = true; fail = RAPT_ST_MAXSTEPS; }
    else if (0.1 * fabs(h) <= fabs(rt) * kUround) { ended = true; fail = RAPT_ST_HMIN; }
    else {
      if ((rt + 1.01 * h - xend) * posneg > 0.0) { h = xend - rt; last = true; }
      ++nst;
      --budget;
      DF y1[6];
      double err;
      dop853_attempt_df<6>(rhs, rt, y, k1, h, scale, P.rtol, P.atol, y1, err);
      nfcn += 11;
      st.rhs += 11;
      double hnew = h * (double)ctl.accept_factor(err, expo1, safe, facc1, facc2);
      if (left_grid<M>(err)) {
        ended = true;
        fail = RAPT_ST_OUT_OF_GRID;
      } else if (err <= 1.0) {
        ctl.accepted(err, beta);
        ++nacc; ++nacc_int; st.acc++;
        const double xph = rt + h;
        for (int i = 0; i < 6; ++i) y[i] = y1[i];
        rhs(xph, y, k1);
        nfcn += 1;
        st.rhs++;
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
        hnew = h * 0.3;  // a rejected DOP853 step shrinks by dfactor (h * 0.3), as SciPy's dop853 does
        reject = true;
        if (nacc_int >= 1) { ++nrej; st.rej++; }
        last = false;
        h = hnew;
      }
    }

    if (ended) {
      in_interval = false;
      double s[6];
      state_si(s);
      if (fail) { seg_ok = false; status = fail; }
      if (!all_finite<6>(s)) { seg_ok = false; status = RAPT_ST_NONFINITE; }
      // a Grid step outside the grid (ValueError) or an RKF45 step below hmin
      // (RuntimeError): the reference raises inside the interval, adding no row
      const bool row = !(M == RAPT_GRID && status == RAPT_ST_OUT_OF_GRID) && status != RAPT_ST_RKF_HMIN;
      if (row) {
        t_row = rowt;
        tcur = rt + dt;
        put_row(E, P, idx, nrows, rowt, s, 6, RAPT_MODE_PARTICLE);
      }
      if (row && (flags & RAPT_FLAG_CHECK_ADIABATICITY) && status != RAPT_ST_NONFINITE &&
          particle_isadiabatic<M>(P, t_row, s, mass, charge)) {
        if (P.kind == RAPT_KIND_ADAPTIVE) {
          double g[6], mu, vs;
          if (particle_to_gc<M>(P.f, t_row, s, mass, charge, g, mu, vs)) {
            for (int i = 0; i < 6; ++i) E.s[i][idx] = g[i];
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
            const double first[6] = {g[0], g[1], g[2], g[3], mu, vs};
            put_row(E, P, idx, nrows, t_row, first, 6, RAPT_MODE_GC);
            st.sw++;
            st.pend++;
            E.t_int[idx] = rt; E.t_row[idx] = t_row; E.tcur[idx] = tcur;
            E.naccept[idx] = nacc; E.nreject[idx] = nrej; E.nfcn[idx] = nfcn;
            E.status[idx] = status; E.flags[idx] = flags; E.nrows[idx] = nrows; E.nswitch[idx] = nswitch;
            E.nseg[idx] = nseg; E.seg_active[idx] = 0;
            idx = -1;
            continue;
          }
          status = RAPT_ST_GC_NOCONV;
          flags |= RAPT_FLAG_DONE;
          st.done++;
          st.fail++;
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

template <int M, int LRN = 0>
// LRN: 0 plain controller, 1 training-sample collection, 2 MLP step proposals.
// 8 blocks of 128 threads per SM, 64 registers: the balance between resident
// warps (the float-float stages are long dependent FP32 chains) and the
// local-memory traffic of spills. Measured on the 1M guiding-centre step
// (FP32 / learned + FP32 accepted steps/s): 4 blocks/SM 1.44e9 / 1.04e9,
// 6: 1.45e9 / 1.15e9, 8: 1.51e9 / 1.21e9, 12: 1.30e9 / 1.04e9, 16: 0.95e9 / 0.79e9.
__global__ void __launch_bounds__(128, 8) k_gc32(DevEnsemble E, const __grid_constant__ KParams P, Scratch* S) {
  int64_t idx = -1;
  bool exhausted = false;
  long long budget = P.budget;
  LaneStats st;
  StepLearner<LRN> lr;
  lr.init(P);
  double errold = 1e-4;  // previous accepted error (learner feature)

  DF y[4];
  DF k1[4];
  double scale[4] = {1, 1, 1, 1};
  double rt = 0, t_row = 0, tcur = 0, dt = 0, stop = 0, mass = 0, charge = 0, delta = 0, mu = 0, vs = 0;
  DF kmu{0.f, 0.f}, mcq{0.f, 0.f}, muq{0.f, 0.f}, qmc{0.f, 0.f};
  long long nacc = 0, nrej = 0, nfcn = 0;
  int status = 0, flags = 0, nrows = 0, nsw = 0, nseg = 0, nswitch = 0;
  bool k1_valid = false, seg_ok = true, in_interval = false;
  double xend = 0, h = 0, hmax = 0, posneg = 1;
  StepFactorF32 ctl{1.f, 1.f};
  bool reject = false, last = false;
  int nst = 0, nacc_int = 0;

  constexpr float beta = 0.04f, safe = 0.9f;
  constexpr float expo1 = 0.2f - beta * 0.75f, facc1 = 1.0f / 0.2f, facc2 = 1.0f / 10.0f;

  auto state_si = [&](double* s) {
    for (int i = 0; i < 4; ++i) s[i] = df_to_double(y[i]) * scale[i];
    s[4] = 0.0;
    s[5] = 0.0;
  };
  auto begin_segment = [&](double seg_delta) {
    rt = t_row;
    dt = P.gctimestep;
    stop = t_row + seg_delta;
    seg_ok = true;
    if (dt == 0.0 && P.fl_scratch) {  // bounce-period cadence (GuidingCenter.py:443-446)
      double s4[6];
      state_si(s4);
      double* scr = P.fl_scratch + (size_t)(blockIdx.x * blockDim.x + threadIdx.x) * (size_t)P.fl_stride;
      dt = gc_bounceperiod<M>(P.f, t_row, s4, mu, mass, P.flres, scr, P.fl_cap) / P.bounceres;
      if (!(dt > 0.0) || !isfinite(dt)) { seg_ok = false; status = RAPT_ST_FIELDLINE; dt = 0.0; }
    }
    if (!(dt > 0.0) && status != RAPT_ST_FIELDLINE) { seg_ok = false; status = RAPT_ST_BAD_INPUT; }
    k1_valid = false;
    in_interval = false;
  };
  auto load = [&](int64_t k) {
    mass = E.mass[k]; charge = E.charge[k]; delta = E.delta[k];
    mu = E.mu[k]; vs = E.v[k];
    const double mc = mass * kC;
    scale[0] = scale[1] = scale[2] = 1.0;
    scale[3] = mc;
    for (int i = 0; i < 4; ++i) y[i] = df_from_double(E.s[i][k] / scale[i]);
    lr.load(mass, charge, vs, mc);
    kmu = df_from_double(2.0 * mu / (mass * kC * kC));
    mcq = df_from_double(mc / charge);
    muq = df_from_double(mu / charge);
    qmc = df_from_double(charge / mc);
    rt = E.t_int[k]; t_row = E.t_row[k]; tcur = E.tcur[k];
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
  };
  auto store = [&](int64_t k, bool active) {
    double s[6];
    state_si(s);
    for (int i = 0; i < 6; ++i) E.s[i][k] = s[i];
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

    const GcRHSdf<M> rhs{P.f, kmu, mcq, muq, qmc, P.enforce_eq != 0};
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
      if (budget <= 0) { store(idx, true); idx = -1; exhausted = true; st.pend++; continue; }
      if (nrows + 2 > P.max_rows) { status = RAPT_ST_ROWS_FULL; store(idx, true); idx = -1; continue; }
      xend = rt + dt;
      hmax = fabs(xend - rt);
      posneg = copysign(1.0, xend - rt);
      nst = 0;
      nacc_int = 0;
      if (!k1_valid) {
        rhs(rt, y, k1);
        k1_valid = true;
        st.rhs++;
      }
      if (LRN == 2 && lr.have_prop) {
        // learned first step of the interval instead of HINIT
        h = posneg * fmin(fabs(h), hmax);
        lr.have_prop = false;
        nfcn += 1;
      } else {
        h = hinit_df<4>(rhs, rt, y, k1, scale, posneg, 1.0 / 5.0, hmax, P.rtol, P.atol);
        st.rhs++;
        nfcn += 2;
      }
      ctl.reset(beta);
      errold = 1e-4;
      reject = false;
      last = false;
      in_interval = true;
    }

    bool ended = false;
    int fail = 0;
    if (nst > P.nsteps) { ended = true; fail = RAPT_ST_MAXSTEPS; }
    else if (0.1 * fabs(h) <= fabs(rt) * kUround) { ended = true; fail = RAPT_ST_HMIN; }
    else {
      if ((rt + 1.01 * h - xend) * posneg > 0.0) { lr.before_clip(h); h = xend - rt; last = true; }
      ++nst;
      --budget;
      DF y1[4], k7[4];
      double err;
      dopri5_attempt_df_rolled<4>(rhs, rt, y, k1, h, scale, P.rtol, P.atol, y1, k7, err);
      nfcn += 6;
      st.rhs += 6;
      lr.on_attempt(P, h, err, last);
      double hnew = h * (double)ctl.accept_factor(err, expo1, safe, facc1, facc2);
      if (left_grid<M>(err)) {
        ended = true;
        fail = RAPT_ST_OUT_OF_GRID;
      } else if (err <= 1.0) {
        const double errprev = errold;
        const bool rej_before = reject;
        const double hstep = h;
        ctl.accepted(err, beta);
        errold = fmax(err, 1.0e-4);
        ++nacc; ++nacc_int; st.acc++;
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
                     y[0].hi, y[1].hi, y[2].hi,
                     y[3].hi, vs, interval_progress(xend, rt, hmax));
      } else {
        hnew = h * (double)ctl.reject_factor(safe, facc1);
        reject = true;
        if (nacc_int >= 1) { ++nrej; st.rej++; }
        last = false;
        h = hnew;
      }
    }

    if (ended) {
      in_interval = false;
      double s[6];
      state_si(s);
      if (fail) { seg_ok = false; status = fail; }
      if (!all_finite<4>(s)) { seg_ok = false; status = RAPT_ST_NONFINITE; }
      // a Grid step outside the grid (ValueError) or an RKF45 step below hmin
      // (RuntimeError): the reference raises inside the interval, adding no row
      const bool row = !(M == RAPT_GRID && status == RAPT_ST_OUT_OF_GRID) && status != RAPT_ST_RKF_HMIN;
      if (row) {
        t_row = rt;
        tcur = rt;
        put_row(E, P, idx, nrows, rt, s, 4, RAPT_MODE_GC);
      }
      const bool row_chk = row && (flags & RAPT_FLAG_CHECK_ADIABATICITY) && status != RAPT_ST_NONFINITE;
      const bool nonadi = row_chk && !gc_isadiabatic<M>(P, t_row, s, mu, mass, charge);
      if (row_chk) lr.on_row(P, nonadi);
      if (nonadi) {
        if (P.kind == RAPT_KIND_ADAPTIVE) {
          double s6[6];
          gc_to_particle<M>(P.f, t_row, s, mu, mass, charge, s6);
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
          E.t_int[idx] = rt; E.t_row[idx] = t_row; E.tcur[idx] = tcur;
          E.naccept[idx] = nacc; E.nreject[idx] = nrej; E.nfcn[idx] = nfcn;
          E.status[idx] = status; E.flags[idx] = flags; E.nrows[idx] = nrows; E.nswitch[idx] = nswitch;
          E.nseg[idx] = nseg; E.seg_active[idx] = 0;
          idx = -1;
          continue;
        }
        flags |= RAPT_FLAG_RAISED | RAPT_FLAG_DONE;
        st.done++;
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

// Right-hand sides of the FP32 form at given states, for checks (rapt_rhs_eval
// with an FP32 form configured): the float-float equations of k_particle32 and
// k_gc32 (the Tao-Chan-Brizard equations; the FP32 forms run no other)
// evaluated at the FP64 states and returned in SI units, state[n][8] = (t,
// y0..y5, gm | mu), out[n][6] as k_rhs_eval.
template <int M>
__global__ void k_rhs_eval32(KParams P, int mode, int64_t n, const double* state, const double* mass,
                             const double* charge, double* out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double* s = state + 8 * i;
  const double m = mass[i], q = charge[i], mc = m * kC;
  double o[6] = {0, 0, 0, 0, 0, 0};
  if (mode == 0) {
    const DF Y[6] = {dfd(s[1]), dfd(s[2]), dfd(s[3]), dfd(s[4] / mc), dfd(s[5] / mc), dfd(s[6] / mc)};
    const ParticleRHSdf<M> rhs{P.f, dfd(q / mc), dfd(q / m), dfd(m / s[7]), P.enforce_eq != 0};
    DF d[6];
    rhs(s[0], Y, d);
    for (int k = 0; k < 6; ++k) o[k] = df_to_double(d[k]) * (k < 3 ? 1.0 : mc);
  } else {
    const double mu = s[7];
    const DF Y[4] = {dfd(s[1]), dfd(s[2]), dfd(s[3]), dfd(s[4] / mc)};
    const GcRHSdf<M> rhs{P.f, dfd(2.0 * mu / (m * kC * kC)), dfd(mc / q), dfd(mu / q), dfd(q / mc),
                         P.enforce_eq != 0};
    DF d[4];
    rhs(s[0], Y, d);
    for (int k = 0; k < 4; ++k) o[k] = df_to_double(d[k]) * (k < 3 ? 1.0 : mc);
  }
  for (int k = 0; k < 6; ++k) out[6 * i + k] = o[k];
}

}  // namespace rapt
