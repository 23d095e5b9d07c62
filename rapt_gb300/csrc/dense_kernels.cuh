// dense_kernels.cuh -- guiding-centre advance with dense output (no reference
// counterpart; an option of rapt_config).
//
// GuidingCenter.advance (GuidingCenter.py:397-458) restarts SciPy's dopri5 at
// every output time: each interval begins with an automatic initial step
// (2 right-hand sides) and its last step is cut to land on the output time.
// Here one DOPRI5 integration runs through the whole advance() call, with the
// step size bounded by kDenseSpan output intervals (the reference's hmax is one
// interval), and each output row is the order-4 continuous extension of the
// step that covers its time: with a fine cadence the step size is set by the
// tolerance alone. Rows are at the reference's times (t0 + dt,
// + dt, ... until the segment end is reached), the adiabaticity check runs on
// each row, and the segment ends in the last row's state. The integrator state
// (step size, facold, steps since the last row) is carried between steps in
// the ensemble, so a launch can end between any two steps (step budget, full
// row buffer) and the result does not depend on where it ended.
#pragma once
#include "tracer_kernels.cuh"

namespace rapt {

// hmax of the dense-output integration in output intervals; a step then covers
// at most kDenseSpan + 1 row times, which the row buffer must hold
constexpr int kDenseSpan = 16;

template <int M>
__global__ void __launch_bounds__(128) k_gc_dense(DevEnsemble E, KParams P, Scratch* S) {
  int64_t idx = -1;
  bool exhausted = false;
  long long budget = P.budget;
  LaneStats st;

  double y[4] = {0, 0, 0, 0}, k1[4] = {0, 0, 0, 0};
  double rt = 0, t_row = 0, tcur = 0, dt = 0, stop = 0, mass = 0, charge = 0, delta = 0, mu = 0, vs = 0;
  double qinv = 0, minv = 0, kmu = 0, inv_mc = 0, igv = 0, gmv = 0, gmv2 = 0;
  long long nacc = 0, nrej = 0, nfcn = 0;
  int status = 0, flags = 0, nrows = 0, nsw = 0, nseg = 0, nswitch = 0;
  bool seg_ok = true, k1_valid = false;
  double h = 0, facold = 1e-4;  // h == 0: the integration of this segment has not started
  int nst = 0;                  // steps since the last row (SciPy's nsteps per interval)
  bool reject = false;

  constexpr double beta = 0.04, safe = 0.9;
  constexpr double expo1 = 0.2 - beta * 0.75, facc1 = 1.0 / 0.2, facc2 = 1.0 / 10.0;

  auto begin_segment = [&](double seg_delta) {
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
    h = 0.0;
    facold = 1e-4;
    nst = 0;
    reject = false;
    k1_valid = false;
  };

  auto load = [&](int64_t k) {
#pragma unroll
    for (int i = 0; i < 4; ++i) y[i] = E.s[i][k];
    rt = E.t_int[k]; t_row = E.t_row[k]; tcur = E.tcur[k];
    mass = E.mass[k]; charge = E.charge[k]; delta = E.delta[k];
    mu = E.mu[k]; vs = E.v[k];
    {
      const double gv = 1.0 / sqrt(1.0 - (vs / kC) * (vs / kC));
      qinv = 1.0 / charge; minv = 1.0 / mass; kmu = 2.0 * mu / (mass * kC * kC); inv_mc = 1.0 / (mass * kC);
      igv = 1.0 / gv; gmv = gv * mass; gmv2 = gv * mass * vs * vs;
    }
    nacc = E.naccept[k]; nrej = E.nreject[k]; nfcn = E.nfcn[k];
    status = E.status[k]; flags = E.flags[k]; nrows = E.nrows[k]; nswitch = E.nswitch[k];
    nseg = E.nseg[k];
    nsw = nswitch;
    seg_ok = true;
    k1_valid = false;
    if (E.seg_active[k]) {
      stop = E.seg_stop[k]; dt = E.seg_dt[k];
      h = E.carry_h[k]; facold = E.carry_fac[k]; nst = (int)E.carry_nst[k];
      reject = (flags & RAPT_FLAG_REJECTED) != 0;
    } else {
      begin_segment((P.kind == RAPT_KIND_ADAPTIVE && nseg > 0) ? delta - tcur : delta);
    }
  };

  auto store = [&](int64_t k, bool active) {
#pragma unroll
    for (int i = 0; i < 4; ++i) E.s[i][k] = y[i];
    E.s[4][k] = 0.0;
    E.s[5][k] = 0.0;
    E.t_int[k] = rt; E.t_row[k] = t_row; E.tcur[k] = tcur;
    E.naccept[k] = nacc; E.nreject[k] = nrej; E.nfcn[k] = nfcn;
    flags = reject ? (flags | RAPT_FLAG_REJECTED) : (flags & ~RAPT_FLAG_REJECTED);
    E.status[k] = status; E.flags[k] = flags; E.nrows[k] = nrows; E.nswitch[k] = nswitch; E.nseg[k] = nseg;
    E.seg_active[k] = active ? 1 : 0;
    E.seg_stop[k] = stop; E.seg_dt[k] = dt;
    E.carry_h[k] = active ? h : 0.0; E.carry_fac[k] = facold; E.carry_nst[k] = (double)nst;
  };

  for (;;) {
    warp_refill(&S->queue[1], E, RAPT_MODE_GC, idx, exhausted, load);
    if (__all_sync(kFull, idx < 0)) break;
    if (idx < 0) continue;

    const GcRHS<M> rhs{P.f, charge, qinv, mu, minv, kmu, inv_mc, igv, gmv, gmv2, P.gc_eom, P.enforce_eq != 0};

    // ---- between steps: segment end, launch budget, row capacity
    if (!(seg_ok && t_row < stop)) {
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
    if (nrows + kDenseSpan + 1 > P.max_rows) {  // room for the rows one step can cover
      status = RAPT_ST_ROWS_FULL;
      store(idx, true);
      idx = -1;
      continue;
    }
    if (!k1_valid) {  // the FSAL slope at (rt, y): recomputed after a load, bit for bit
      rhs(rt, y, k1);
      k1_valid = true;
      st.rhs++;
      if (h == 0.0) nfcn += 1;  // counted once per integration, not per launch
    }
    if (h == 0.0) {  // start of the segment's integration: HINIT once
      h = hinit<4>(rhs, rt, y, k1, 1.0, 1.0 / 5.0, kDenseSpan * dt, P.rtol, P.atol);
      st.rhs++;
      nfcn += 1;
      facold = 1e-4;
      reject = false;
      nst = 0;
    }

    // ---- one DOPRI5 attempt
    int fail = 0;
    bool row_end = false;  // the segment ended (last row, failure or a raised check)
    if (nst > P.nsteps) fail = RAPT_ST_MAXSTEPS;
    else if (0.1 * fabs(h) <= fabs(rt) * kUround) fail = RAPT_ST_HMIN;
    else {
      ++nst;
      --budget;
      double y1[4], k7[4], dd[4], err;
      dopri5_attempt_rolled<4, GcRHS<M>, true>(rhs, rt, y, k1, h, P.rtol, P.atol, y1, k7, err, dd);
      nfcn += 6;
      st.rhs += 6;
      const double fac11 = pow_fp64(err, expo1);
      double fac = fac11 / pow_fp64(facold, beta);
      fac = fmax(facc2, fmin(facc1, fac / safe));
      double hnew = h / fac;
      if (left_grid<M>(err)) {
        fail = RAPT_ST_OUT_OF_GRID;
      } else if (err <= 1.0) {
        facold = fmax(err, 1.0e-4);
        ++nacc; st.acc++;
        const double told = rt, hs = h;
        rt = rt + h;
        if (fabs(hnew) > kDenseSpan * dt) hnew = kDenseSpan * dt;
        if (reject) hnew = fmin(fabs(hnew), fabs(h));
        reject = false;
        h = hnew;
        // rows whose times this step covers
        for (int r = 0; r <= kDenseSpan && !row_end; ++r) {
          const double tn = t_row + dt;
          if (!(tn <= rt)) break;
          double yr[4];
          dopri5_dense<4>(y, y1, k1, k7, dd, hs, (tn - told) / hs, yr);
          t_row = tn;
          tcur = tn;
          nst = 0;
          put_row(E, P, idx, nrows, tn, yr, 4, RAPT_MODE_GC);
          bool nonadi = false;
          if ((flags & RAPT_FLAG_CHECK_ADIABATICITY) && all_finite<4>(yr))
            nonadi = !gc_isadiabatic<M>(P, t_row, yr, mu, mass, charge);
          if (nonadi || !(t_row < stop)) {
            // the segment ends in this row's state
#pragma unroll
            for (int i = 0; i < 4; ++i) y[i] = yr[i];
            rt = t_row;
            k1_valid = false;
            h = 0.0;
            row_end = true;
            if (nonadi) {
              if (P.kind == RAPT_KIND_ADAPTIVE) {
                double s6[6];
                gc_to_particle<M>(P.f, t_row, y, mu, mass, charge, s6);
#pragma unroll
                for (int i = 0; i < 6; ++i) E.s[i][idx] = s6[i];
                E.mode[idx] = RAPT_MODE_PARTICLE;
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
                E.status[idx] = status; E.flags[idx] = flags & ~RAPT_FLAG_REJECTED; E.nrows[idx] = nrows;
                E.nswitch[idx] = nswitch; E.nseg[idx] = nseg; E.seg_active[idx] = 0; E.carry_h[idx] = 0.0;
                idx = -1;
              } else {
                flags |= RAPT_FLAG_RAISED | RAPT_FLAG_DONE;
                st.done++;
                store(idx, false);
                idx = -1;
              }
            }
          }
        }
        if (idx < 0) continue;
        if (!row_end) {
#pragma unroll
          for (int i = 0; i < 4; ++i) { k1[i] = k7[i]; y[i] = y1[i]; }
        }
      } else {
        hnew = h / fmin(facc1, fac11 / safe);
        reject = true;
        ++nrej;
        st.rej++;
        h = hnew;
      }
    }
    if (fail) {
      // the integration stops; as in the restarting kernel a failed interval
      // still leaves a row at the integrator's time (none outside a grid)
      seg_ok = false;
      status = fail;
      if (!(M == RAPT_GRID && fail == RAPT_ST_OUT_OF_GRID)) {
        t_row = rt;
        tcur = rt;
        put_row(E, P, idx, nrows, rt, y, 4, RAPT_MODE_GC);
      }
      h = 0.0;
    }
    if (seg_ok && !all_finite<4>(y)) { seg_ok = false; status = RAPT_ST_NONFINITE; h = 0.0; }
  }
  st.flush(S);
}

}  // namespace rapt
