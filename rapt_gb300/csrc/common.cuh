// common.cuh -- shared device-side types and helpers of the GB300 ensemble tracer.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/rapt_gpu.h"

namespace rapt {

// Physical constants, rapt/__init__.py:5-10.
constexpr double kC = 299792458.0;
constexpr double kB0 = 3.07e-5;
constexpr double kRe = 6378137.0;
constexpr double kPi = 3.141592653589793;
constexpr double kRe3 = kRe * kRe * kRe;

constexpr unsigned kFull = 0xffffffffu;

// Field model parameters as seen by the kernels (passed by value: they live in
// the kernel-parameter constant bank, uniform across the grid).
struct FieldP {
  int model;
  int is_static;      // _Field.static
  double p[8];        // constructor parameters
  double gradstep;    // _Field.gradientstepsize
  double timestep;    // _Field.timederivstepsize
  double inv2d;       // 1 / (2 gradstep)
  double c0, c1, c2;  // model constants precomputed on the host
  float dh[4], dl[4]; // float-float model constants (hi, lo) for the FP32 form
  // RAPT_GRID: axes and [nt][nx][ny][nz][3] snapshots resident on the device
  const double *gt, *gx, *gy, *gz;
  const double *gB, *gE;  // gE null: zero electric field
  double ginv[4];         // (n - 1) / (g[n-1] - g[0]) per axis (t, x, y, z): the cell guess
  int nt, nx, ny, nz;
};

// rapt.params plus device options, resolved on the host.
struct KParams {
  FieldP f;
  double rtol, atol, cycres, gctimestep, epss, epst;
  double rkf_tol, rkf_hmin;
  int enforce_eq, tableau, gc_eom, nsteps, kind, form;
  long long budget;        // RK step attempts per thread per launch
  int max_rows, max_sw;    // per-tracer output capacity
  int max_segments;        // Adaptive: cap on advance() calls per tracer
  // step-size MLP (learned forms) and training-sample collection
  const uint32_t* mlp_w;   // packed BF16 weights
  const float* mlp_p;      // FP32 biases and normalisation
  float learn_scale;       // multiplier on the learned step proposal
  float* samp;             // [samp_cap][18] collected samples
  unsigned long long* samp_count;
  long long samp_cap;
  unsigned long long samp_mask;  // an accepted step is sampled when its hash & mask == 0
  int collect;             // learned kernels: also record samples (on-policy data)
  int learn_every;         // run the MLP on every k-th accepted step, reuse its correction between
  // bounce-period cadence (gctimestep == 0): per-thread field-line scratch
  double bounceres, flres; // params["bounceresolution"], params["fieldlineresolution"]
  double* fl_scratch;      // fl_stride doubles per thread of the launch
  long long fl_stride;
  int fl_cap;              // trace points per direction
};

// Device SoA ensemble (all arrays length n unless noted).
struct DevEnsemble {
  int64_t n;
  int8_t* mode;
  int32_t* status;
  int32_t* flags;
  double* t_int;     // integrator time r.t
  double* t_row;     // time of the last trajectory row
  double* tcur;
  double* s[6];
  double* mu;
  double* v;
  double* mass;
  double* charge;
  int64_t* naccept;
  int64_t* nreject;
  int64_t* nfcn;
  int32_t* nswitch;
  // per-call advance bookkeeping
  double* delta;       // the delta of this call (Particle/GC advance, or Adaptive delta)
  double* seg_stop;    // t0 + delta of the current tracer.advance() call
  double* seg_dt;      // output cadence of the current call
  double* seg_gm;      // gamma*m frozen at the start of a Particle.advance call
  // dense-output guiding-centre integration carried between steps and launches:
  // step size (0: not started), facold, steps since the last row
  double* carry_h;
  double* carry_fac;
  double* carry_nst;
  int8_t* seg_active;  // 1 while a tracer.advance() call is in progress
  int32_t* nseg;       // advance() calls made by Adaptive in this call
  // outputs
  double* rows;        // [n][max_rows][7]
  int8_t* row_mode;    // [n][max_rows]
  int32_t* nrows;
  double* sw_time;     // [n][max_sw]
  int8_t* sw_mode;     // [n][max_sw]
};

// Scratch words used by the persistent kernels (one block of device memory).
struct Scratch {
  unsigned long long queue[2];   // work-queue heads (particle kernel, GC kernel)
  unsigned long long pending;    // tracers left unfinished by the last launch pair
  unsigned long long accepted, rejected, rhs, switches, done, failed;
};

__device__ __forceinline__ double dot3(const double* a, const double* b) {
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}
__device__ __forceinline__ void cross3(const double* a, const double* b, double* o) {
  o[0] = a[1] * b[2] - a[2] * b[1];
  o[1] = a[2] * b[0] - a[0] * b[2];
  o[2] = a[0] * b[1] - a[1] * b[0];
}

}  // namespace rapt
