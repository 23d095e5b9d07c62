/*
 * rapt_gpu.h -- C ABI of librapt_gpu.so, the GB300 ensemble tracer.
 *
 * RAPT (mkozturk/rapt) has no FFI: its boundary is the Python class API
 * (Particle, GuidingCenter, Adaptive, rapt.params, the field objects). This
 * header is the layer that a Python facade with the same classes binds through
 * ctypes; each entry point names the reference interface it stands in for.
 *
 * Conventions
 *  - Every call returns an int: RAPT_OK (0) or an RAPT_ERR_* code. The text of
 *    the last error of a context is returned by rapt_last_error().
 *  - Host buffers are owned by the caller (C-contiguous, float64 unless stated).
 *    The context owns all device memory.
 *  - One context per host thread; calls on one context are not thread-safe.
 *  - Kernels never trap: per-tracer failures come back in the status array.
 */
#ifndef RAPT_GPU_H
#define RAPT_GPU_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RAPT_GPU_ABI_VERSION 1

/* Return codes. */
enum {
  RAPT_OK = 0,
  RAPT_ERR_INVALID = 1,     /* bad argument */
  RAPT_ERR_CUDA = 2,        /* CUDA runtime error */
  RAPT_ERR_NOMEM = 3,       /* device allocation failed */
  RAPT_ERR_UNSUPPORTED = 4, /* e.g. field model without a device implementation */
  RAPT_ERR_STATE = 5        /* call out of order (no ensemble, no field, ...) */
};

/* Field models with a device implementation (rapt/fields.py). */
enum {
  RAPT_EARTH_DIPOLE = 0,       /* EarthDipole(B0)                 fields.py:282-317 */
  RAPT_DOUBLE_DIPOLE = 1,      /* DoubleDipole(B0, distance, k)   fields.py:319-362 */
  RAPT_UNIFORM_BZ = 2,         /* UniformBz(Bz)                   fields.py:364-390 */
  RAPT_UNIFORM_CROSSED_EB = 3, /* UniformCrossedEB(Ey, Bz)        fields.py:392-427 */
  RAPT_VAR_EARTH_DIPOLE = 4,   /* VarEarthDipole(amp, period)     fields.py:429-470 */
  RAPT_PARABOLIC = 5,          /* Parabolic(B0, Bn, d)            fields.py:472-511 */
  RAPT_HARRIS = 6,             /* Harris sheet (B0, L, Bn, Ey): no reference counterpart */
  RAPT_COMPRESSED_DIPOLE = 7,  /* breathing dipole + induced E (B0, amp, period): no counterpart */
  RAPT_GRID = 8,               /* Grid(filelist): gridded snapshots   fields.py:513-814 (rapt_grid_set) */
  RAPT_N_MODELS = 9
};

/* Tracer modes and run kinds. */
enum { RAPT_MODE_PARTICLE = 0, RAPT_MODE_GC = 1 };
enum { RAPT_KIND_PARTICLE = 0, RAPT_KIND_GC = 1, RAPT_KIND_ADAPTIVE = 2 };

/* Arithmetic forms. */
enum {
  RAPT_FORM_PLAIN = 0,        /* FP64 throughout, reference controller semantics */
  RAPT_FORM_FP32 = 1,         /* FP32 stages, compensated accumulation, FP64 control; guiding
                                 centres: FP32 stencil differences, position tolerance floored
                                 at 3e-9 of a step's displacement */
  RAPT_FORM_LEARNED = 2,      /* FP64 with MLP step proposals */
  RAPT_FORM_LEARNED_FP32 = 3  /* FP32 stages with MLP step proposals */
};

/* Per-tracer status words. */
enum {
  RAPT_ST_OK = 0,
  RAPT_ST_MAXSTEPS = 2,       /* SciPy idid -2: more than nsteps steps in one output interval */
  RAPT_ST_HMIN = 3,           /* SciPy idid -3: step size too small */
  RAPT_ST_NONFINITE = 4,      /* NaN/Inf in the state */
  RAPT_ST_GC_NOCONV = 5,      /* utils.guidingcenter did not converge (reference returns None) */
  RAPT_ST_ROWS_FULL = 6,      /* output row buffer full: drain rows and call again to resume */
  RAPT_ST_BAD_INPUT = 7,      /* e.g. a GC cadence that is not > 0 */
  RAPT_ST_RKF_HMIN = 8,       /* rkf.py RuntimeError at hmin */
  RAPT_ST_ADAPTIVE_LIMIT = 9, /* adaptive segment cap reached */
  RAPT_ST_FIELDLINE = 10,     /* bounce period: field-line trace longer than the device buffer, or no finite result */
  RAPT_ST_OUT_OF_GRID = 11    /* RAPT_GRID: a step evaluated the field outside the grid (the reference's
                                 RegularGridInterpolator raises ValueError); the state is the last accepted one */
};

/* Per-tracer flag bits (rapt_host_state.flags). */
enum {
  RAPT_FLAG_CHECK_ADIABATICITY = 1, /* tracer.check_adiabaticity */
  RAPT_FLAG_RAISED = 2,             /* out: Adiabatic / NonAdiabatic was raised */
  RAPT_FLAG_DONE = 4,               /* internal: advance finished for this call */
  RAPT_FLAG_REJECTED = 8            /* internal: dense output, the last attempt was rejected */
};

/* Mirrors rapt.params (rapt/__init__.py:21-34) plus device options. */
typedef struct {
  double rtol, atol;             /* params["solvertolerances"] */
  double cyclotronresolution;    /* params["cyclotronresolution"] */
  double gctimestep;             /* params["GCtimestep"]; 0: bounce-period cadence */
  double epss, epst;             /* params["epss"], params["epst"] */
  int32_t enforce_equatorial;    /* params["enforce equatorial"] */
  int32_t tableau;               /* 0: DOP853 particle / DOPRI5 GC (as the reference); 1: RKF45 (rkf.py) */
  int32_t gc_eom;                /* 0 TaoChanBrizard, 1 BrizardChan, 2 NorthropTeller */
  int32_t nsteps;                /* SciPy ode nsteps per output interval (500) */
  double rkf_tol, rkf_hmin;      /* RKF45 tableau: rkf.py tol and hmin */
  int32_t form;                  /* RAPT_FORM_* */
  int32_t threads_per_block;     /* 0: default */
  int64_t max_steps_per_launch;  /* per-thread RK-step budget of one launch (0: default) */
  int32_t blocks_per_sm;         /* 0: default */
  int32_t use_graph;             /* 1: capture a chunk of launch rounds (queue resets, particle and
                                    guiding-centre kernels, pending read-back) once per call as a CUDA
                                    graph and replay it until no tracer is pending */
  int32_t collect;               /* 1: record step-size training samples (GC, DOPRI5; any form) */
  double learned_scale;          /* learned forms: multiplier on each MLP step proposal (0: 1) */
  int32_t learned_every;         /* learned forms: a warp runs the MLP on every k-th iteration of its step
                                    loop, for the lanes that accepted a step since its last call; each lane
                                    scales the controller's steps by its latest correction (0 or 1: every
                                    iteration) */
  int32_t per_tracer_launches;   /* 1: one launch sequence per tracer (the unbatched pattern, for
                                    comparison); 0: one persistent grid for the whole ensemble */
  double bounceresolution;       /* params["bounceresolution"]: with gctimestep == 0 the GC cadence is
                                    bounceperiod() / bounceresolution (GuidingCenter.py:443-446) */
  double fieldlineresolution;    /* params["fieldlineresolution"] (fieldline.py:31-35) */
  int32_t dense_output;          /* 1: guiding centres integrate through each advance() call without restarting
                                    at the output times (steps up to 16 output intervals) and output rows from
                                    DOPRI5's order-4 continuous extension; plain form, DOPRI5 only, max_rows >= 18.
                                    No reference counterpart (the reference restarts SciPy's dopri5 per row) */
} rapt_config;

/* Host-side SoA view of an ensemble. Any pointer may be NULL on download to
 * skip that array. s[0..5]: particle x,y,z,px,py,pz; GC x,y,z,ppar,0,0. */
typedef struct {
  int64_t n;
  int8_t* mode;        /* RAPT_MODE_* */
  int32_t* status;     /* RAPT_ST_* */
  int32_t* flags;      /* RAPT_FLAG_* */
  double* t_int;       /* integrator time r.t */
  double* t_row;       /* time of the last trajectory row (trajectory[-1,0]) */
  double* tcur;        /* tracer.tcur */
  double* s[6];
  double* mu;          /* GC magnetic moment */
  double* v;           /* GC speed attribute (GuidingCenter.v) */
  double* mass;
  double* charge;
  int64_t* naccept;    /* accepted RK steps (SciPy NACCPT summed) */
  int64_t* nreject;    /* rejected RK steps (NREJCT) */
  int64_t* nfcn;       /* RHS evaluations as the reference counts them (NFCN) */
  int32_t* nswitch;    /* Adaptive switches */
} rapt_host_state;

typedef struct {
  int64_t accepted, rejected, rhs_evals, switches;
  int64_t done, failed, launches, kernel_launches;
  double kernel_ms;    /* device time of the advance, CUDA events on the context stream */
} rapt_stats;

/* --- context ------------------------------------------------------------ */
int rapt_abi_version(void);
/* Create a context on a CUDA device (its own stream). */
int rapt_ctx_create(int device, void** ctx_out);
void rapt_ctx_destroy(void* ctx);
const char* rapt_last_error(const void* ctx);

/* --- configuration ------------------------------------------------------- */
/* Stand-in for passing a field object (rapt/fields.py) to a tracer. params
 * override the model's constructor defaults in order. */
int rapt_field_set(void* ctx, int model, const double* params, int nparams);
/* Stand-in for assigning field.gradientstepsize / field.timederivstepsize
 * (fields.py:38-41); call after rapt_field_set. */
int rapt_field_set_steps(void* ctx, double gradientstepsize, double timederivstepsize);
/* Stand-in for assigning field.static (fields.py:41). The analytic models'
 * static-ness follows from their equations and ignores it; RAPT_GRID honours it
 * (Grid leaves static = True, fields.py:41 via :577, even for time-dependent data). */
int rapt_field_set_static(void* ctx, int is_static);
/* Grid (fields.py:513-814): field snapshots at times t[nt] (strictly ascending)
 * on the rectilinear axes x[nx], y[ny], z[nz] (strictly ascending, >= 2 points,
 * spacing free). B and E are [nt][nx][ny][nz][3] float64 (component fastest);
 * E may be NULL (zero electric field). nt == 1 is the time-independent case
 * (3-D interpolation); nt >= 2 interpolates linearly in time between adjacent
 * snapshots. Every snapshot stays resident on the device: the reference's
 * three-snapshot sliding window (fields.py:695-705, :733-734) gives the same values on
 * the interval it covers. Interpolation is SciPy's RegularGridInterpolator,
 * method "linear" (corners in itertools.product order, FP64, no FMA), so values
 * agree bit for bit. Selects RAPT_GRID as the field, gradientstepsize 1e-3 Re
 * (fields.py:578), timederivstepsize 1e-3, static = 1. A later
 * rapt_field_set(ctx, RAPT_GRID, NULL, 0) re-selects the resident grid. */
int rapt_grid_set(void* ctx, int32_t nt, const double* t, int32_t nx, const double* x, int32_t ny,
                  const double* y, int32_t nz, const double* z, const double* B, const double* E);
/* Stand-in for rapt.params (rapt/__init__.py:21-34). */
void rapt_config_default(rapt_config* cfg);
int rapt_config_set(void* ctx, const rapt_config* cfg);

/* --- ensemble ------------------------------------------------------------ */
/* Allocate device SoA storage for n tracers, max_rows output rows and
 * max_switch switch-log entries per tracer. */
int rapt_ensemble_alloc(void* ctx, int64_t n, int32_t max_rows, int32_t max_switch);
/* Tracer construction state (Particle.__init__ Particle.py:59-109,
 * GuidingCenter.__init__ GuidingCenter.py:63-133) copied host -> device. */
int rapt_ensemble_upload(void* ctx, const rapt_host_state* h);
int rapt_ensemble_download(void* ctx, rapt_host_state* h);
/* Trajectory rows appended since the last reset (tracer.trajectory[1:]):
 * rows[n][max_rows][7] = (t, s0..s5), row_mode[n][max_rows], nrows[n];
 * switch log sw_time[n][max_switch], sw_mode[n][max_switch]. Any pointer may be
 * NULL. reset != 0 empties the device row buffers afterwards. */
int rapt_rows_download(void* ctx, double* rows, int8_t* row_mode, int32_t* nrows,
                       double* sw_time, int8_t* sw_mode, int reset);

/* --- advance ------------------------------------------------------------- */
/* Particle.advance(delta)       Particle.py:230-309      kind RAPT_KIND_PARTICLE
 * GuidingCenter.advance(delta)  GuidingCenter.py:397-458 kind RAPT_KIND_GC
 * Adaptive.advance(delta)       Adaptive.py:187-222      kind RAPT_KIND_ADAPTIVE
 * for every tracer of the ensemble at once. delta: per-tracer array (length n)
 * or NULL to use delta_all. Returns when the device work has completed. */
int rapt_advance(void* ctx, int kind, const double* delta, double delta_all, rapt_stats* stats);
/* Continue the last rapt_advance after tracers stopped with RAPT_ST_ROWS_FULL
 * (drain their rows with rapt_rows_download(..., reset=1) first). */
int rapt_advance_resume(void* ctx, int kind, rapt_stats* stats);

/* Adaptive.__init__ mode pick (Adaptive.py:70-104) on device: tracers given as
 * particles are converted to guiding centres where Particle.isadiabatic() holds. */
int rapt_adaptive_init(void* ctx);

/* Single-point field evaluation for checks (fields.py _Field methods):
 * what = 0 B, 1 E, 2 gradB, 3 curlb, 4 magB, 5 unitb, 6 lengthscale,
 * 7 dbdt, 8 jacobianB (9 values), 9 dBdt, 10 timescale.
 * tpos[n][4] host, out[n][9] host. */
int rapt_field_eval(void* ctx, int what, int64_t n, const double* tpos, double* out);

/* Right-hand sides at given states for checks (Particle.py:284-298,
 * GuidingCenter.py:329-395). state[n][8] = (t, y0..y5, gm|mu), per-tracer
 * mass/charge/v; out[n][6]. With an FP32 form configured, the FP32 form's
 * float-float equations (and its FP32 stencil differences) in SI units. */
int rapt_rhs_eval(void* ctx, int mode, int64_t n, const double* state, const double* mass,
                  const double* charge, const double* v, double* out);

/* GuidingCenter.bounceperiod (GuidingCenter.py:593-606; field-line trace and
 * flutils.halfbouncepath, flutils.py:254-316) for n states, one GPU thread each:
 * state[n][7] = (t, x, y, z, ppar, mu, mass) host, out[n] host (s); NaN where
 * the trace exceeds the device buffer (1024 points per direction). Uses the
 * config's fieldlineresolution. */
int rapt_gc_bounce_period(void* ctx, int64_t n, const double* state, double* out);

/* --- BounceCenter (rapt/BounceCenter.py) and the second invariant ----------
 * BounceCenter.advance(delta) (BounceCenter.py:214-252) for n bounce centres at
 * once, one GPU thread each (field-line traces in a per-thread scratch slot: 8 KB in passes of
 * 16,384 tracers; a tracer that meets a non-finite value is rerun with 64 KB slots): the
 * drift gamma m v^2 / (q S_b |B|^2) (grad I x B) with S_b = halfbouncepath
 * and grad I = flutils.gradI (five field-line traces per right-hand side),
 * rows every bctimestep x the bounce period at the start, SciPy-dopri5
 * restarts per row (config rtol, atol, nsteps; fieldlineresolution).
 *   state[n][5] in/out = (t, x, y, z, tcur): t, x, y, z = trajectory[-1]
 *   cst[n][4] = (v, mu, mass, charge)
 *   rows[n][max_rows][4] out = (t, x, y, z): the reference's rows, each stamped
 *     with the time its interval began (np.arange(tcur, tcur + delta, dt));
 *     nrows[n] out counts all rows (rows past max_rows are not stored)
 *   status[n] out: RAPT_ST_*; counters[n][4] (NFCN, NSTEP, NACCPT, NREJCT) or NULL
 * The field must be static (BounceCenter.py:95-97). The reference's
 * flutils.eye raises NameError below 70 degrees equatorial pitch angle (its
 * Simpson branch calls an undefined name); the device uses the spline branch
 * at every pitch angle. */
int rapt_bc_advance(void* ctx, int64_t n, double* state, const double* cst, double delta, double bctimestep,
                    double eyegradientstep, double* rows, int32_t max_rows, int32_t* nrows, int32_t* status,
                    int64_t* counters);
/* Field-line quantities at tpos[n][4] with mirror fields Bm[n]: what 0
 * flutils.eye (out[n][3], first value), 1 flutils.gradI, 2 the bounce-averaged
 * drift velocity (needs cst[n][4] as above), 3 flutils.halfbouncepath (first
 * value; flutils.py:254-316). NaN where a trace overflows or the reference raises. */
int rapt_bc_eval(void* ctx, int what, int64_t n, const double* tpos, const double* Bm, double eyegradientstep,
                 const double* cst, double* out);

/* --- allocation-free guiding-centre advance ------------------------------- */
/* No counterpart in the reference: RAPT has no device code and no notion of
 * memory ownership. This entry point is for callers that cannot call
 * cudaMalloc -- applications that must not allocate once running (real-time
 * loops), libraries that own all device memory through their own pool, and code
 * that must not trigger the implicit device synchronisation an allocation or
 * free can cause. It advances up to RAPT_NOALLOC_MAX_TRACERS guiding centres by
 * delta (the same advance as rapt_advance with RAPT_KIND_GC) whose state lives
 * in caller-owned device memory, creates no context, and allocates nothing:
 * the work-queue heads, counters and per-tracer bookkeeping live in one fixed
 * __device__ array of RAPT_NOALLOC_SCRATCH_BYTES that every GPU loading the
 * library holds until the process exits.
 *  - n > RAPT_NOALLOC_MAX_TRACERS returns RAPT_ERR_INVALID and touches nothing.
 *  - It runs the plain FP64 form with a fixed cadence only: cfg->form other than
 *    RAPT_FORM_PLAIN, cfg->gctimestep == 0 (the bounce-period cadence, which
 *    needs field-line scratch), cfg->dense_output or cfg->collect returns
 *    RAPT_ERR_UNSUPPORTED. rapt_config_default sets gctimestep = 0, so set it.
 *  - The first call on a device looks up that array's address (again after the
 *    device's context was reset); make it before any stream capture on that device.
 *  - All calls share the array: calls whose GPU work overlaps (other threads or
 *    streams on the same device) race and must be serialised by the caller.
 *  - The call is synchronous: it returns after the GPU work has completed.
 *    RAPT_ERR_STATE: tracers were still pending after 1,000,000 launch rounds.
 *  - nrows is reset to 0 by each call; rows[n][max_rows][7] receive the rows
 *    (t, x, y, z, ppar, 0, 0) of this call. */
#define RAPT_NOALLOC_MAX_TRACERS 65536
#define RAPT_NOALLOC_SCRATCH_BYTES 5242880
typedef struct {
  int64_t n;
  double* t;              /* in/out: time of the last trajectory row */
  double* x;              /* in/out */
  double* y;              /* in/out */
  double* z;              /* in/out */
  double* ppar;           /* in/out: parallel momentum */
  const double* mu;       /* in */
  const double* v;        /* in: GuidingCenter.v */
  const double* mass;     /* in */
  const double* charge;   /* in */
  int32_t* status;        /* out: RAPT_ST_* */
  int64_t* naccept;       /* in/out: accumulated */
  int64_t* nreject;       /* in/out */
  int64_t* nfcn;          /* in/out */
  double* rows;           /* out */
  int8_t* row_mode;       /* out */
  int32_t* nrows;         /* out */
  int32_t max_rows;       /* rows per tracer, >= 2 */
} rapt_gc_device_state;
int rapt_gc_advance_noalloc(int device, int model, const double* params, int nparams, const rapt_config* cfg,
                            const rapt_gc_device_state* state, double delta, void* stream, rapt_stats* stats);

/* --- step-size / switch MLP (learned forms) ---------------------------------
 * No counterpart in the reference, whose controllers are SciPy's. A 16 -> 64 ->
 * 64 -> 2 ReLU network (14 features used, BF16 weights, FP32 accumulation)
 * proposes a multiplicative correction of the plain controller's next step
 * (output 0) and the logit of an Adaptive switch (output 1). Parameter vector
 * (floats): W1T[64][16] b1[64] W2T[64][64] b2[64] W3T[8][64] b3[8] (trainable,
 * RAPT_MLP_NTRAIN) then feature mean[16], feature scale[16], target mean[8],
 * target scale[8]. A sample is 18 floats: 16 raw features, the step target
 * (log of the ideal next step over the controller's), the switch label (-1:
 * none). Inference and training run on the device (mma.sync BF16). */
#define RAPT_MLP_NPARAMS 5816
#define RAPT_MLP_NTRAIN 5768
#define RAPT_MLP_SAMPLE 18
int rapt_mlp_set_params(void* ctx, const float* params, int32_t n);
int rapt_mlp_get_params(void* ctx, float* params, int32_t n);
/* Batch inference: features[n][16] host -> out[n][2] host (target units). */
int rapt_mlp_forward(void* ctx, const float* features, int64_t n, float* out);
/* Gradient of the mean loss over samples[n][18] (host) w.r.t. the trainable
 * parameters -> grad[RAPT_MLP_NTRAIN] host; loss[2] = (step, switch) parts. */
int rapt_mlp_grad(void* ctx, const float* samples, int64_t n, float switch_weight, float* grad, double* loss);
/* Device sample buffer: capacity in samples; an accepted step is sampled when
 * a hash of (tracer, step count) & mask == 0. Resets the count. */
int rapt_mlp_samples_reserve(void* ctx, int64_t capacity, uint64_t mask);
int rapt_mlp_samples_count(void* ctx, int64_t* count);
int rapt_mlp_samples_download(void* ctx, float* out, int64_t first, int64_t n);
int rapt_mlp_samples_upload(void* ctx, const float* samples, int64_t n);
/* Put samples [first, first + n) into a canonical order (sorted by a 64-bit
 * hash of each sample's words). The kernels append samples in an order set by
 * device atomics; after this call the order, and so the minibatches that
 * rapt_mlp_train draws, depend only on which samples were collected. */
int rapt_mlp_samples_sort(void* ctx, int64_t first, int64_t n);
/* Adam (0.9, 0.999, 1e-8) on minibatches drawn from the device samples;
 * loss[2] = mean (step, switch) loss over the last tenth of the steps.
 * Deterministic: gradients are reduced in a fixed order (no floating-point
 * atomics), so equal samples, seed and parameters give equal results. */
int rapt_mlp_train(void* ctx, int64_t steps, int32_t batch, float lr, float switch_weight, uint64_t seed,
                   double* loss);

/* Page-lock (pin) a caller-owned host buffer so that uploads and downloads
 * through it run at full PCIe/NVLink-C2C speed; unregister before freeing. */
int rapt_host_register(void* p, uint64_t bytes);
int rapt_host_unregister(void* p);

/* Measured FP64 and FP32 FMA throughput of this device (TFLOP/s), from a
 * dependent-chain microkernel; used as roofline denominators. */
int rapt_measure_peaks(void* ctx, double* fp64_tflops, double* fp32_tflops);

#ifdef __cplusplus
}
#endif
#endif /* RAPT_GPU_H */
