/*
 * rapt_oracle.h -- CPU restatement of RAPT's tracer hot path.
 *
 * TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py as the checker. The product library
 * (rapt_gb300/librapt_gpu.so) never links or calls this code.
 *
 * Parity pin: this restatement is checked against the unmodified Python
 * reference (imported through oracle/shim.py) by tests/golden/make_golden.py,
 * which writes the golden fixtures under tests/golden/, and by
 * tests/test_oracle.py, which compares the two.
 */
#ifndef RAPT_ORACLE_H
#define RAPT_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Field model ids (shared with include/rapt_gpu.h). */
enum {
  ORC_EARTH_DIPOLE = 0,      /* rapt/fields.py:282-317 */
  ORC_DOUBLE_DIPOLE = 1,     /* rapt/fields.py:319-362 */
  ORC_UNIFORM_BZ = 2,        /* rapt/fields.py:364-390 */
  ORC_UNIFORM_CROSSED_EB = 3,/* rapt/fields.py:392-427 */
  ORC_VAR_EARTH_DIPOLE = 4,  /* rapt/fields.py:429-470 */
  ORC_PARABOLIC = 5,         /* rapt/fields.py:472-511 */
  ORC_HARRIS = 6,            /* not in the reference: Harris sheet + uniform Ey */
  ORC_COMPRESSED_DIPOLE = 7, /* not in the reference: breathing dipole + induced E */
  ORC_GRID = 8               /* rapt/fields.py:513-814 (Grid), data in the grid fields below */
};

typedef struct {
  int model;
  int is_static;      /* _Field.static */
  double p[8];        /* model parameters */
  double gradstep;    /* _Field.gradientstepsize */
  double timestep;    /* _Field.timederivstepsize */
  /* ORC_GRID: axes and [nt][nx][ny][nz][3] snapshots (host memory, owned by the caller) */
  const double *gt, *gx, *gy, *gz, *gB, *gE;
  int nt, nx, ny, nz;
} orc_field;

typedef struct {
  double rtol, atol;       /* params["solvertolerances"] */
  double cycres;           /* params["cyclotronresolution"] */
  double gctimestep;       /* params["GCtimestep"] (0: bounce-period cadence) */
  double epss, epst;       /* params["epss"], params["epst"] */
  int enforce_equatorial;  /* params["enforce equatorial"] */
  int tableau;             /* 0: DOP853 (particle) / DOPRI5 (GC); 1: RKF45 (rkf.py) */
  int gc_eom;              /* 0 TaoChanBrizard, 1 BrizardChan, 2 NorthropTeller */
  int nsteps;              /* SciPy ode nsteps (500) */
  double rkf_tol, rkf_hmin;/* RKF45 tableau: rkf.py tol and hmin */
  double bounceres;        /* params["bounceresolution"]: GC cadence T_b / bounceres when gctimestep == 0 */
  double flres;            /* params["fieldlineresolution"] */
  int bounce_quad;         /* half-bounce integral: 0 QAGS as the reference, 1 converged */
  int dense;               /* guiding centres: dense output without restarts (no reference counterpart) */
} orc_config;

/* One tracer (a Particle or a GuidingCenter segment). */
typedef struct {
  int mode;          /* 0 particle (t,x,y,z,px,py,pz), 1 guiding centre (t,x,y,z,ppar) */
  int status;        /* ORC_ST_* */
  double t;          /* time of the last trajectory row */
  double s[6];       /* particle: x,y,z,px,py,pz; GC: x,y,z,ppar */
  double mu;         /* GC magnetic moment */
  double v;          /* GC attribute self.v (speed) */
  double mass, charge;
  double tcur;       /* tracer .tcur */
  int64_t naccept, nreject, nfcn, nstep;
} orc_tracer;

enum {
  ORC_ST_OK = 0, ORC_ST_MAXSTEPS = 2, ORC_ST_HMIN = 3, ORC_ST_NONFINITE = 4,
  ORC_ST_GC_NOCONV = 5, ORC_ST_ROWS_FULL = 6, ORC_ST_BAD_INPUT = 7,
  ORC_ST_RKF_HMIN = 8, ORC_ST_ADAPTIVE_LIMIT = 9, ORC_ST_FIELDLINE = 10, ORC_ST_OUT_OF_GRID = 11
};

void orc_field_init(orc_field* f, int model, const double* params, int nparams);
void orc_config_default(orc_config* c);

/* _Field methods (rapt/fields.py:42-280). tpos = (t,x,y,z). */
void orc_B(const orc_field* f, const double* tpos, double* out3);
void orc_E(const orc_field* f, const double* tpos, double* out3);
double orc_magB(const orc_field* f, const double* tpos);
void orc_unitb(const orc_field* f, const double* tpos, double* out3);
void orc_gradB(const orc_field* f, const double* tpos, double* out3);
void orc_jacobianB(const orc_field* f, const double* tpos, double* out9);
double orc_curvature(const orc_field* f, const double* tpos);
void orc_curlb(const orc_field* f, const double* tpos, double* out3);
double orc_dBdt(const orc_field* f, const double* tpos);
void orc_dbdt(const orc_field* f, const double* tpos, double* out3);
double orc_lengthscale(const orc_field* f, const double* tpos);
double orc_timescale(const orc_field* f, const double* tpos);

/* Right-hand sides. */
void orc_particle_rhs(const orc_field* f, const orc_config* c, double mass, double charge,
                      double gm, double t, const double* Y6, double* out6);
void orc_gc_rhs(const orc_field* f, const orc_config* c, int eom, double mass, double charge,
                double mu, double v, double t, const double* Y4, double* out4);

/* One SciPy-ode integrate() call: 0 = DOP853, 1 = DOPRI5. Returns idid. */
int orc_integrate_particle(const orc_field* f, const orc_config* c, int method, double mass,
                           double charge, double gm, double* x, double* y6, double xend,
                           double beta, int64_t* counters4);
int orc_integrate_gc(const orc_field* f, const orc_config* c, int method, double mass,
                     double charge, double mu, double v, double* x, double* y4, double xend,
                     int64_t* counters4);

/* Constructors and conversions. */
void orc_particle_new(const double* pos, const double* vel, double t0, double mass,
                      double charge, orc_tracer* out);
void orc_gc_new_pa(const orc_field* f, const double* pos, double v, double pa, double t0,
                   double mass, double charge, orc_tracer* out);
int orc_guidingcenter(const orc_field* f, double t, const double* r, const double* v,
                      double mass, double charge, double* gc3, double* vp, double* speed);
void orc_gctofp(const orc_field* f, double t, const double* R, double vp, double speed,
                double mass, double charge, double gyrophase, double* pos3, double* vel3);
int orc_gc_from_particle(const orc_field* f, const orc_tracer* p, orc_tracer* out);
void orc_particle_from_gc(const orc_field* f, const orc_tracer* g, orc_tracer* out);

int orc_particle_isadiabatic(const orc_field* f, const orc_config* c, const orc_tracer* p);
int orc_gc_isadiabatic(const orc_field* f, const orc_config* c, const orc_tracer* g);

/* Tracer advance. rows: max_rows x 7 doubles (t, s0..s5); *nrows counts rows written.
 * Returns 0 (ran to the end), 1 (Adiabatic / NonAdiabatic raised). */
int orc_particle_advance(const orc_field* f, const orc_config* c, orc_tracer* p, double delta,
                         int check_adiabaticity, double* rows, int max_rows, int* nrows);
int orc_gc_advance(const orc_field* f, const orc_config* c, orc_tracer* g, double delta,
                   int check_adiabaticity, double* rows, int max_rows, int* nrows);

/* Field lines and the bounce period (fieldline_oracle.cpp): GuidingCenter.bounceperiod
 * (GuidingCenter.py:593-606), flutils.halfbouncepath (flutils.py:254-316), the
 * (s, |B|) samples of Fieldline.trace (fieldline.py:37-107), and QAGS on test
 * integrands (for pinning against scipy.integrate.quad). quad 0: the half-bounce
 * integral by QAGS at epsrel 1e-4 as the reference; 1: converged (substitution
 * and composite Gauss-Legendre, the device's method). */
double orc_gc_bounceperiod(const orc_field* f, const orc_tracer* g, double flres, int quad);
double orc_halfbouncepath(const orc_field* f, const double* tpos, double Bm, double flres, int quad, int* npts);
/* flutils.eye and flutils.gradI (second invariant and its gradient), quad as above;
 * eye is NaN where the reference raises (its Simpson branch below 70 degrees
 * equatorial pitch angle calls an undefined name; failed trim assertion). */
double orc_eye(const orc_field* f, const double* tpos, double Bm, double flres, int quad);
void orc_gradI(const orc_field* f, const double* tpos, double Bm, double d, double flres, int quad, double* out3);
/* BounceCenter (rapt/BounceCenter.py): the constructor's magnetic moment, the
 * bounce-averaged drift velocity and advance(delta). state[5] = (t, x, y, z,
 * tcur) in/out; rows[max_rows][4]. Returns a status. */
double orc_bc_mu(const orc_field* f, const double* pos, double v, double pa, double t0, double mass);
void orc_bc_rhs(const orc_field* f, const double* tpos, double mass, double charge, double v, double Bm, double d,
                double flres, int quad, double* out3);
int orc_bc_advance(const orc_field* f, const orc_config* c, double* state, double v, double mu, double mass,
                   double charge, double delta, double bctimestep, double d, int quad, double* rows, int max_rows,
                   int* nrows, int64_t* counters4);
int orc_fieldline_sB(const orc_field* f, const double* tpos, double Bm, double flres, double* s, double* B,
                     int cap);
double orc_qags_test(int which, double a, double b, double epsabs, double epsrel, int limit, int* ier);

/* Adaptive (rapt/Adaptive.py). init returns the starting tracer. advance writes
 * rows (with a per-row mode byte) and a switch log (time, new mode). */
int orc_adaptive_init(const orc_field* f, const orc_config* c, const double* pos,
                      const double* vel, double t0, double mass, double charge, orc_tracer* out);
int orc_adaptive_advance(const orc_field* f, const orc_config* c, orc_tracer* cur, double delta,
                         double* rows, int8_t* row_mode, int max_rows, int* nrows,
                         double* sw_time, int8_t* sw_mode, int max_sw, int* nsw);

/* Batched runner over independent tracers with OpenMP threads.
 * kind: 0 particle, 1 GC, 2 adaptive. Tracers are advanced in place. */
void orc_batch_advance(const orc_field* f, const orc_config* c, int kind, int64_t n,
                       orc_tracer* tr, const double* delta, int nthreads);

#ifdef __cplusplus
}
#endif
#endif
