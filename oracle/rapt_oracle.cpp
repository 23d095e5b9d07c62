// rapt_oracle.cpp -- CPU restatement of RAPT's tracer hot path (test oracle).
//
// TEST INFRASTRUCTURE ONLY. Imported by tests/, __graft_entry__.smoke() and the
// CPU-baseline leg of bench.py; never linked into the product library.
//
// Each function cites the reference file:line it restates. The ODE drivers
// restate the published Dormand-Prince methods as implemented by Hairer's
// DOPRI5 and DOP853 codes (Hairer, Norsett & Wanner, "Solving Ordinary
// Differential Equations I", 2nd ed., Sec. II.4-II.5 and II.10), which SciPy's
// `ode` integrators "dopri5"/"dop853" wrap (scipy/integrate/_ode.py, SciPy
// 1.18.1 installed here; the reference pins SciPy 1.3.1, requirements.txt:2).
// Their controller parameters are the ones SciPy passes (safety 0.9,
// dfactor/ifactor 0.2/10 for dopri5 and 0.3/6 for dop853, nsteps 500,
// beta as given) and the automatic initial step is recomputed at every
// integrate() call, exactly as observed from SciPy's per-call counters.
//
// Compiled with -ffp-contract=off so that x86 and Arm builds round alike.
#include "rapt_oracle.h"

#include <cmath>
#include <cstring>
#include <algorithm>

namespace {

// rapt/__init__.py:5-10
const double kE = 1.602176565e-19;
const double kC = 299792458.0;
const double kB0 = 3.07e-5;
const double kRe = 6378137.0;
const double kPi = 3.141592653589793;

// numpy's 3-element np.dot (OpenBLAS ddot on the x86 host where the reference
// was pinned) rounds as fma(a2,b2, fma(a1,b1, a0*b0)); using the same form keeps
// the oracle bit-identical to the reference on that host.
inline double dot3(const double* a, const double* b) { return std::fma(a[2], b[2], std::fma(a[1], b[1], a[0] * b[0])); }
inline void cross3(const double* a, const double* b, double* o) {
  o[0] = a[1] * b[2] - a[2] * b[1];
  o[1] = a[2] * b[0] - a[0] * b[2];
  o[2] = a[0] * b[1] - a[1] * b[0];
}
inline double sgn(double x) { return (x > 0) - (x < 0); }

}  // namespace

extern "C" {

void orc_config_default(orc_config* c) {
  // rapt/__init__.py:21-34
  c->rtol = 1.49012e-8;
  c->atol = 1.49012e-8;
  c->cycres = 10;
  c->gctimestep = 0;
  c->epss = 5e-2;
  c->epst = 5e-2;
  c->enforce_equatorial = 0;
  c->tableau = 0;
  c->gc_eom = 0;
  c->nsteps = 500;
  c->bounceres = 10;
  c->flres = 50;
  c->bounce_quad = 0;
  c->rkf_tol = 1e-3;
  c->rkf_hmin = 1e-12;
}

void orc_field_init(orc_field* f, int model, const double* params, int nparams) {
  std::memset(f, 0, sizeof(*f));
  f->model = model;
  f->gradstep = 1e-6;  // _Field.__init__, fields.py:38-41
  f->timestep = 1e-3;
  f->is_static = 1;
  double* p = f->p;
  switch (model) {
    case ORC_EARTH_DIPOLE:  // fields.py:297-300
      p[0] = kB0;
      f->gradstep = kRe * 1e-6;
      break;
    case ORC_DOUBLE_DIPOLE:  // fields.py:336-342
      p[0] = kB0; p[1] = 20 * kRe; p[2] = 1;
      f->gradstep = kRe / 1000;
      break;
    case ORC_UNIFORM_BZ:  // fields.py:376-378
      p[0] = 1;
      break;
    case ORC_UNIFORM_CROSSED_EB:  // fields.py:408-412 (Ey, Bz)
      p[0] = 1; p[1] = 1;
      f->is_static = 0;
      break;
    case ORC_VAR_EARTH_DIPOLE:  // fields.py:449-454 (amp, period)
      p[0] = 0.1; p[1] = 10;
      f->gradstep = kRe / 1000;
      f->is_static = 0;
      break;
    case ORC_PARABOLIC:  // fields.py:500-504 (B0, Bn, d)
      p[0] = 10.0; p[1] = 1.0; p[2] = 0.2;
      break;
    case ORC_HARRIS:  // (B0, L, Bn, Ey); FD step L*1e-4
      p[0] = 20e-9; p[1] = 0.5 * kRe; p[2] = 2e-9; p[3] = 0.2e-3;
      f->is_static = 0;
      break;
    case ORC_COMPRESSED_DIPOLE:  // (B0, amp, period)
      p[0] = kB0; p[1] = 0.1; p[2] = 60.0;
      f->gradstep = kRe / 1000;
      f->is_static = 0;
      break;
    case ORC_GRID:  // fields.py:577-578; the data are attached by the caller
      f->gradstep = 1e-3 * kRe;
      break;
    default:
      break;
  }
  for (int i = 0; i < nparams && i < 8; ++i) p[i] = params[i];
  if (model == ORC_HARRIS) f->gradstep = p[1] * 1e-4;
}

// ---------------------------------------------------------------- Grid
// Grid.Bgrid / Egrid (rapt/fields.py:707-771) evaluate SciPy's
// RegularGridInterpolator (method "linear", bounds_error=True) over
// (t, x, y, z), or (x, y, z) for one snapshot. Restated from SciPy 1.18
// interpolate/_rgi.py: _prepare_xi (bounds check: ValueError unless
// g[0] <= v <= g[-1] on every axis), find_indices (the cell i with
// g[i] <= v < g[i+1], the last cell for v == g[-1]; w = (v - g[i]) /
// (g[i+1] - g[i])) and _evaluate_linear (corners in itertools.product order,
// lower weight 1 - w, upper w; weight = ((1 * w_0) * w_1) ...; value summed from
// 0 corner by corner). The reference's three-snapshot window (fields.py:695-705)
// gives the same values as one interpolator over all snapshots on the interval
// it covers. Outside the grid this returns NaN (the reference raises).
namespace {
bool grid_inside(const double* g, int n, double v) { return g[0] <= v && v <= g[n - 1]; }

int grid_cell(const double* g, int n, double v, double* w) {
  int i = 0;
  while (i + 2 < n && g[i + 1] <= v) ++i;  // linear scan: the oracle favours plainness
  *w = (v - g[i]) / (g[i + 1] - g[i]);
  return i;
}

void grid_eval(const orc_field* f, const double* V, const double* tpos, double* o) {
  const double t = tpos[0], x = tpos[1], y = tpos[2], z = tpos[3];
  if (!grid_inside(f->gx, f->nx, x) || !grid_inside(f->gy, f->ny, y) || !grid_inside(f->gz, f->nz, z) ||
      (f->nt > 1 && !grid_inside(f->gt, f->nt, t))) {
    o[0] = o[1] = o[2] = NAN;
    return;
  }
  // axes in the interpolator's order; one snapshot drops the time axis
  const int nd = f->nt > 1 ? 4 : 3;
  const double* g[4];
  int n[4];
  double v[4];
  int k = 0;
  if (nd == 4) { g[k] = f->gt; n[k] = f->nt; v[k++] = t; }
  g[k] = f->gx; n[k] = f->nx; v[k++] = x;
  g[k] = f->gy; n[k] = f->ny; v[k++] = y;
  g[k] = f->gz; n[k] = f->nz; v[k++] = z;
  int idx[4];
  double w[4];
  for (int d = 0; d < nd; ++d) idx[d] = grid_cell(g[d], n[d], v[d], &w[d]);
  double val[3] = {0.0, 0.0, 0.0};
  for (int corner = 0; corner < (1 << nd); ++corner) {  // bit nd-1-d set: upper corner on axis d
    double weight = 1.0;
    int64_t node = 0;
    for (int d = 0; d < nd; ++d) {
      const int up = (corner >> (nd - 1 - d)) & 1;
      weight = weight * (up ? w[d] : 1.0 - w[d]);
      node = node * n[d] + idx[d] + up;
    }
    for (int c = 0; c < 3; ++c) val[c] = val[c] + V[3 * node + c] * weight;
  }
  o[0] = val[0]; o[1] = val[1]; o[2] = val[2];
}
}  // namespace

// ---------------------------------------------------------------- fields
void orc_B(const orc_field* f, const double* tpos, double* o) {
  const double t = tpos[0], x = tpos[1], y = tpos[2], z = tpos[3];
  const double* p = f->p;
  switch (f->model) {
    case ORC_EARTH_DIPOLE: {  // fields.py:301-317
      const double coeff = -3 * p[0] * (kRe * kRe * kRe);
      const double r2 = x * x + y * y + z * z;
      const double s = coeff / std::pow(r2, 2.5);
      o[0] = s * (x * z); o[1] = s * (y * z); o[2] = s * (z * z - r2 / 3);
      return;
    }
    case ORC_DOUBLE_DIPOLE: {  // fields.py:344-362
      const double coeff = -p[0] * (kRe * kRe * kRe);
      double d1 = std::pow(x * x + y * y + z * z, 5.0 / 2.0);
      double b1[3] = {3 * x * z / d1, 3 * y * z / d1, (2 * z * z - x * x - y * y) / d1};
      const double x2 = x - p[1];
      double d2 = std::pow(x2 * x2 + y * y + z * z, 5.0 / 2.0);
      const double k = p[2];
      double b2[3] = {k * (3 * x2 * z) / d2, k * (3 * y * z) / d2, k * (2 * z * z - x2 * x2 - y * y) / d2};
      for (int i = 0; i < 3; ++i) o[i] = coeff * (b1[i] + b2[i]);
      return;
    }
    case ORC_UNIFORM_BZ:
      o[0] = 0; o[1] = 0; o[2] = p[0];
      return;
    case ORC_UNIFORM_CROSSED_EB:
      o[0] = 0; o[1] = 0; o[2] = p[1];
      return;
    case ORC_VAR_EARTH_DIPOLE: {  // fields.py:455-470
      const double s = -kB0 * (kRe * kRe * kRe) * (1 + p[0] * std::sin(2 * kPi * t / p[1]));
      const double d = std::pow(x * x + y * y + z * z, 5.0 / 2.0);
      o[0] = s * (3 * x * z) / d; o[1] = s * (3 * y * z) / d; o[2] = s * (2 * z * z - x * x - y * y) / d;
      return;
    }
    case ORC_PARABOLIC: {  // fields.py:506-511; the |z|>1 branch uses the module-level
                           // B0 (3.07e-5 T), not self.B0 -- kept as in the reference.
      if (std::fabs(z) <= 1.0) { o[0] = p[0] * z / p[2]; o[1] = 0; o[2] = p[1]; }
      else { o[0] = sgn(z) * kB0; o[1] = 0; o[2] = p[1]; }
      return;
    }
    case ORC_HARRIS:
      o[0] = p[0] * std::tanh(z / p[1]); o[1] = 0; o[2] = p[2];
      return;
    case ORC_GRID:
      grid_eval(f, f->gB, tpos, o);
      return;
    case ORC_COMPRESSED_DIPOLE: {  // VarEarthDipole form with B0(t) = B0 (1 + amp sin(2 pi t / P))
      const double s = -p[0] * (kRe * kRe * kRe) * (1 + p[1] * std::sin(2 * kPi * t / p[2]));
      const double d = std::pow(x * x + y * y + z * z, 5.0 / 2.0);
      o[0] = s * (3 * x * z) / d; o[1] = s * (3 * y * z) / d; o[2] = s * (2 * z * z - x * x - y * y) / d;
      return;
    }
    default:
      o[0] = o[1] = o[2] = 0;
  }
}

void orc_E(const orc_field* f, const double* tpos, double* o) {
  const double* p = f->p;
  o[0] = o[1] = o[2] = 0;  // _Field.E, fields.py:60-75
  switch (f->model) {
    case ORC_UNIFORM_CROSSED_EB: o[1] = p[0]; return;  // fields.py:413-427
    case ORC_HARRIS: o[1] = p[3]; return;
    case ORC_GRID:
      if (f->gE) grid_eval(f, f->gE, tpos, o);
      return;
    case ORC_COMPRESSED_DIPOLE: {
      // E = -dA/dt with A = B0(t) Re^3 (y, -x, 0) / r^3, whose curl is B above.
      const double t = tpos[0], x = tpos[1], y = tpos[2], z = tpos[3];
      const double w = 2 * kPi / p[2];
      const double dB0dt = p[0] * p[1] * w * std::cos(w * t);
      const double r3 = std::pow(x * x + y * y + z * z, 1.5);
      const double s = -dB0dt * (kRe * kRe * kRe) / r3;
      o[0] = s * y; o[1] = -s * x; o[2] = 0;
      return;
    }
    default: return;
  }
}

double orc_magB(const orc_field* f, const double* tpos) {  // fields.py:94-109
  double b[3];
  orc_B(f, tpos, b);
  return std::sqrt(dot3(b, b));
}

void orc_unitb(const orc_field* f, const double* tpos, double* o) {  // fields.py:77-92
  double b[3];
  orc_B(f, tpos, b);
  const double m = std::sqrt(dot3(b, b));
  o[0] = b[0] / m; o[1] = b[1] / m; o[2] = b[2] / m;
}

static inline void shifted(const double* tpos, int axis, double d, double* out) {
  out[0] = tpos[0]; out[1] = tpos[1]; out[2] = tpos[2]; out[3] = tpos[3];
  out[axis] = tpos[axis] + d;
}

void orc_gradB(const orc_field* f, const double* tpos, double* o) {  // fields.py:111-131
  const double d = f->gradstep;
  for (int i = 0; i < 3; ++i) {
    double tp[4], tm[4];
    shifted(tpos, i + 1, d, tp);
    shifted(tpos, i + 1, -d, tm);
    o[i] = (orc_magB(f, tp) - orc_magB(f, tm)) / (2 * d);
  }
}

void orc_jacobianB(const orc_field* f, const double* tpos, double* o) {  // fields.py:133-153
  const double d = f->gradstep;
  for (int j = 0; j < 3; ++j) {
    double tp[4], tm[4], bp[3], bm[3];
    shifted(tpos, j + 1, d, tp);
    shifted(tpos, j + 1, -d, tm);
    orc_B(f, tp, bp);
    orc_B(f, tm, bm);
    for (int i = 0; i < 3; ++i) o[3 * i + j] = (bp[i] - bm[i]) / (2 * d);
  }
}

double orc_curvature(const orc_field* f, const double* tpos) {  // fields.py:155-174
  double b[3], gb[3];
  orc_B(f, tpos, b);
  const double B = std::sqrt(dot3(b, b));
  orc_gradB(f, tpos, gb);
  // np.dot(gB, B) with the scalar |B| is an elementwise product in the
  // reference (fields.py:173), so each component is scaled separately.
  double gp[3];
  for (int i = 0; i < 3; ++i) gp[i] = gb[i] - (gb[i] * B / (B * B)) * b[i];
  return std::sqrt(dot3(gp, gp)) / B;
}

void orc_curlb(const orc_field* f, const double* tpos, double* o) {  // fields.py:176-200, _M1 :33-36
  const double d = f->gradstep;
  double u[6][3];
  for (int j = 0; j < 3; ++j) {
    double tp[4], tm[4];
    shifted(tpos, j + 1, d, tp);
    shifted(tpos, j + 1, -d, tm);
    orc_unitb(f, tp, u[2 * j]);
    orc_unitb(f, tm, u[2 * j + 1]);
  }
  // Rows of _M1 applied to beta = (b(x+d), b(x-d), b(y+d), b(y-d), b(z+d), b(z-d)).
  // The association order is the one numpy's np.dot(_M1, beta) (OpenBLAS dgemv
  // on the x86 host where the reference was pinned) rounds with, so the oracle
  // stays bit-identical to the reference there.
  o[0] = ((u[2][2] + (-u[4][1] - u[3][2])) + u[5][1]) / (2 * d);
  o[1] = ((u[4][0] - u[0][2]) + (u[1][2] - u[5][0])) / (2 * d);
  o[2] = ((-u[1][1] - u[2][0]) + (u[0][1] + u[3][0])) / (2 * d);
}

double orc_dBdt(const orc_field* f, const double* tpos) {  // fields.py:202-223
  if (f->is_static) return 0;
  const double d = f->timestep;
  double a[4] = {tpos[0] - d, tpos[1], tpos[2], tpos[3]};
  double b[4] = {tpos[0] + d, tpos[1], tpos[2], tpos[3]};
  return (orc_magB(f, b) - orc_magB(f, a)) / d / 2;
}

void orc_dbdt(const orc_field* f, const double* tpos, double* o) {  // fields.py:225-245
  if (f->is_static) { o[0] = o[1] = o[2] = 0; return; }
  const double d = f->timestep;
  double a[4] = {tpos[0] - d, tpos[1], tpos[2], tpos[3]};
  double b[4] = {tpos[0] + d, tpos[1], tpos[2], tpos[3]};
  double b1[3], b2[3];
  orc_unitb(f, a, b1);
  orc_unitb(f, b, b2);
  for (int i = 0; i < 3; ++i) o[i] = (b2[i] - b1[i]) / d / 2;
}

double orc_lengthscale(const orc_field* f, const double* tpos) {  // fields.py:247-261
  double J[9];
  orc_jacobianB(f, tpos, J);
  double m = 0;
  for (int i = 0; i < 9; ++i) m = std::max(m, std::fabs(J[i]));
  return orc_magB(f, tpos) / m;
}

double orc_timescale(const orc_field* f, const double* tpos) {  // fields.py:263-280
  if (f->is_static) return NAN;  // reference returns None; never used when static
  return orc_magB(f, tpos) / std::fabs(orc_dBdt(f, tpos));
}

// ---------------------------------------------------------------- EOMs
void orc_particle_rhs(const orc_field* f, const orc_config* c, double mass, double charge,
                      double gm, double t, const double* Y, double* out) {
  // Particle.advance eom closure, rapt/Particle.py:284-298. When the field is
  // not static gm is recomputed from the stage momentum; otherwise the value
  // frozen at the start of advance() is used.
  double tpos[4] = {t, Y[0], Y[1], Y[2]};
  const double* mom = Y + 3;
  if (!f->is_static) gm = std::sqrt(mass * mass + dot3(mom, mom) / (kC * kC));
  out[0] = Y[3] / gm; out[1] = Y[4] / gm; out[2] = Y[5] / gm;
  double E[3], B[3], pxB[3];
  orc_E(f, tpos, E);
  orc_B(f, tpos, B);
  cross3(mom, B, pxB);
  for (int i = 0; i < 3; ++i) out[3 + i] = charge * (E[i] + pxB[i] / gm);
  if (c->enforce_equatorial) out[2] = out[5] = 0;
}

void orc_gc_rhs(const orc_field* f, const orc_config* c, int eom, double mass, double charge,
                double mu, double v, double t, const double* Y, double* out) {
  double tpos[4] = {t, Y[0], Y[1], Y[2]};
  const double ppar = Y[3];
  double B[3];
  orc_B(f, tpos, B);
  const double Bmag = std::sqrt(dot3(B, B));
  const double ub[3] = {B[0] / Bmag, B[1] / Bmag, B[2] / Bmag};
  if (eom == 0) {  // _TaoChanBrizardEOM, rapt/GuidingCenter.py:329-355
    const double gamma = std::sqrt(1 + 2 * mu * Bmag / (mass * kC * kC) + std::pow(ppar / (mass * kC), 2));
    double cb[3], E[3], db[3], gB[3];
    orc_curlb(f, tpos, cb);
    double Bs[3];
    for (int i = 0; i < 3; ++i) Bs[i] = B[i] + ppar * cb[i] / charge;
    const double Bspar = dot3(Bs, ub);
    orc_E(f, tpos, E);
    orc_dbdt(f, tpos, db);
    orc_gradB(f, tpos, gB);
    double Es[3];
    for (int i = 0; i < 3; ++i) Es[i] = E[i] - (ppar * db[i] + mu * gB[i] / gamma) / charge;
    double Exb[3];
    cross3(Es, ub, Exb);
    for (int i = 0; i < 3; ++i) out[i] = (ppar * Bs[i] / (gamma * mass) + Exb[i]) / Bspar;
    out[3] = charge * dot3(Es, Bs) / Bspar;
  } else if (eom == 1) {  // _BrizardChanEOM, rapt/GuidingCenter.py:357-379
    const double gamma = 1.0 / std::sqrt(1 - std::pow(v / kC, 2));
    double gB[3], cb[3];
    orc_gradB(f, tpos, gB);
    orc_curlb(f, tpos, cb);
    double Bs[3];
    for (int i = 0; i < 3; ++i) Bs[i] = B[i] + ppar * cb[i] / charge;
    const double Bspar = dot3(Bs, ub);
    double bxg[3];
    cross3(ub, gB, bxg);
    for (int i = 0; i < 3; ++i)
      out[i] = (ppar * Bs[i] / (gamma * mass) + mu * bxg[i] / (charge * gamma)) / Bspar;
    out[3] = -mu * dot3(Bs, gB) / (gamma * Bspar);
  } else {  // _NorthropTellerEOM, rapt/GuidingCenter.py:381-395
    const double gamma = 1.0 / std::sqrt(1 - std::pow(v / kC, 2));
    const double gm = gamma * mass;
    double gB[3];
    orc_gradB(f, tpos, gB);
    double bxg[3];
    cross3(ub, gB, bxg);
    const double s = (gm * (v * v) + ppar * ppar / gm) / ((2 * charge) * (Bmag * Bmag));
    for (int i = 0; i < 3; ++i) out[i] = s * bxg[i] + ppar * ub[i] / gm;
    out[3] = -mu * dot3(ub, gB) / gamma;
  }
  if (c->enforce_equatorial) out[2] = out[3] = 0;
}

}  // extern "C"

// ---------------------------------------------------------------- ODE drivers
namespace {

struct Counters {
  int64_t nfcn = 0, nstep = 0, naccpt = 0, nrejct = 0;
  bool stop_nan = false;  // Grid: a NaN error norm means a stage left the grid (idid -6)
};

// Automatic initial step (Hairer's HINIT, Solving ODEs I, Sec. II.4).
template <class F>
double hinit(F& f, int n, double x, const double* y, double posneg, const double* f0, int iord,
             double hmax, double atol, double rtol) {
  double dnf = 0, dny = 0;
  for (int i = 0; i < n; ++i) {
    const double sk = atol + rtol * std::fabs(y[i]);
    dnf += (f0[i] / sk) * (f0[i] / sk);
    dny += (y[i] / sk) * (y[i] / sk);
  }
  double h = (dnf <= 1e-10 || dny <= 1e-10) ? 1e-6 : std::sqrt(dny / dnf) * 0.01;
  h = std::min(h, hmax);
  h = std::copysign(h, posneg);
  double y1[6], f1[6];
  for (int i = 0; i < n; ++i) y1[i] = y[i] + h * f0[i];
  f(x + h, y1, f1);
  double der2 = 0;
  for (int i = 0; i < n; ++i) {
    const double sk = atol + rtol * std::fabs(y[i]);
    der2 += ((f1[i] - f0[i]) / sk) * ((f1[i] - f0[i]) / sk);
  }
  der2 = std::sqrt(der2) / h;
  const double der12 = std::max(std::fabs(der2), std::sqrt(dnf));
  const double h1 = (der12 <= 1e-15) ? std::max(1e-6, std::fabs(h) * 1e-3) : std::pow(0.01 / der12, 1.0 / iord);
  h = std::min(std::min(100 * std::fabs(h), h1), hmax);
  return std::copysign(h, posneg);
}

// DOPRI5 core (Dormand-Prince 5(4), FSAL, Lund stabilisation).
template <class F>
int dopri5(F& f, int n, double& x, double* y, double xend, double rtol, double atol, int nmax,
           Counters& cnt, double safe = 0.9, double fac1 = 0.2, double fac2 = 10.0, double beta = 0.04) {
  const double c2 = 0.2, c3 = 0.3, c4 = 0.8, c5 = 8.0 / 9.0;
  const double a21 = 0.2, a31 = 3.0 / 40.0, a32 = 9.0 / 40.0;
  const double a41 = 44.0 / 45.0, a42 = -56.0 / 15.0, a43 = 32.0 / 9.0;
  const double a51 = 19372.0 / 6561.0, a52 = -25360.0 / 2187.0, a53 = 64448.0 / 6561.0, a54 = -212.0 / 729.0;
  const double a61 = 9017.0 / 3168.0, a62 = -355.0 / 33.0, a63 = 46732.0 / 5247.0, a64 = 49.0 / 176.0,
               a65 = -5103.0 / 18656.0;
  const double a71 = 35.0 / 384.0, a73 = 500.0 / 1113.0, a74 = 125.0 / 192.0, a75 = -2187.0 / 6784.0,
               a76 = 11.0 / 84.0;
  const double e1 = 71.0 / 57600.0, e3 = -71.0 / 16695.0, e4 = 71.0 / 1920.0, e5 = -17253.0 / 339200.0,
               e6 = 22.0 / 525.0, e7 = -1.0 / 40.0;
  const double uround = 2.3e-16;
  double facold = 1e-4;
  const double expo1 = 0.2 - beta * 0.75, facc1 = 1.0 / fac1, facc2 = 1.0 / fac2;
  const double posneg = std::copysign(1.0, xend - x);
  const double hmax = std::fabs(xend - x);
  double k1[6], k2[6], k3[6], k4[6], k5[6], k6[6], y1[6], ysti[6];
  f(x, y, k1);
  double h = hinit(f, n, x, y, posneg, k1, 5, hmax, atol, rtol);
  cnt.nfcn += 2;
  bool reject = false, last = false;
  for (;;) {
    if (cnt.nstep > nmax) return -2;
    if (0.1 * std::fabs(h) <= std::fabs(x) * uround) return -3;
    if ((x + 1.01 * h - xend) * posneg > 0.0) { h = xend - x; last = true; }
    cnt.nstep++;
    for (int i = 0; i < n; ++i) y1[i] = y[i] + h * a21 * k1[i];
    f(x + c2 * h, y1, k2);
    for (int i = 0; i < n; ++i) y1[i] = y[i] + h * (a31 * k1[i] + a32 * k2[i]);
    f(x + c3 * h, y1, k3);
    for (int i = 0; i < n; ++i) y1[i] = y[i] + h * (a41 * k1[i] + a42 * k2[i] + a43 * k3[i]);
    f(x + c4 * h, y1, k4);
    for (int i = 0; i < n; ++i) y1[i] = y[i] + h * (a51 * k1[i] + a52 * k2[i] + a53 * k3[i] + a54 * k4[i]);
    f(x + c5 * h, y1, k5);
    for (int i = 0; i < n; ++i)
      ysti[i] = y[i] + h * (a61 * k1[i] + a62 * k2[i] + a63 * k3[i] + a64 * k4[i] + a65 * k5[i]);
    const double xph = x + h;
    f(xph, ysti, k6);
    for (int i = 0; i < n; ++i)
      y1[i] = y[i] + h * (a71 * k1[i] + a73 * k3[i] + a74 * k4[i] + a75 * k5[i] + a76 * k6[i]);
    f(xph, y1, k2);
    for (int i = 0; i < n; ++i)
      k4[i] = (e1 * k1[i] + e3 * k3[i] + e4 * k4[i] + e5 * k5[i] + e6 * k6[i] + e7 * k2[i]) * h;
    cnt.nfcn += 6;
    double err = 0;
    for (int i = 0; i < n; ++i) {
      const double sk = atol + rtol * std::max(std::fabs(y[i]), std::fabs(y1[i]));
      err += (k4[i] / sk) * (k4[i] / sk);
    }
    err = std::sqrt(err / n);
    if (cnt.stop_nan && std::isnan(err)) return -6;
    const double fac11 = std::pow(err, expo1);
    double fac = fac11 / std::pow(facold, beta);
    fac = std::max(facc2, std::min(facc1, fac / safe));
    double hnew = h / fac;
    if (err <= 1.0) {
      facold = std::max(err, 1.0e-4);
      cnt.naccpt++;
      for (int i = 0; i < n; ++i) { k1[i] = k2[i]; y[i] = y1[i]; }
      x = xph;
      if (last) return 1;
      if (std::fabs(hnew) > hmax) hnew = posneg * hmax;
      if (reject) hnew = posneg * std::min(std::fabs(hnew), std::fabs(h));
      reject = false;
    } else {
      hnew = h / std::min(facc1, fac11 / safe);
      reject = true;
      if (cnt.naccpt >= 1) cnt.nrejct++;
      last = false;
    }
    h = hnew;
  }
}

// DOP853 coefficients (Dormand-Prince 8(5,3), as published with Hairer's DOP853).
namespace d8 {
const double c2 = 0.526001519587677318785587544488e-01, c3 = 0.789002279381515978178381316732e-01,
             c4 = 0.118350341907227396726757197510e+00, c5 = 0.281649658092772603273242802490e+00,
             c6 = 0.333333333333333333333333333333e+00, c7 = 0.25e+00,
             c8 = 0.307692307692307692307692307692e+00, c9 = 0.651282051282051282051282051282e+00,
             c10 = 0.6e+00, c11 = 0.857142857142857142857142857142e+00;
const double b1 = 5.42937341165687622380535766363e-2, b6 = 4.45031289275240888144113950566e0,
             b7 = 1.89151789931450038304281599044e0, b8 = -5.8012039600105847814672114227e0,
             b9 = 3.1116436695781989440891606237e-1, b10 = -1.52160949662516078556178806805e-1,
             b11 = 2.01365400804030348374776537501e-1, b12 = 4.47106157277725905176885569043e-2;
const double bhh1 = 0.244094488188976377952755905512e+00, bhh2 = 0.733846688281611857341361741547e+00,
             bhh3 = 0.220588235294117647058823529412e-01;
const double er1 = 0.1312004499419488073250102996e-01, er6 = -0.1225156446376204440720569753e+01,
             er7 = -0.4957589496572501915214079952e+00, er8 = 0.1664377182454986536961530415e+01,
             er9 = -0.3503288487499736816886487290e+00, er10 = 0.3341791187130174790297318841e+00,
             er11 = 0.8192320648511571246570742613e-01, er12 = -0.2235530786388629525884427845e-01;
const double a21 = 5.26001519587677318785587544488e-2, a31 = 1.97250569845378994544595329183e-2,
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
}  // namespace d8

template <class F>
int dop853(F& f, int n, double& x, double* y, double xend, double rtol, double atol, int nmax,
           Counters& cnt, double beta, double safe = 0.9, double fac1 = 0.3, double fac2 = 6.0) {
  using namespace d8;
  const double uround = 2.3e-16;
  double facold = 1e-4;
  const double expo1 = 1.0 / 8.0 - beta * 0.2, facc1 = 1.0 / fac1, facc2 = 1.0 / fac2;
  const double posneg = std::copysign(1.0, xend - x);
  const double hmax = std::fabs(xend - x);
  double k1[6], k2[6], k3[6], k4[6], k5[6], k6[6], k7[6], k8[6], k9[6], k10[6], y1[6];
  f(x, y, k1);
  double h = hinit(f, n, x, y, posneg, k1, 8, hmax, atol, rtol);
  cnt.nfcn += 2;
  bool reject = false, last = false;
  for (;;) {
    if (cnt.nstep > nmax) return -2;
    if (0.1 * std::fabs(h) <= std::fabs(x) * uround) return -3;
    if ((x + 1.01 * h - xend) * posneg > 0.0) { h = xend - x; last = true; }
    cnt.nstep++;
    for (int i = 0; i < n; ++i) y1[i] = y[i] + h * a21 * k1[i];
    f(x + c2 * h, y1, k2);
    for (int i = 0; i < n; ++i) y1[i] = y[i] + h * (a31 * k1[i] + a32 * k2[i]);
    f(x + c3 * h, y1, k3);
    for (int i = 0; i < n; ++i) y1[i] = y[i] + h * (a41 * k1[i] + a43 * k3[i]);
    f(x + c4 * h, y1, k4);
    for (int i = 0; i < n; ++i) y1[i] = y[i] + h * (a51 * k1[i] + a53 * k3[i] + a54 * k4[i]);
    f(x + c5 * h, y1, k5);
    for (int i = 0; i < n; ++i) y1[i] = y[i] + h * (a61 * k1[i] + a64 * k4[i] + a65 * k5[i]);
    f(x + c6 * h, y1, k6);
    for (int i = 0; i < n; ++i) y1[i] = y[i] + h * (a71 * k1[i] + a74 * k4[i] + a75 * k5[i] + a76 * k6[i]);
    f(x + c7 * h, y1, k7);
    for (int i = 0; i < n; ++i)
      y1[i] = y[i] + h * (a81 * k1[i] + a84 * k4[i] + a85 * k5[i] + a86 * k6[i] + a87 * k7[i]);
    f(x + c8 * h, y1, k8);
    for (int i = 0; i < n; ++i)
      y1[i] = y[i] + h * (a91 * k1[i] + a94 * k4[i] + a95 * k5[i] + a96 * k6[i] + a97 * k7[i] + a98 * k8[i]);
    f(x + c9 * h, y1, k9);
    for (int i = 0; i < n; ++i)
      y1[i] = y[i] + h * (a101 * k1[i] + a104 * k4[i] + a105 * k5[i] + a106 * k6[i] + a107 * k7[i] +
                          a108 * k8[i] + a109 * k9[i]);
    f(x + c10 * h, y1, k10);
    for (int i = 0; i < n; ++i)
      y1[i] = y[i] + h * (a111 * k1[i] + a114 * k4[i] + a115 * k5[i] + a116 * k6[i] + a117 * k7[i] +
                          a118 * k8[i] + a119 * k9[i] + a1110 * k10[i]);
    f(x + c11 * h, y1, k2);
    const double xph = x + h;
    for (int i = 0; i < n; ++i)
      y1[i] = y[i] + h * (a121 * k1[i] + a124 * k4[i] + a125 * k5[i] + a126 * k6[i] + a127 * k7[i] +
                          a128 * k8[i] + a129 * k9[i] + a1210 * k10[i] + a1211 * k2[i]);
    f(xph, y1, k3);
    cnt.nfcn += 11;
    for (int i = 0; i < n; ++i) {
      k4[i] = b1 * k1[i] + b6 * k6[i] + b7 * k7[i] + b8 * k8[i] + b9 * k9[i] + b10 * k10[i] + b11 * k2[i] +
              b12 * k3[i];
      k5[i] = y[i] + h * k4[i];
    }
    double err = 0, err2 = 0;
    for (int i = 0; i < n; ++i) {
      const double sk = atol + rtol * std::max(std::fabs(y[i]), std::fabs(k5[i]));
      double erri = k4[i] - bhh1 * k1[i] - bhh2 * k9[i] - bhh3 * k3[i];
      err2 += (erri / sk) * (erri / sk);
      erri = er1 * k1[i] + er6 * k6[i] + er7 * k7[i] + er8 * k8[i] + er9 * k9[i] + er10 * k10[i] +
             er11 * k2[i] + er12 * k3[i];
      err += (erri / sk) * (erri / sk);
    }
    double deno = err + 0.01 * err2;
    if (deno <= 0.0) deno = 1.0;
    err = std::fabs(h) * err * std::sqrt(1.0 / (n * deno));
    if (cnt.stop_nan && std::isnan(err)) return -6;
    const double fac11 = std::pow(err, expo1);
    double fac = fac11 / std::pow(facold, beta);
    fac = std::max(facc2, std::min(facc1, fac / safe));
    double hnew = h / fac;
    if (err <= 1.0) {
      facold = std::max(err, 1.0e-4);
      cnt.naccpt++;
      f(xph, k5, k4);
      cnt.nfcn++;
      for (int i = 0; i < n; ++i) { k1[i] = k4[i]; y[i] = k5[i]; }
      x = xph;
      if (last) return 1;
      if (std::fabs(hnew) > hmax) hnew = posneg * hmax;
      if (reject) hnew = posneg * std::min(std::fabs(hnew), std::fabs(h));
      reject = false;
    } else {
      // SciPy 1.18.1's dop853 shrinks a rejected step by dfactor (h * 0.3):
      // pinned on 300/300 output intervals against its per-call counters and
      // its accepted-step times (ode.set_solout). DOPRI5 keeps Hairer's
      // h / min(1/fac1, err^expo1 / safe).
      hnew = h / facc1;
      reject = true;
      if (cnt.naccpt >= 1) cnt.nrejct++;
      last = false;
    }
    h = hnew;
  }
}

// RKF45 over one interval, restating rapt/rkf.py:13-143 (Fehlberg 4(5),
// absolute tolerance on max|err|/h, h *= clamp(0.84 (tol/r)^(1/4), 0.1, 4)).
// Returns 1 on success, -5 where rkf.py raises at hmin (rkf.py:136-139).
template <class F>
int rkf45(F& f, int n, double& t, double* x, double b, double tol, double hmax, double hmin,
          Counters& cnt, int max_iter) {
  // the decimal coefficients of rkf.py:48-87 (several differ from the exact
  // fractions in the last bit)
  const double a2 = 2.500000000000000e-01, a3 = 3.750000000000000e-01, a4 = 9.230769230769231e-01, a5 = 1.0,
               a6 = 5.000000000000000e-01;
  const double b21 = 2.500000000000000e-01, b31 = 9.375000000000000e-02, b32 = 2.812500000000000e-01,
               b41 = 8.793809740555303e-01, b42 = -3.277196176604461e+00, b43 = 3.320892125625853e+00,
               b51 = 2.032407407407407e+00, b52 = -8.000000000000000e+00, b53 = 7.173489278752436e+00,
               b54 = -2.058966861598441e-01, b61 = -2.962962962962963e-01, b62 = 2.000000000000000e+00,
               b63 = -1.381676413255361e+00, b64 = 4.529727095516569e-01, b65 = -2.750000000000000e-01;
  const double r1 = 2.777777777777778e-03, r3 = -2.994152046783626e-02, r4 = -2.919989367357789e-02,
               r5 = 2.000000000000000e-02, r6 = 3.636363636363636e-02;
  const double c1 = 1.157407407407407e-01, c3 = 5.489278752436647e-01, c4 = 5.353313840155945e-01,
               c5 = -2.000000000000000e-01;
  double h = hmax;
  double k1[6], k2[6], k3[6], k4[6], k5[6], k6[6], xt[6];
  int it = 0;
  while (t < b) {
    if (++it > max_iter) return -2;
    if (t + h > b) h = b - t;
    f(t, x, k1);
    for (int i = 0; i < n; ++i) { k1[i] *= h; xt[i] = x[i] + b21 * k1[i]; }
    f(t + a2 * h, xt, k2);
    for (int i = 0; i < n; ++i) { k2[i] *= h; xt[i] = x[i] + b31 * k1[i] + b32 * k2[i]; }
    f(t + a3 * h, xt, k3);
    for (int i = 0; i < n; ++i) { k3[i] *= h; xt[i] = x[i] + b41 * k1[i] + b42 * k2[i] + b43 * k3[i]; }
    f(t + a4 * h, xt, k4);
    for (int i = 0; i < n; ++i) {
      k4[i] *= h;
      xt[i] = x[i] + b51 * k1[i] + b52 * k2[i] + b53 * k3[i] + b54 * k4[i];
    }
    f(t + a5 * h, xt, k5);
    for (int i = 0; i < n; ++i) {
      k5[i] *= h;
      xt[i] = x[i] + b61 * k1[i] + b62 * k2[i] + b63 * k3[i] + b64 * k4[i] + b65 * k5[i];
    }
    f(t + a6 * h, xt, k6);
    for (int i = 0; i < n; ++i) k6[i] *= h;
    cnt.nfcn += 6;
    cnt.nstep++;
    double r = 0;
    bool nan_term = false;
    for (int i = 0; i < n; ++i) {
      const double ri = std::fabs(r1 * k1[i] + r3 * k3[i] + r4 * k4[i] + r5 * k5[i] + r6 * k6[i]) / h;
      r = std::max(r, ri);
      nan_term = nan_term || std::isnan(ri);
    }
    if (cnt.stop_nan && nan_term) return -6;
    if (r <= tol) {
      t = t + h;
      for (int i = 0; i < n; ++i) x[i] = x[i] + c1 * k1[i] + c3 * k3[i] + c4 * k4[i] + c5 * k5[i];
      cnt.naccpt++;
    } else {
      cnt.nrejct++;
    }
    h = h * std::min(std::max(0.84 * std::pow(tol / r, 0.25), 0.1), 4.0);
    if (h > hmax) h = hmax;
    else if (h < hmin) return -5;
  }
  return 1;
}

bool finite_n(const double* y, int n) {
  for (int i = 0; i < n; ++i)
    if (!std::isfinite(y[i])) return false;
  return true;
}

}  // namespace

extern "C" {

int orc_integrate_particle(const orc_field* f, const orc_config* c, int method, double mass,
                           double charge, double gm, double* x, double* y6, double xend,
                           double beta, int64_t* counters4) {
  auto rhs = [&](double t, const double* Y, double* o) { orc_particle_rhs(f, c, mass, charge, gm, t, Y, o); };
  Counters cnt;
  cnt.stop_nan = f->model == ORC_GRID;
  int idid;
  if (method == 0) idid = dop853(rhs, 6, *x, y6, xend, c->rtol, c->atol, c->nsteps, cnt, beta);
  else if (method == 1) idid = dopri5(rhs, 6, *x, y6, xend, c->rtol, c->atol, c->nsteps, cnt);
  else idid = rkf45(rhs, 6, *x, y6, xend, c->rkf_tol, xend - *x, c->rkf_hmin, cnt, 1000000);
  counters4[0] = cnt.nfcn; counters4[1] = cnt.nstep; counters4[2] = cnt.naccpt; counters4[3] = cnt.nrejct;
  return idid;
}

int orc_integrate_gc(const orc_field* f, const orc_config* c, int method, double mass,
                     double charge, double mu, double v, double* x, double* y4, double xend,
                     int64_t* counters4) {
  auto rhs = [&](double t, const double* Y, double* o) { orc_gc_rhs(f, c, c->gc_eom, mass, charge, mu, v, t, Y, o); };
  Counters cnt;
  cnt.stop_nan = f->model == ORC_GRID;
  int idid;
  if (method == 0) idid = dop853(rhs, 4, *x, y4, xend, c->rtol, c->atol, c->nsteps, cnt, 0.0);
  else if (method == 1) idid = dopri5(rhs, 4, *x, y4, xend, c->rtol, c->atol, c->nsteps, cnt);
  else idid = rkf45(rhs, 4, *x, y4, xend, c->rkf_tol, xend - *x, c->rkf_hmin, cnt, 1000000);
  counters4[0] = cnt.nfcn; counters4[1] = cnt.nstep; counters4[2] = cnt.naccpt; counters4[3] = cnt.nrejct;
  return idid;
}

// ---------------------------------------------------------------- constructors
void orc_particle_new(const double* pos, const double* vel, double t0, double mass, double charge,
                      orc_tracer* o) {
  // Particle.__init__, rapt/Particle.py:95-109
  std::memset(o, 0, sizeof(*o));
  o->mode = 0;
  o->mass = mass;
  o->charge = charge;
  o->t = t0;
  o->tcur = t0;
  const double gamma = 1 / std::sqrt(1 - dot3(vel, vel) / (kC * kC));
  for (int i = 0; i < 3; ++i) { o->s[i] = pos[i]; o->s[3 + i] = mass * gamma * vel[i]; }
}

static double magnetic_moment(const orc_field* f, double t, const double* pos, double vpar, double v,
                              double mass) {
  // rapt/utils.py:189-216
  const double gamma = 1.0 / std::sqrt(1 - std::pow(v / kC, 2));
  double tpos[4] = {t, pos[0], pos[1], pos[2]};
  const double Bmag = orc_magB(f, tpos);
  return gamma * gamma * mass * (v - vpar) * (v + vpar) / (2 * Bmag);
}

static void gc_new_ppar(const orc_field* f, const double* pos, double v, double ppar, double t0,
                        double mass, double charge, orc_tracer* o) {
  // GuidingCenter.__init__ with ppar given, rapt/GuidingCenter.py:108-133
  std::memset(o, 0, sizeof(*o));
  o->mode = 1;
  o->mass = mass; o->charge = charge; o->v = v;
  o->t = t0; o->tcur = t0;
  const double gamma = 1 / std::sqrt(1 - std::pow(v / kC, 2));
  o->mu = magnetic_moment(f, t0, pos, ppar / (mass * gamma), v, mass);
  o->s[0] = pos[0]; o->s[1] = pos[1]; o->s[2] = pos[2]; o->s[3] = ppar;
}

void orc_gc_new_pa(const orc_field* f, const double* pos, double v, double pa, double t0,
                   double mass, double charge, orc_tracer* o) {
  // rapt/GuidingCenter.py:123-133
  const double gamma = 1 / std::sqrt(1 - std::pow(v / kC, 2));
  const double vpar = (pa == 90) ? 0.0 : v * std::cos(pa * kPi / 180);
  const double ppar = gamma * mass * vpar;
  gc_new_ppar(f, pos, v, ppar, t0, mass, charge, o);
}

int orc_guidingcenter(const orc_field* f, double t, const double* r, const double* v, double mass,
                      double charge, double* gc3, double* vp, double* speed) {
  // rapt/utils.py:251-326, tol 1e-3, maxiter 20
  auto gyrovector = [&](const double* rr, double* o) {
    const double vsq = dot3(v, v);
    const double gamma = 1 / std::sqrt(1 - vsq / (kC * kC));
    double tpos[4] = {t, rr[0], rr[1], rr[2]};
    double B[3];
    orc_B(f, tpos, B);
    const double Bsq = dot3(B, B);
    const double s = gamma * mass / (charge * Bsq);
    double Bxv[3];
    cross3(B, v, Bxv);
    for (int i = 0; i < 3; ++i) o[i] = s * Bxv[i];
  };
  double g[3], old[3], cur[3];
  gyrovector(r, g);
  for (int i = 0; i < 3; ++i) old[i] = r[i] - g[i];
  for (int it = 1; it <= 20; ++it) {
    gyrovector(old, g);
    for (int i = 0; i < 3; ++i) cur[i] = r[i] - g[i];
    double d[3] = {cur[0] - old[0], cur[1] - old[1], cur[2] - old[2]};
    if (std::sqrt(dot3(d, d)) / std::sqrt(dot3(cur, cur)) < 1e-3) {
      double tpos[4] = {t, cur[0], cur[1], cur[2]};
      double B[3];
      orc_B(f, tpos, B);
      *vp = dot3(v, B) / std::sqrt(dot3(B, B));
      *speed = std::sqrt(dot3(v, v));
      gc3[0] = cur[0]; gc3[1] = cur[1]; gc3[2] = cur[2];
      return 0;
    }
    for (int i = 0; i < 3; ++i) old[i] = cur[i];
  }
  return -1;  // reference prints and returns None (utils.py:326)
}

static void getperp(const double* v, double* o) {  // rapt/utils.py:328-374
  if (v[0] == 0) { o[0] = 1; o[1] = 0; o[2] = 0; return; }
  if (v[1] == 0) { o[0] = 0; o[1] = 1; o[2] = 0; return; }
  if (v[2] == 0) { o[0] = 0; o[1] = 0; o[2] = 1; return; }
  const double cc = -1.0 * (v[0] + v[1]) / v[2];
  const double n = std::sqrt(2 + cc * cc);
  o[0] = 1 / n; o[1] = 1 / n; o[2] = cc / n;
}

void orc_gctofp(const orc_field* f, double t, const double* R, double vp, double speed, double mass,
                double charge, double gyrophase, double* pos, double* vel) {
  // rapt/utils.py:376-433
  double tpos[4] = {t, R[0], R[1], R[2]};
  double B[3];
  orc_B(f, tpos, B);
  const double Bsq = dot3(B, B);
  const double bn = std::sqrt(Bsq);
  const double b[3] = {B[0] / bn, B[1] / bn, B[2] / bn};
  const double pa = std::acos(vp / speed);
  // cyclotron_radius2, rapt/utils.py:147-187
  const double gamma = 1.0 / std::sqrt(1 - std::pow(speed / kC, 2));
  const double vperp = std::sqrt((speed - vp) * (speed + vp));
  const double rc = gamma * mass * vperp / (std::fabs(charge) * bn);
  double u[3];
  getperp(B, u);
  const double un = std::sqrt(dot3(u, u));
  for (int i = 0; i < 3; ++i) u[i] = u[i] / un;
  double w[3];
  cross3(b, u, w);
  const double s = sgn(charge);
  const double cg = std::cos(gyrophase), sg = std::sin(gyrophase);
  const double cp = std::cos(pa), sp = std::sin(pa);
  for (int i = 0; i < 3; ++i) {
    pos[i] = R[i] + rc * (cg * u[i] + sg * w[i]);
    vel[i] = speed * (cp * b[i] + s * sp * sg * u[i] - s * sp * cg * w[i]);
  }
}

int orc_gc_from_particle(const orc_field* f, const orc_tracer* p, orc_tracer* o) {
  // GuidingCenter.init(Particle), rapt/GuidingCenter.py:168-187
  const double* mom = p->s + 3;
  const double gm = std::sqrt(p->mass * p->mass + dot3(mom, mom) / (kC * kC));
  const double vel[3] = {mom[0] / gm, mom[1] / gm, mom[2] / gm};
  double gc[3], vp, v;
  if (orc_guidingcenter(f, p->t, p->s, vel, p->mass, p->charge, gc, &vp, &v) != 0) return -1;
  const double gamma = 1 / std::sqrt(1 - std::pow(v / kC, 2));
  gc_new_ppar(f, gc, v, p->mass * gamma * vp, p->t, p->mass, p->charge, o);
  return 0;
}

void orc_particle_from_gc(const orc_field* f, const orc_tracer* g, orc_tracer* o) {
  // Particle.init(GuidingCenter), rapt/Particle.py:149-164. GCtoFP is called
  // with the new, empty Particle's tcur, i.e. t = 0 (quirk kept).
  double tpos[4] = {g->t, g->s[0], g->s[1], g->s[2]};
  const double B = orc_magB(f, tpos);
  const double ppar = g->s[3];
  const double gammasq = 1 + 2 * g->mu * B / (g->mass * kC * kC) + std::pow(ppar / g->mass / kC, 2);
  double v;
  if (std::sqrt(gammasq) - 1 < 1e-6) v = std::sqrt(2 * g->mu * B / g->mass + std::pow(ppar / g->mass, 2));
  else v = kC * std::sqrt(1 - 1 / gammasq);
  const double vpar = ppar / g->mass / std::sqrt(gammasq);
  double pos[3], vel[3];
  orc_gctofp(f, 0.0, g->s, vpar, v, g->mass, g->charge, 0.0, pos, vel);
  orc_particle_new(pos, vel, g->t, g->mass, g->charge, o);
}

// ---------------------------------------------------------------- adiabaticity
static double particle_cycper(const orc_field* f, const orc_tracer* p) {
  // Particle.cycper -> utils.cyclotron_period, rapt/Particle.py:489-494, utils.py:62-66
  const double* mom = p->s + 3;
  const double gm = std::sqrt(p->mass * p->mass + dot3(mom, mom) / (kC * kC));
  const double v[3] = {mom[0] / gm, mom[1] / gm, mom[2] / gm};
  const double gamma = 1.0 / std::sqrt(1 - dot3(v, v) / (kC * kC));
  double tpos[4] = {p->t, p->s[0], p->s[1], p->s[2]};
  const double B = orc_magB(f, tpos);
  return 2 * kPi * gamma * p->mass / B / std::fabs(p->charge);
}

int orc_particle_isadiabatic(const orc_field* f, const orc_config* c, const orc_tracer* p) {
  // rapt/Particle.py:345-384
  const double* mom = p->s + 3;
  const double gm = std::sqrt(p->mass * p->mass + dot3(mom, mom) / (kC * kC));
  const double v[3] = {mom[0] / gm, mom[1] / gm, mom[2] / gm};
  double tpos[4] = {p->t, p->s[0], p->s[1], p->s[2]};
  // cyclotron_radius, rapt/utils.py:141-145
  const double vsq = dot3(v, v);
  const double gamma = 1.0 / std::sqrt(1 - vsq / (kC * kC));
  double B[3];
  orc_B(f, tpos, B);
  const double Bmag = std::sqrt(dot3(B, B));
  const double vpar = dot3(v, B) / Bmag;
  const double vperp = std::sqrt(vsq - vpar * vpar);
  const double cycrad = gamma * p->mass * vperp / (std::fabs(p->charge) * Bmag);
  const bool sp = cycrad / orc_lengthscale(f, tpos) < c->epss;
  if (f->is_static) return sp;
  return sp && (particle_cycper(f, p) / orc_timescale(f, tpos) < c->epst);
}

int orc_gc_isadiabatic(const orc_field* f, const orc_config* c, const orc_tracer* g) {
  // rapt/GuidingCenter.py:287-327 with cycrad :517-530 and cycper :532-541
  double tpos[4] = {g->t, g->s[0], g->s[1], g->s[2]};
  const double pp = g->s[3], m = g->mass;
  const double Bmag = orc_magB(f, tpos);
  double gamma = std::sqrt(1 + 2 * g->mu * Bmag / (m * kC * kC) + std::pow(pp / m / kC, 2));
  double vp, v;
  if (gamma - 1 < 1e-6) { vp = pp / m; v = std::sqrt(2 * g->mu * Bmag / m + vp * vp); }
  else { vp = pp / m / gamma; v = kC * std::sqrt(1 - 1 / (gamma * gamma)); }
  double B[3];
  orc_B(f, tpos, B);
  const double Bm2 = std::sqrt(dot3(B, B));
  const double g2 = 1.0 / std::sqrt(1 - std::pow(v / kC, 2));
  const double cycrad = g2 * m * std::sqrt((v - vp) * (v + vp)) / (std::fabs(g->charge) * Bm2);
  const bool sp = cycrad / orc_lengthscale(f, tpos) < c->epss;
  if (f->is_static) return sp;
  if (!sp) return 0;
  // GuidingCenter.cycper squares ppar without dividing by m c (:535): kept.
  gamma = std::sqrt(1 + 2 * g->mu * Bmag / (m * kC * kC) + pp * pp);
  double v2;
  if (gamma - 1 < 1e-6) { const double vp2 = pp / m; v2 = std::sqrt(2 * g->mu * Bmag / m + vp2 * vp2); }
  else v2 = kC * std::sqrt(1 - 1 / (gamma * gamma));
  const double g3 = 1.0 / std::sqrt(1 - std::pow(v2 / kC, 2));
  const double cycper = 2 * kPi * g3 * m / Bmag / std::fabs(g->charge);
  return cycper / orc_timescale(f, tpos) < c->epst;
}

// ---------------------------------------------------------------- tracer advance
static void put_row(double* rows, int max_rows, int* nrows, double t, const double* s, int ns) {
  if (!rows || *nrows >= max_rows) { ++*nrows; return; }
  double* r = rows + 7 * (size_t)(*nrows);
  r[0] = t;
  for (int i = 0; i < 6; ++i) r[1 + i] = (i < ns) ? s[i] : 0.0;
  ++*nrows;
}

int orc_particle_advance(const orc_field* f, const orc_config* c, orc_tracer* p, double delta,
                         int check_adiabaticity, double* rows, int max_rows, int* nrows) {
  // Particle.advance, rapt/Particle.py:230-309
  const double t0 = p->t;
  const double* mom = p->s + 3;
  const double gm = std::sqrt(p->mass * p->mass + dot3(mom, mom) / (kC * kC));
  // dt from utils.cyclotron_period at the start state (Particle.py:282; the
  // Ptimestep branch at :277-280 is overwritten and has no effect).
  const double dt = particle_cycper(f, p) / c->cycres;
  double rt = p->t;
  double y[6];
  std::memcpy(y, p->s, sizeof(y));
  bool ok = true;
  int64_t guard = 0;
  while (ok && rt < t0 + delta) {
    if (++guard > 100000000) { p->status = ORC_ST_MAXSTEPS; break; }
    const double rowt = rt + dt;
    int64_t cnt[4];
    const int method = (c->tableau == 1) ? 2 : 0;
    const int idid = orc_integrate_particle(f, c, method, p->mass, p->charge, gm, &rt, y, rt + dt, 0.1, cnt);
    p->nfcn += cnt[0]; p->nstep += cnt[1]; p->naccept += cnt[2]; p->nreject += cnt[3];
    if (idid == -6 || idid == -5) {
      // Grid: the reference raises ValueError inside r.integrate(); RKF45: rkf.py
      // raises RuntimeError at hmin (rkf.py:136-139). No row, state kept.
      p->status = idid == -6 ? ORC_ST_OUT_OF_GRID : ORC_ST_RKF_HMIN;
      break;
    }
    if (idid < 0) {
      ok = false;
      p->status = (idid == -2) ? ORC_ST_MAXSTEPS : (idid == -3) ? ORC_ST_HMIN : (idid == -6) ? ORC_ST_OUT_OF_GRID : ORC_ST_RKF_HMIN;
    }
    if (!finite_n(y, 6)) { p->status = ORC_ST_NONFINITE; ok = false; }
    p->t = rowt;
    std::memcpy(p->s, y, sizeof(y));
    p->tcur = rt + dt;  // Particle.py:306: tcur runs one dt ahead (quirk kept)
    put_row(rows, max_rows, nrows, rowt, y, 6);
    if (check_adiabaticity && orc_particle_isadiabatic(f, c, p)) return 1;
  }
  return 0;
}

// Dense-output guiding-centre advance (no reference counterpart; the option
// rapt_config.dense_output of the GPU library): one DOPRI5 integration through
// the whole call with hmax = 16 output intervals, rows at the reference's output times from the
// order-4 continuous extension of the step that covers each (Hairer, Norsett &
// Wanner, Solving ODEs I, II.6, the DOPRI5 code's CONTD5 coefficients), the
// adiabaticity check on each row, and the call ending in the last row's state.
static int gc_advance_dense(const orc_field* f, const orc_config* c, orc_tracer* g, double delta, double dt,
                            int check_adiabaticity, double* rows, int max_rows, int* nrows) {
  const double a21 = 0.2, a31 = 3.0 / 40.0, a32 = 9.0 / 40.0;
  const double a41 = 44.0 / 45.0, a42 = -56.0 / 15.0, a43 = 32.0 / 9.0;
  const double a51 = 19372.0 / 6561.0, a52 = -25360.0 / 2187.0, a53 = 64448.0 / 6561.0, a54 = -212.0 / 729.0;
  const double a61 = 9017.0 / 3168.0, a62 = -355.0 / 33.0, a63 = 46732.0 / 5247.0, a64 = 49.0 / 176.0,
               a65 = -5103.0 / 18656.0;
  const double a71 = 35.0 / 384.0, a73 = 500.0 / 1113.0, a74 = 125.0 / 192.0, a75 = -2187.0 / 6784.0,
               a76 = 11.0 / 84.0;
  const double e1 = 71.0 / 57600.0, e3 = -71.0 / 16695.0, e4 = 71.0 / 1920.0, e5 = -17253.0 / 339200.0,
               e6 = 22.0 / 525.0, e7 = -1.0 / 40.0;
  const double d1 = -12715105075.0 / 11282082432.0, d3 = 87487479700.0 / 32700410799.0,
               d4 = -10690763975.0 / 1880347072.0, d5 = 701980252875.0 / 199316789632.0,
               d6 = -1453857185.0 / 822651844.0, d7 = 69997945.0 / 29380423.0;
  const double beta = 0.04, safe = 0.9, expo1 = 0.2 - beta * 0.75, facc1 = 5.0, facc2 = 0.1;
  const double uround = 2.3e-16;
  auto F = [&](double t, const double* Y, double* o) {
    orc_gc_rhs(f, c, c->gc_eom, g->mass, g->charge, g->mu, g->v, t, Y, o);
  };
  const int n = 4;
  const double stop = g->t + delta;
  double t_row = g->t, rt = g->t, y[4], k1[4];
  std::memcpy(y, g->s, sizeof(y));
  if (!(t_row < stop)) return 0;
  F(rt, y, k1);
  const double hmax = 16 * dt;
  double h = hinit(F, n, rt, y, 1.0, k1, 5, hmax, c->atol, c->rtol);
  g->nfcn += 2;
  double facold = 1e-4;
  bool reject = false;
  int nst = 0;
  for (int64_t guard = 0; guard < 100000000; ++guard) {
    if (nst > c->nsteps || 0.1 * std::fabs(h) <= std::fabs(rt) * uround) {
      g->status = nst > c->nsteps ? ORC_ST_MAXSTEPS : ORC_ST_HMIN;
      g->t = rt; g->tcur = rt;
      std::memcpy(g->s, y, sizeof(y));
      put_row(rows, max_rows, nrows, rt, y, 4);
      return 0;
    }
    ++nst;
    g->nstep++;
    double k2[4], k3[4], k4[4], k5[4], k6[4], k7[4], y1[4], yt[4];
    for (int i = 0; i < n; ++i) yt[i] = y[i] + h * (a21 * k1[i]);
    F(rt + 0.2 * h, yt, k2);
    for (int i = 0; i < n; ++i) yt[i] = y[i] + h * (a31 * k1[i] + a32 * k2[i]);
    F(rt + 0.3 * h, yt, k3);
    for (int i = 0; i < n; ++i) yt[i] = y[i] + h * (a41 * k1[i] + a42 * k2[i] + a43 * k3[i]);
    F(rt + 0.8 * h, yt, k4);
    for (int i = 0; i < n; ++i) yt[i] = y[i] + h * (a51 * k1[i] + a52 * k2[i] + a53 * k3[i] + a54 * k4[i]);
    F(rt + (8.0 / 9.0) * h, yt, k5);
    for (int i = 0; i < n; ++i)
      yt[i] = y[i] + h * (a61 * k1[i] + a62 * k2[i] + a63 * k3[i] + a64 * k4[i] + a65 * k5[i]);
    F(rt + h, yt, k6);
    for (int i = 0; i < n; ++i) y1[i] = y[i] + h * (a71 * k1[i] + a73 * k3[i] + a74 * k4[i] + a75 * k5[i] + a76 * k6[i]);
    F(rt + h, y1, k7);
    g->nfcn += 6;
    double err = 0, dd[4];
    for (int i = 0; i < n; ++i) {
      const double ei = (e1 * k1[i] + e3 * k3[i] + e4 * k4[i] + e5 * k5[i] + e6 * k6[i] + e7 * k7[i]) * h;
      const double sk = c->atol + c->rtol * std::max(std::fabs(y[i]), std::fabs(y1[i]));
      err += (ei / sk) * (ei / sk);
      dd[i] = h * (d1 * k1[i] + d3 * k3[i] + d4 * k4[i] + d5 * k5[i] + d6 * k6[i] + d7 * k7[i]);
    }
    err = std::sqrt(err / n);
    if (f->model == ORC_GRID && std::isnan(err)) {  // the reference raises ValueError: no row
      g->status = ORC_ST_OUT_OF_GRID;
      return 0;
    }
    const double fac11 = std::pow(err, expo1);
    double fac = fac11 / std::pow(facold, beta);
    fac = std::max(facc2, std::min(facc1, fac / safe));
    double hnew = h / fac;
    if (err <= 1.0) {
      facold = std::max(err, 1.0e-4);
      g->naccept++;
      const double told = rt, hs = h;
      rt = rt + h;
      if (std::fabs(hnew) > hmax) hnew = hmax;
      if (reject) hnew = std::min(std::fabs(hnew), std::fabs(h));
      reject = false;
      h = hnew;
      for (int r = 0; r <= 16; ++r) {
        const double tn = t_row + dt;
        if (!(tn <= rt)) break;
        const double th = (tn - told) / hs, th1 = 1.0 - th;
        double yr[4];
        for (int i = 0; i < n; ++i) {
          const double ydiff = y1[i] - y[i];
          const double bspl = hs * k1[i] - ydiff;
          const double r4 = ydiff - hs * k7[i] - bspl;
          yr[i] = y[i] + th * (ydiff + th1 * (bspl + th * (r4 + th1 * dd[i])));
        }
        t_row = tn;
        nst = 0;
        put_row(rows, max_rows, nrows, tn, yr, 4);
        g->t = tn; g->tcur = tn;
        std::memcpy(g->s, yr, sizeof(yr));
        if (check_adiabaticity && finite_n(yr, 4) && !orc_gc_isadiabatic(f, c, g)) return 1;
        if (!(t_row < stop)) {
          if (!finite_n(yr, 4)) g->status = ORC_ST_NONFINITE;
          return 0;
        }
      }
      std::memcpy(k1, k7, sizeof(k1));
      std::memcpy(y, y1, sizeof(y));
      if (!finite_n(y, 4)) {
        g->status = ORC_ST_NONFINITE;
        return 0;
      }
    } else {
      hnew = h / std::min(facc1, fac11 / safe);
      reject = true;
      g->nreject++;
      h = hnew;
    }
  }
  g->status = ORC_ST_MAXSTEPS;
  return 0;
}

int orc_gc_advance(const orc_field* f, const orc_config* c, orc_tracer* g, double delta,
                   int check_adiabaticity, double* rows, int max_rows, int* nrows) {
  // GuidingCenter.advance, rapt/GuidingCenter.py:397-458 (dopri5 at :450)
  // cadence: GCtimestep, or the bounce period at the current state / bounceresolution (:443-446)
  const double dt = c->gctimestep != 0 ? c->gctimestep : orc_gc_bounceperiod(f, g, c->flres, c->bounce_quad) / c->bounceres;
  if (!(dt > 0) || !std::isfinite(dt)) { g->status = ORC_ST_BAD_INPUT; return 0; }
  if (c->dense) return gc_advance_dense(f, c, g, delta, dt, check_adiabaticity, rows, max_rows, nrows);
  const double t0 = g->t;
  double rt = g->t;
  double y[4];
  std::memcpy(y, g->s, sizeof(y));
  bool ok = true;
  int64_t guard = 0;
  while (ok && rt < t0 + delta) {
    if (++guard > 100000000) { g->status = ORC_ST_MAXSTEPS; break; }
    int64_t cnt[4];
    const int method = (c->tableau == 1) ? 2 : 1;
    const int idid = orc_integrate_gc(f, c, method, g->mass, g->charge, g->mu, g->v, &rt, y, rt + dt, cnt);
    g->nfcn += cnt[0]; g->nstep += cnt[1]; g->naccept += cnt[2]; g->nreject += cnt[3];
    if (idid == -6 || idid == -5) {
      // Grid: the reference raises ValueError inside r.integrate(); RKF45: rkf.py
      // raises RuntimeError at hmin (rkf.py:136-139). No row, state kept.
      g->status = idid == -6 ? ORC_ST_OUT_OF_GRID : ORC_ST_RKF_HMIN;
      break;
    }
    if (idid < 0) {
      ok = false;
      g->status = (idid == -2) ? ORC_ST_MAXSTEPS : (idid == -3) ? ORC_ST_HMIN : (idid == -6) ? ORC_ST_OUT_OF_GRID : ORC_ST_RKF_HMIN;
    }
    if (!finite_n(y, 4)) { g->status = ORC_ST_NONFINITE; ok = false; }
    g->t = rt;
    std::memcpy(g->s, y, sizeof(y));
    g->tcur = rt;
    put_row(rows, max_rows, nrows, rt, y, 4);
    if (check_adiabaticity && !orc_gc_isadiabatic(f, c, g)) return 1;
  }
  return 0;
}

// ---------------------------------------------------------------- BounceCenter
double orc_bc_mu(const orc_field* f, const double* pos, double v, double pa, double t0, double mass) {
  // BounceCenter.__init__, rapt/BounceCenter.py:100-104: the parallel speed is
  // v cos(pa) with pa in degrees handed to np.cos as radians (kept)
  return magnetic_moment(f, t0, pos, v * std::cos(pa), v, mass);
}

void orc_bc_rhs(const orc_field* f, const double* tpos, double mass, double charge, double v, double Bm, double d,
                double flres, int quad, double* o) {
  // BounceCenter.advance deriv (BounceCenter.py:236-245), the non-equatorial
  // branch: gamma m v^2 / (q S_b B^2) (grad I x B)
  const double gamma = 1.0 / std::sqrt(1 - (v / kC) * (v / kC));
  double B[3], gI[3];
  orc_B(f, tpos, B);
  const double magBsq = dot3(B, B);
  const double Sb = orc_halfbouncepath(f, tpos, Bm, flres, quad, nullptr);
  orc_gradI(f, tpos, Bm, d, flres, quad, gI);
  const double k = gamma * mass * v * v / (charge * Sb * magBsq);
  o[0] = k * (gI[1] * B[2] - gI[2] * B[1]);
  o[1] = k * (gI[2] * B[0] - gI[0] * B[2]);
  o[2] = k * (gI[0] * B[1] - gI[1] * B[0]);
}

int orc_bc_advance(const orc_field* f, const orc_config* c, double* state, double v, double mu, double mass,
                   double charge, double delta, double bctimestep, double d, int quad, double* rows, int max_rows,
                   int* nrows, int64_t* counters4) {
  // BounceCenter.advance, rapt/BounceCenter.py:214-252: cadence BCtimestep x the
  // bounce period at the start; rows stamped with np.arange(tcur, tcur + delta,
  // dt), i.e. each row carries the time its interval began (kept); one SciPy
  // dopri5 restart per row
  const double gamma = 1.0 / std::sqrt(1 - (v / kC) * (v / kC));
  const double Bm = mass * (gamma * gamma) * (v * v) / (2 * mu);
  double tpos[4] = {state[0], state[1], state[2], state[3]};
  const double bp = (2 / v) * orc_halfbouncepath(f, tpos, Bm, c->flres, quad, nullptr);
  const double dt = bctimestep * bp;
  if (!(dt > 0) || !std::isfinite(dt)) return ORC_ST_FIELDLINE;
  const double tcur = state[4];
  const int64_t K = (int64_t)std::ceil(((tcur + delta) - tcur) / dt);
  const double dstep = (tcur + dt) - tcur;
  auto rhs = [&](double t, const double* Y, double* o) {
    const double tp[4] = {t, Y[0], Y[1], Y[2]};
    orc_bc_rhs(f, tp, mass, charge, v, Bm, d, c->flres, quad, o);
  };
  double rt = state[0], y[3] = {state[1], state[2], state[3]};
  int status = ORC_ST_OK;
  for (int64_t k = 0; k < K; ++k) {
    const double tk = k == 0 ? tcur : (k == 1 ? tcur + dt : tcur + (double)k * dstep);
    Counters cnt;
    const int idid = dopri5(rhs, 3, rt, y, rt + dt, c->rtol, c->atol, c->nsteps, cnt);
    counters4[0] += cnt.nfcn; counters4[1] += cnt.nstep; counters4[2] += cnt.naccpt; counters4[3] += cnt.nrejct;
    if (idid < 0) status = idid == -2 ? ORC_ST_MAXSTEPS : ORC_ST_HMIN;
    if (!finite_n(y, 3)) status = ORC_ST_NONFINITE;
    put_row(rows, max_rows, nrows, tk, y, 3);
    state[0] = tk; state[1] = y[0]; state[2] = y[1]; state[3] = y[2]; state[4] = tk;
    if (status != ORC_ST_OK) break;
  }
  return status;
}

int orc_adaptive_init(const orc_field* f, const orc_config* c, const double* pos, const double* vel,
                      double t0, double mass, double charge, orc_tracer* out) {
  // Adaptive.__init__, rapt/Adaptive.py:70-104
  orc_tracer p;
  orc_particle_new(pos, vel, t0, mass, charge, &p);
  if (orc_particle_isadiabatic(f, c, &p)) {
    if (orc_gc_from_particle(f, &p, out) != 0) { *out = p; out->status = ORC_ST_GC_NOCONV; return -1; }
    return 1;
  }
  *out = p;
  return 0;
}

int orc_adaptive_advance(const orc_field* f, const orc_config* c, orc_tracer* cur, double delta,
                         double* rows, int8_t* row_mode, int max_rows, int* nrows, double* sw_time,
                         int8_t* sw_mode, int max_sw, int* nsw) {
  // Adaptive.advance, rapt/Adaptive.py:187-222. t is the absolute tcur of the
  // current tracer compared with the relative delta (correct for t0 = 0; kept).
  double t = 0;
  int guard = 0;
  while (t < delta) {
    if (++guard > 100000) { cur->status = ORC_ST_ADAPTIVE_LIMIT; return -1; }
    const int before = *nrows;
    int raised;
    if (cur->mode == 0) raised = orc_particle_advance(f, c, cur, delta - t, 1, rows, max_rows, nrows);
    else raised = orc_gc_advance(f, c, cur, delta - t, 1, rows, max_rows, nrows);
    if (row_mode)
      for (int i = before; i < *nrows && i < max_rows; ++i) row_mode[i] = (int8_t)cur->mode;
    if (cur->status != ORC_ST_OK && !raised) {
      // The reference would re-enter advance() with the same state; a failed
      // integrator makes no progress there, so stop with the status set.
      return -1;
    }
    if (raised) {
      orc_tracer nxt;
      const int64_t a = cur->naccept, r = cur->nreject, fc = cur->nfcn, ns = cur->nstep;
      if (cur->mode == 1) {
        orc_particle_from_gc(f, cur, &nxt);
      } else if (orc_gc_from_particle(f, cur, &nxt) != 0) {
        cur->status = ORC_ST_GC_NOCONV;
        return -1;
      }
      nxt.naccept = a; nxt.nreject = r; nxt.nfcn = fc; nxt.nstep = ns;
      *cur = nxt;
      if (*nsw < max_sw && sw_time) { sw_time[*nsw] = cur->tcur; sw_mode[*nsw] = (int8_t)cur->mode; }
      ++*nsw;
      // first row of the new segment (its trajectory[0])
      const int b2 = *nrows;
      put_row(rows, max_rows, nrows, cur->t, cur->s, cur->mode == 0 ? 6 : 4);
      if (row_mode && b2 < max_rows) row_mode[b2] = (int8_t)cur->mode;
    }
    t = cur->tcur;
  }
  return 0;
}

void orc_batch_advance(const orc_field* f, const orc_config* c, int kind, int64_t n, orc_tracer* tr,
                       const double* delta, int nthreads) {
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
  for (int64_t i = 0; i < n; ++i) {
    int nrows = 0, nsw = 0;
    if (kind == 0) orc_particle_advance(f, c, &tr[i], delta[i], 0, nullptr, 0, &nrows);
    else if (kind == 1) orc_gc_advance(f, c, &tr[i], delta[i], 0, nullptr, 0, &nrows);
    else orc_adaptive_advance(f, c, &tr[i], delta[i], nullptr, nullptr, 0, &nrows, nullptr, nullptr, 0, &nsw);
  }
}

}  // extern "C"
