// fields.cuh -- analytic E/B field models on the device (rapt/fields.py).
//
// Each model is a compile-time specialisation so that the stepper kernels are
// instantiated per model with no runtime dispatch in the right-hand side.
// Powers of r use one FP64 rsqrt instead of the reference's pow(r2, 2.5) and
// division (same quantity, different rounding: a few ulp).
//
// Values that feed a central difference (field components, |B|, unit vectors)
// end in an explicitly rounded multiply (__dmul_rn): otherwise the compiler may
// fuse the last product into the difference, which then sees the unrounded
// product and no longer takes the difference of two field values as the
// reference's scheme does (a constant field would get a nonzero gradient).
#pragma once
#include "common.cuh"

namespace rapt {

template <int M>
struct Field;

// EarthDipole, fields.py:282-317: B = -3 B0 Re^3 / r^5 (xz, yz, z^2 - r^2/3).
// c0 = -3 B0 Re^3.
template <>
struct Field<RAPT_EARTH_DIPOLE> {
  static constexpr bool kStatic = true;
  __device__ __forceinline__ static void B(const FieldP& f, double, double x, double y, double z, double* o) {
    const double r2 = x * x + y * y + z * z;
    const double ri = rsqrt(r2);
    const double ri2 = ri * ri;
    const double s = f.c0 * (ri2 * ri2 * ri);
    o[0] = __dmul_rn(s, x * z);
    o[1] = __dmul_rn(s, y * z);
    o[2] = __dmul_rn(s, z * z - r2 * (1.0 / 3.0));
  }
  __device__ __forceinline__ static void E(const FieldP&, double, double, double, double, double* o) {
    o[0] = o[1] = o[2] = 0.0;
  }
};

// DoubleDipole, fields.py:319-362: two parallel dipoles, the image at x = distance
// with relative strength k. c0 = -B0 Re^3, p[1] = distance, p[2] = k.
template <>
struct Field<RAPT_DOUBLE_DIPOLE> {
  static constexpr bool kStatic = true;
  __device__ __forceinline__ static void B(const FieldP& f, double, double x, double y, double z, double* o) {
    const double yz2 = y * y + z * z;
    const double r2a = x * x + yz2;
    const double ia = rsqrt(r2a);
    const double ia2 = ia * ia;
    const double sa = ia2 * ia2 * ia;
    const double x2 = x - f.p[1];
    const double r2b = x2 * x2 + yz2;
    const double ib = rsqrt(r2b);
    const double ib2 = ib * ib;
    const double sb = f.p[2] * (ib2 * ib2 * ib);
    const double tz = 3.0 * z;
    const double zz2 = 2.0 * z * z;
    o[0] = __dmul_rn(f.c0, tz * (x * sa + x2 * sb));
    o[1] = __dmul_rn(f.c0, tz * y * (sa + sb));
    o[2] = __dmul_rn(f.c0, (zz2 - x * x - y * y) * sa + (zz2 - x2 * x2 - y * y) * sb);
  }
  __device__ __forceinline__ static void E(const FieldP&, double, double, double, double, double* o) {
    o[0] = o[1] = o[2] = 0.0;
  }
};

// UniformBz, fields.py:364-390.
template <>
struct Field<RAPT_UNIFORM_BZ> {
  static constexpr bool kStatic = true;
  __device__ __forceinline__ static void B(const FieldP& f, double, double, double, double, double* o) {
    o[0] = 0.0; o[1] = 0.0; o[2] = f.p[0];
  }
  __device__ __forceinline__ static void E(const FieldP&, double, double, double, double, double* o) {
    o[0] = o[1] = o[2] = 0.0;
  }
};

// UniformCrossedEB, fields.py:392-427: E = (0, Ey, 0), B = (0, 0, Bz); static = False.
template <>
struct Field<RAPT_UNIFORM_CROSSED_EB> {
  static constexpr bool kStatic = false;
  __device__ __forceinline__ static void B(const FieldP& f, double, double, double, double, double* o) {
    o[0] = 0.0; o[1] = 0.0; o[2] = f.p[1];
  }
  __device__ __forceinline__ static void E(const FieldP& f, double, double, double, double, double* o) {
    o[0] = 0.0; o[1] = f.p[0]; o[2] = 0.0;
  }
};

// VarEarthDipole, fields.py:429-470: dipole moment times (1 + amp sin(2 pi t / period)),
// induced E ignored as in the reference. c0 = -B0 Re^3, c1 = 2 pi / period.
template <>
struct Field<RAPT_VAR_EARTH_DIPOLE> {
  static constexpr bool kStatic = false;
  __device__ __forceinline__ static void B(const FieldP& f, double t, double x, double y, double z, double* o) {
    const double r2 = x * x + y * y + z * z;
    const double ri = rsqrt(r2);
    const double ri2 = ri * ri;
    const double s = f.c0 * (1.0 + f.p[0] * sin(f.c1 * t)) * (ri2 * ri2 * ri);
    o[0] = __dmul_rn(s, 3.0 * x * z);
    o[1] = __dmul_rn(s, 3.0 * y * z);
    o[2] = __dmul_rn(s, 2.0 * z * z - x * x - y * y);
  }
  __device__ __forceinline__ static void E(const FieldP&, double, double, double, double, double* o) {
    o[0] = o[1] = o[2] = 0.0;
  }
};

// Parabolic, fields.py:472-511: (B0 z/d, 0, Bn) for |z| <= 1, else
// (sign(z) * 3.07e-5, 0, Bn) -- the reference uses the module-level B0 there.
template <>
struct Field<RAPT_PARABOLIC> {
  static constexpr bool kStatic = true;
  __device__ __forceinline__ static void B(const FieldP& f, double, double, double, double z, double* o) {
    if (fabs(z) <= 1.0) o[0] = f.p[0] * z / f.p[2];
    else o[0] = (z > 0.0) ? kB0 : ((z < 0.0) ? -kB0 : 0.0);
    o[1] = 0.0;
    o[2] = f.p[1];
  }
  __device__ __forceinline__ static void E(const FieldP&, double, double, double, double, double* o) {
    o[0] = o[1] = o[2] = 0.0;
  }
};

// Harris current sheet with a normal component and a uniform dawn-dusk E:
// B = (B0 tanh(z/L), 0, Bn), E = (0, Ey, 0). Not in the reference. c0 = 1/L.
template <>
struct Field<RAPT_HARRIS> {
  static constexpr bool kStatic = false;
  __device__ __forceinline__ static void B(const FieldP& f, double, double, double, double z, double* o) {
    o[0] = __dmul_rn(f.p[0], tanh(z * f.c0));
    o[1] = 0.0;
    o[2] = f.p[2];
  }
  __device__ __forceinline__ static void E(const FieldP& f, double, double, double, double, double* o) {
    o[0] = 0.0; o[1] = f.p[3]; o[2] = 0.0;
  }
};

// Breathing dipole B0(t) = B0 (1 + amp sin(w t)) with its induced azimuthal E,
// E = -dB0/dt Re^3 (y, -x, 0) / r^3. Not in the reference.
// c0 = -B0 Re^3, c1 = w = 2 pi / period, c2 = B0 amp w Re^3.
template <>
struct Field<RAPT_COMPRESSED_DIPOLE> {
  static constexpr bool kStatic = false;
  __device__ __forceinline__ static void B(const FieldP& f, double t, double x, double y, double z, double* o) {
    const double r2 = x * x + y * y + z * z;
    const double ri = rsqrt(r2);
    const double ri2 = ri * ri;
    const double s = f.c0 * (1.0 + f.p[1] * sin(f.c1 * t)) * (ri2 * ri2 * ri);
    o[0] = __dmul_rn(s, 3.0 * x * z);
    o[1] = __dmul_rn(s, 3.0 * y * z);
    o[2] = __dmul_rn(s, 2.0 * z * z - x * x - y * y);
  }
  __device__ __forceinline__ static void E(const FieldP& f, double t, double x, double y, double z, double* o) {
    const double r2 = x * x + y * y + z * z;
    const double ri = rsqrt(r2);
    const double s = -f.c2 * cos(f.c1 * t) * (ri * ri * ri);
    o[0] = s * y;
    o[1] = -s * x;
    o[2] = 0.0;
  }
};

// Grid, fields.py:513-814 (Bgrid :707-738, Egrid :740-771): SciPy's
// RegularGridInterpolator, method "linear", over (t, x, y, z), or (x, y, z)
// for a single snapshot, restated from SciPy's _rgi.py _evaluate_linear and
// find_indices. Per axis the cell i with g[i] <= v < g[i+1] (the last cell for
// v == g[n-1]) and w = (v - g[i]) / (g[i+1] - g[i]); the 2^d corners in
// itertools.product order (last axis fastest), the lower corner weighted 1 - w
// and the upper w; a corner's weight is the running product over the axes, and
// the value is summed corner by corner from 0. Every product and sum is rounded
// on its own (no FMA), as numpy evaluates them, so values agree bit for bit.
// Outside the grid (or at a NaN coordinate) the reference raises ValueError
// from the interpolator's bounds check; here each component is NaN, which the
// steppers report as RAPT_ST_OUT_OF_GRID.
struct GridV {
  double a, b, c;
};

// Cell index and normalised distance on a strictly ascending axis, v in
// [g[0], g[n-1]]: the cell of a uniform axis is guessed from inv = (n-1) /
// (g[n-1] - g[0]) and checked against the axis values (so the cell is exactly
// the one SciPy's search finds); a wrong guess (non-uniform axis) falls back to
// a binary search.
__device__ __forceinline__ int grid_cell(const double* __restrict__ g, int n, double inv, double v, double& w) {
  const double g0 = __ldg(g);
  int i = min(max((int)((v - g0) * inv), 0), n - 2);
  double lo = __ldg(g + i), hi = __ldg(g + i + 1);
  if (!(lo <= v && (v < hi || i == n - 2))) {
    int a = 0, b = n - 1;
    while (b - a > 1) {
      const int mid = (a + b) >> 1;
      if (__ldg(g + mid) <= v) a = mid;
      else b = mid;
    }
    i = a;
    lo = __ldg(g + i);
    hi = __ldg(g + i + 1);
  }
  w = (v - lo) / (hi - lo);
  return i;
}

__device__ __forceinline__ bool grid_inside(const double* __restrict__ g, int n, double v) {
  return __ldg(g) <= v && v <= __ldg(g + n - 1);
}

struct GridCell {
  int64_t base;          // node index of the lower corner at the lower snapshot
  int64_t sx, sy, st;    // node strides
  double wt, wx, wy, wz;
  int ntc;               // time corners: 1 (one snapshot) or 2
  bool ok;
};

__device__ __forceinline__ GridCell grid_locate(const double* __restrict__ gt, const double* __restrict__ gx,
                                                const double* __restrict__ gy, const double* __restrict__ gz,
                                                const double* inv, int nt, int nx, int ny, int nz, double t, double x,
                                                double y, double z) {
  GridCell c;
  c.ok = grid_inside(gx, nx, x) && grid_inside(gy, ny, y) && grid_inside(gz, nz, z) &&
         (nt == 1 || grid_inside(gt, nt, t));
  c.sy = nz; c.sx = (int64_t)ny * nz; c.st = (int64_t)nx * c.sx;
  c.ntc = nt > 1 ? 2 : 1;
  c.wt = 1.0;
  c.base = 0;
  if (!c.ok) return c;
  const int ix = grid_cell(gx, nx, inv[1], x, c.wx);
  const int iy = grid_cell(gy, ny, inv[2], y, c.wy);
  const int iz = grid_cell(gz, nz, inv[3], z, c.wz);
  const int it = nt > 1 ? grid_cell(gt, nt, inv[0], t, c.wt) : 0;
  c.base = it * c.st + ix * c.sx + iy * c.sy + iz;
  return c;
}

// Corner sum of K arrays (3 components each) at one located point. One
// snapshot: weights (1 * wx) * wy * wz, the same products as the 3-D
// interpolator's, since 1 * w == w.
template <int K>
__device__ __forceinline__ void grid_sum(const GridCell& c, const double* const* V, double* out) {
#pragma unroll
  for (int k = 0; k < 3 * K; ++k) out[k] = 0.0;
  for (int ct = 0; ct < c.ntc; ++ct) {
    const double w1 = c.ntc == 1 ? 1.0 : (ct ? c.wt : 1.0 - c.wt);
#pragma unroll
    for (int cx = 0; cx < 2; ++cx) {
      const double w2 = __dmul_rn(w1, cx ? c.wx : 1.0 - c.wx);
#pragma unroll
      for (int cy = 0; cy < 2; ++cy) {
        const double w3 = __dmul_rn(w2, cy ? c.wy : 1.0 - c.wy);
        const int64_t node = c.base + ct * c.st + cx * c.sx + cy * c.sy;
#pragma unroll
        for (int cz = 0; cz < 2; ++cz) {
          const double w = __dmul_rn(w3, cz ? c.wz : 1.0 - c.wz);
#pragma unroll
          for (int k = 0; k < K; ++k) {
            const double* p = V[k] + 3 * (node + cz);
#pragma unroll
            for (int j = 0; j < 3; ++j) out[3 * k + j] = __dadd_rn(out[3 * k + j], __dmul_rn(__ldg(p + j), w));
          }
        }
      }
    }
  }
}

// The device-resident grid as scalars, so that the non-inlined interpolation
// functions take their arguments in registers.
#define RAPT_GRID_ARGS                                                                                      \
  const double *__restrict__ gt, const double *__restrict__ gx, const double *__restrict__ gy,              \
      const double *__restrict__ gz, double it_, double ix_, double iy_, double iz_, int nt, int nx, int ny, \
      int nz
#define RAPT_GRID_PASS(f) \
  f.gt, f.gx, f.gy, f.gz, f.ginv[0], f.ginv[1], f.ginv[2], f.ginv[3], f.nt, f.nx, f.ny, f.nz

struct GridV6 {
  double v[6];
};

// One interpolation of a [nt][nx][ny][nz][3] array: not inlined, so that the
// evaluations of a guiding-centre right-hand side share one copy.
static __device__ __noinline__ GridV grid_interp(RAPT_GRID_ARGS, const double* __restrict__ V, double t, double x,
                                                 double y, double z) {
  const double inv[4] = {it_, ix_, iy_, iz_};
  const GridCell c = grid_locate(gt, gx, gy, gz, inv, nt, nx, ny, nz, t, x, y, z);
  if (!c.ok) {
    const double qnan = __longlong_as_double(0x7ff8000000000000LL);
    return GridV{qnan, qnan, qnan};
  }
  const double* arr[1] = {V};
  double o[3];
  grid_sum<1>(c, arr, o);
  return GridV{o[0], o[1], o[2]};
}

// B and E at one point from one cell search (the right-hand sides need both).
static __device__ __noinline__ GridV6 grid_interp_BE(RAPT_GRID_ARGS, const double* __restrict__ VB,
                                                     const double* __restrict__ VE, double t, double x, double y,
                                                     double z) {
  const double inv[4] = {it_, ix_, iy_, iz_};
  const GridCell c = grid_locate(gt, gx, gy, gz, inv, nt, nx, ny, nz, t, x, y, z);
  GridV6 r;
  if (!c.ok) {
    const double qnan = __longlong_as_double(0x7ff8000000000000LL);
#pragma unroll
    for (int k = 0; k < 6; ++k) r.v[k] = qnan;
    return r;
  }
  if (VE) {
    const double* arr[2] = {VB, VE};
    grid_sum<2>(c, arr, r.v);
  } else {
    const double* arr[1] = {VB};
    grid_sum<1>(c, arr, r.v);
    r.v[3] = r.v[4] = r.v[5] = 0.0;
  }
  return r;
}

template <>
struct Field<RAPT_GRID> {
  static constexpr bool kStatic = false;  // the runtime flag f.is_static decides (field_static)
  __device__ __forceinline__ static void B(const FieldP& f, double t, double x, double y, double z, double* o) {
    const GridV r = grid_interp(RAPT_GRID_PASS(f), f.gB, t, x, y, z);
    o[0] = r.a; o[1] = r.b; o[2] = r.c;
  }
  __device__ __forceinline__ static void E(const FieldP& f, double t, double x, double y, double z, double* o) {
    if (!f.gE) { o[0] = o[1] = o[2] = 0.0; return; }
    const GridV r = grid_interp(RAPT_GRID_PASS(f), f.gE, t, x, y, z);
    o[0] = r.a; o[1] = r.b; o[2] = r.c;
  }
};

// |B| and b from B, each product rounded on its own (values that feed a central
// difference).
__device__ __forceinline__ void unit_and_mag_of(const double* b, double* ub, double& mag) {
  const double b2 = dot3(b, b);
  const double ib = rsqrt(b2);
  mag = __dmul_rn(b2, ib);
  ub[0] = __dmul_rn(b[0], ib); ub[1] = __dmul_rn(b[1], ib); ub[2] = __dmul_rn(b[2], ib);
}

// One axis of a located point: the cell index and weight of v (ok: inside).
struct GridAxis {
  int i;
  double w;
  bool ok;
};
__device__ __forceinline__ GridAxis grid_axis(const double* __restrict__ g, int n, double inv, double v) {
  GridAxis a{0, 0.0, grid_inside(g, n, v)};
  if (a.ok) a.i = grid_cell(g, n, inv, v, a.w);
  return a;
}
// The corner sum of K arrays at the point located by its four axes (NaN outside).
template <int K>
__device__ __forceinline__ void grid_sum_axes(const GridAxis& at, const GridAxis& ax, const GridAxis& ay,
                                              const GridAxis& az, int nt, int nx, int ny, int nz,
                                              const double* const* V, double* out) {
  GridCell c;
  c.ok = at.ok && ax.ok && ay.ok && az.ok;
  if (!c.ok) {
#pragma unroll
    for (int k = 0; k < 3 * K; ++k) out[k] = __longlong_as_double(0x7ff8000000000000LL);
    return;
  }
  c.sy = nz; c.sx = (int64_t)ny * nz; c.st = (int64_t)nx * c.sx;
  c.ntc = nt > 1 ? 2 : 1;
  c.wt = nt > 1 ? at.w : 1.0;
  c.wx = ax.w; c.wy = ay.w; c.wz = az.w;
  c.base = (nt > 1 ? at.i : 0) * c.st + ax.i * c.sx + ay.i * c.sy + az.i;
  grid_sum<K>(c, V, out);
}

// Everything a guiding-centre right-hand side takes from a gridded field at one
// point -- B and E, the reference's central differences grad|B| and curl b
// (fields.py:111-131, 175-200) and db/dt (fields.py:225-245) -- from one cell
// search. Each sample of the stencil differs from the centre in one
// coordinate, so only that axis is searched again; the other axes keep the
// centre's cell and weight, which are the values a full search of the sample
// returns: every sample is the number a separate interpolation gives. Outside
// the grid the values are NaN. Not inlined (one copy per kernel).
struct GridFields {
  double B[3], E[3], gB[3], cb[3], db[3];
};
static __device__ __noinline__ GridFields grid_gc_fields(RAPT_GRID_ARGS, const double* __restrict__ VB,
                                                         const double* __restrict__ VE, double t, double x,
                                                         double y, double z, double d, double inv2d, double ts,
                                                         bool timedep) {
  const GridAxis at = nt > 1 ? grid_axis(gt, nt, it_, t) : GridAxis{0, 1.0, true};
  const GridAxis ax = grid_axis(gx, nx, ix_, x), ay = grid_axis(gy, ny, iy_, y), az = grid_axis(gz, nz, iz_, z);
  GridFields r;
  if (VE) {
    const double* arr[2] = {VB, VE};
    double o[6];
    grid_sum_axes<2>(at, ax, ay, az, nt, nx, ny, nz, arr, o);
#pragma unroll
    for (int k = 0; k < 3; ++k) { r.B[k] = o[k]; r.E[k] = o[3 + k]; }
  } else {
    const double* arr[1] = {VB};
    grid_sum_axes<1>(at, ax, ay, az, nt, nx, ny, nz, arr, r.B);
    r.E[0] = r.E[1] = r.E[2] = 0.0;
  }
  const double* arr[1] = {VB};
  const double X[3] = {x, y, z};
  double c0 = 0.0, c1 = 0.0, c2 = 0.0;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const double* g = a == 0 ? gx : (a == 1 ? gy : gz);
    const int n = a == 0 ? nx : (a == 1 ? ny : nz);
    const double inv = a == 0 ? ix_ : (a == 1 ? iy_ : iz_);
    double up[3], um[3], mp, mm, b[3];
    {
      const GridAxis s = grid_axis(g, n, inv, X[a] + d);
      grid_sum_axes<1>(at, a == 0 ? s : ax, a == 1 ? s : ay, a == 2 ? s : az, nt, nx, ny, nz, arr, b);
      unit_and_mag_of(b, up, mp);
    }
    {
      const GridAxis s = grid_axis(g, n, inv, X[a] - d);
      grid_sum_axes<1>(at, a == 0 ? s : ax, a == 1 ? s : ay, a == 2 ? s : az, nt, nx, ny, nz, arr, b);
      unit_and_mag_of(b, um, mm);
    }
    r.gB[a] = (mp - mm) * inv2d;
    if (a == 0) { c1 -= (up[2] - um[2]); c2 += (up[1] - um[1]); }
    if (a == 1) { c0 += (up[2] - um[2]); c2 -= (up[0] - um[0]); }
    if (a == 2) { c0 -= (up[1] - um[1]); c1 += (up[0] - um[0]); }
  }
  r.cb[0] = c0 * inv2d; r.cb[1] = c1 * inv2d; r.cb[2] = c2 * inv2d;
  r.db[0] = r.db[1] = r.db[2] = 0.0;
  if (timedep) {
    double u1[3], u2[3], m1, m2, b[3];
    const GridAxis t1 = nt > 1 ? grid_axis(gt, nt, it_, t - ts) : at;
    grid_sum_axes<1>(t1, ax, ay, az, nt, nx, ny, nz, arr, b);
    unit_and_mag_of(b, u1, m1);
    const GridAxis t2 = nt > 1 ? grid_axis(gt, nt, it_, t + ts) : at;
    grid_sum_axes<1>(t2, ax, ay, az, nt, nx, ny, nz, arr, b);
    unit_and_mag_of(b, u2, m2);
    const double sc = 0.5 / ts;
    r.db[0] = (u2[0] - u1[0]) * sc; r.db[1] = (u2[1] - u1[1]) * sc; r.db[2] = (u2[2] - u1[2]) * sc;
  }
  return r;
}

// B and E at one point: one cell search for a Grid, the two model functions otherwise.
template <int M>
__device__ __forceinline__ void field_BE(const FieldP& f, double t, double x, double y, double z, double* B,
                                         double* E) {
  if constexpr (M == RAPT_GRID) {
    const GridV6 r = grid_interp_BE(RAPT_GRID_PASS(f), f.gB, f.gE, t, x, y, z);
    B[0] = r.v[0]; B[1] = r.v[1]; B[2] = r.v[2];
    E[0] = r.v[3]; E[1] = r.v[4]; E[2] = r.v[5];
  } else {
    Field<M>::B(f, t, x, y, z, B);
    Field<M>::E(f, t, x, y, z, E);
  }
}

// _Field.static (fields.py:41): fixed by the equations of the analytic models,
// the runtime attribute for Grid (which leaves it True by default).
template <int M>
__device__ __forceinline__ bool field_static(const FieldP& f) {
  return Field<M>::kStatic || (M == RAPT_GRID && f.is_static);
}

// A step whose error norm is NaN evaluated a Grid field outside the grid: the
// reference raises ValueError there, the steppers stop with RAPT_ST_OUT_OF_GRID.
template <int M>
__device__ __forceinline__ bool left_grid(double err) {
  return M == RAPT_GRID && isnan(err);
}

// Unit vector and magnitude of B at a point: one rsqrt.
template <int M>
__device__ __forceinline__ void unit_and_mag(const FieldP& f, double t, double x, double y, double z, double* ub,
                                             double& mag) {
  double b[3];
  Field<M>::B(f, t, x, y, z, b);
  unit_and_mag_of(b, ub, mag);
}

// The reference's central-difference stencil (fields.py:111-131 gradB and
// 176-200 curlb) evaluates B at the same six points x +- d e_i twice; here each
// point is evaluated once and feeds both grad|B| and curl b.
template <int M>
__device__ __forceinline__ void stencil_gradB_curlb(const FieldP& f, double t, const double* X, double* gB,
                                                    double* cb) {
  double c0 = 0.0, c1 = 0.0, c2 = 0.0;
  const double d = f.gradstep;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    double up[3], um[3], mp, mm;
    double xp[3] = {X[0], X[1], X[2]}, xm[3] = {X[0], X[1], X[2]};
    xp[a] = X[a] + d;
    xm[a] = X[a] - d;
    unit_and_mag<M>(f, t, xp[0], xp[1], xp[2], up, mp);
    unit_and_mag<M>(f, t, xm[0], xm[1], xm[2], um, mm);
    gB[a] = (mp - mm) * f.inv2d;
    if (a == 0) { c1 -= (up[2] - um[2]); c2 += (up[1] - um[1]); }
    if (a == 1) { c0 += (up[2] - um[2]); c2 -= (up[0] - um[0]); }
    if (a == 2) { c0 -= (up[1] - um[1]); c1 += (up[0] - um[0]); }
  }
  cb[0] = c0 * f.inv2d; cb[1] = c1 * f.inv2d; cb[2] = c2 * f.inv2d;
}

// db/dt by central differences in time (fields.py:225-245); zero when static.
template <int M>
__device__ __forceinline__ void dbdt(const FieldP& f, double t, const double* X, double* o) {
  if (field_static<M>(f)) { o[0] = o[1] = o[2] = 0.0; return; }
  double u1[3], u2[3], m1, m2;
  unit_and_mag<M>(f, t - f.timestep, X[0], X[1], X[2], u1, m1);
  unit_and_mag<M>(f, t + f.timestep, X[0], X[1], X[2], u2, m2);
  const double s = 0.5 / f.timestep;
  o[0] = (u2[0] - u1[0]) * s; o[1] = (u2[1] - u1[1]) * s; o[2] = (u2[2] - u1[2]) * s;
}

// d|B|/dt (fields.py:202-223).
template <int M>
__device__ __forceinline__ double dBdt(const FieldP& f, double t, const double* X) {
  if (field_static<M>(f)) return 0.0;
  double u[3], m1, m2;
  unit_and_mag<M>(f, t - f.timestep, X[0], X[1], X[2], u, m1);
  unit_and_mag<M>(f, t + f.timestep, X[0], X[1], X[2], u, m2);
  return (m2 - m1) / f.timestep / 2.0;
}

// |B| / max|dB_i/dx_j| (fields.py:247-261).
template <int M>
__device__ __forceinline__ double lengthscale(const FieldP& f, double t, const double* X) {
  double mx = 0.0;
  const double d = f.gradstep;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    double xp[3] = {X[0], X[1], X[2]}, xm[3] = {X[0], X[1], X[2]};
    xp[a] = X[a] + d;
    xm[a] = X[a] - d;
    double bp[3], bm[3];
    Field<M>::B(f, t, xp[0], xp[1], xp[2], bp);
    Field<M>::B(f, t, xm[0], xm[1], xm[2], bm);
#pragma unroll
    for (int i = 0; i < 3; ++i) mx = fmax(mx, fabs((bp[i] - bm[i]) * f.inv2d));
  }
  double b[3];
  Field<M>::B(f, t, X[0], X[1], X[2], b);
  return sqrt(dot3(b, b)) / mx;
}

}  // namespace rapt
