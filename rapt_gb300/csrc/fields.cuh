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

// Unit vector and magnitude of B at a point: one rsqrt.
template <int M>
__device__ __forceinline__ void unit_and_mag(const FieldP& f, double t, double x, double y, double z, double* ub,
                                             double& mag) {
  double b[3];
  Field<M>::B(f, t, x, y, z, b);
  const double b2 = dot3(b, b);
  const double ib = rsqrt(b2);
  mag = __dmul_rn(b2, ib);
  ub[0] = __dmul_rn(b[0], ib); ub[1] = __dmul_rn(b[1], ib); ub[2] = __dmul_rn(b[2], ib);
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
  if (Field<M>::kStatic) { o[0] = o[1] = o[2] = 0.0; return; }
  double u1[3], u2[3], m1, m2;
  unit_and_mag<M>(f, t - f.timestep, X[0], X[1], X[2], u1, m1);
  unit_and_mag<M>(f, t + f.timestep, X[0], X[1], X[2], u2, m2);
  const double s = 0.5 / f.timestep;
  o[0] = (u2[0] - u1[0]) * s; o[1] = (u2[1] - u1[1]) * s; o[2] = (u2[2] - u1[2]) * s;
}

// d|B|/dt (fields.py:202-223).
template <int M>
__device__ __forceinline__ double dBdt(const FieldP& f, double t, const double* X) {
  if (Field<M>::kStatic) return 0.0;
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
