// step_math.cuh -- small FP64 algebra of the implicit time step: unit
// quaternions of segment and body orientations, their Lie-algebra maps, and
// 3x3 blocks. Host and device (the body's 6-DOF state is advanced on the
// host, segments and filaments on the device).
//
// Conventions restated from the reference (src/general/quaternion.cpp,
// src/general/matrix.cpp):
//   q = (s, v) scalar first; q1 * q2 the Hamilton product.
//   lie_exp(u) = (cos(|u|/2), sin(|u|/2) u/|u|), identity for |u| < 1e-6.
//   tangent/normal/binormal = the columns of the rotation matrix of q.
//   rcross(v) is the 3x3 matrix with rcross(v) a = a x v.
//   dexpinv(u, v) = v - (u x v)/2 - c u x (u x v), c = (θ/2 cot(θ/2) - 1)/θ²
//   (c = -1/12 for θ < 1e-5); dexpinv_transpose flips the sign of (u x v)/2.
// 3x3 blocks here are row-major: m[3 i + j] = entry (i, j).
#pragma once

#include <cmath>

#ifdef __CUDACC__
#define TFS_HD __host__ __device__ __forceinline__
#else
#define TFS_HD inline
#endif

namespace tfs {
namespace step {

struct Quat {
  double s, x, y, z;
};

TFS_HD Quat qmul(const Quat &p, const Quat &q) {
  Quat r;
  r.s = p.s * q.s - (p.x * q.x + p.y * q.y + p.z * q.z);
  r.x = p.s * q.x + q.s * p.x + p.y * q.z - p.z * q.y;
  r.y = p.s * q.y + q.s * p.y + p.z * q.x - p.x * q.z;
  r.z = p.s * q.z + q.s * p.z + p.x * q.y - p.y * q.x;
  return r;
}

TFS_HD Quat qconj(const Quat &q) { return Quat{q.s, -q.x, -q.y, -q.z}; }

TFS_HD Quat load_q(const double *p) { return Quat{p[0], p[1], p[2], p[3]}; }
TFS_HD void store_q(double *p, const Quat &q) {
  p[0] = q.s;
  p[1] = q.x;
  p[2] = q.y;
  p[3] = q.z;
}

TFS_HD Quat lie_exp(const double *u) {
  const double th = sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
  if (th < 1e-6) return Quat{1.0, 0.0, 0.0, 0.0};
  const double c = cos(0.5 * th), sn = sin(0.5 * th) / th;
  return Quat{c, sn * u[0], sn * u[1], sn * u[2]};
}

// Principal square root of a unit quaternion (quaternion.cpp sqrt_in_place).
TFS_HD Quat qsqrt(const Quat &q) {
  if (q.s < -0.999999999) return Quat{0.0, 0.0, 0.0, 1.0};
  Quat r;
  r.s = sqrt(0.5 * (1.0 + q.s));
  const double t = 2.0 * r.s;
  r.x = q.x / t;
  r.y = q.y / t;
  r.z = q.z / t;
  return r;
}

// Rotation half-way from q1 to q2: sqrt(q2 q1*) q1.
TFS_HD Quat midpoint(const Quat &q1, const Quat &q2) {
  return qmul(qsqrt(qmul(q2, qconj(q1))), q1);
}

// Orientation of a straight filament along dir (filament::initial_setup,
// quaternion::sqrt_in_place_ortho): the root of (d0, 0, -d2, d1), normalised.
TFS_HD Quat along_direction(const double *dir_in) {
  const double nrm = sqrt(dir_in[0] * dir_in[0] + dir_in[1] * dir_in[1] + dir_in[2] * dir_in[2]);
  const double d0 = dir_in[0] / nrm, d1 = dir_in[1] / nrm, d2 = dir_in[2] / nrm;
  Quat q{d0, 0.0, -d2, d1};
  if (q.s < -0.999999) q.s = -0.9999999;
  q.s = sqrt(0.5 * (1.0 + q.s));
  const double t = 2.0 * q.s;
  q.x /= t;
  q.y /= t;
  q.z /= t;
  if (!(d0 >= -0.999999)) {  // the near-antiparallel branch renormalises once more
    const double n0 = sqrt(q.s * q.s + q.x * q.x + q.y * q.y + q.z * q.z);
    q.s *= n0;
    q.x /= n0;
    q.y /= n0;
    q.z /= n0;
  }
  const double n = sqrt(q.s * q.s + q.x * q.x + q.y * q.y + q.z * q.z);
  return Quat{q.s / n, q.x / n, q.y / n, q.z / n};
}

TFS_HD void tangent(const Quat &q, double *t) {
  t[0] = 1.0 - 2.0 * (q.y * q.y + q.z * q.z);
  t[1] = 2.0 * (q.x * q.y + q.s * q.z);
  t[2] = 2.0 * (q.x * q.z - q.s * q.y);
}
TFS_HD void normal(const Quat &q, double *n) {
  n[0] = 2.0 * (q.x * q.y - q.s * q.z);
  n[1] = 1.0 - 2.0 * (q.x * q.x + q.z * q.z);
  n[2] = 2.0 * (q.y * q.z + q.s * q.x);
}
TFS_HD void binormal(const Quat &q, double *b) {
  b[0] = 2.0 * (q.x * q.z + q.s * q.y);
  b[1] = 2.0 * (q.y * q.z - q.s * q.x);
  b[2] = 1.0 - 2.0 * (q.x * q.x + q.y * q.y);
}

// Rotation matrix of q (row-major), in the reference's order of operations.
TFS_HD void rot_mat(const Quat &q, double *R) {
  R[0] = 1.0;
  R[4] = 1.0;
  R[8] = 1.0;
  double t = 2.0 * q.x * q.x;
  R[4] -= t;
  R[8] -= t;
  t = 2.0 * q.y * q.y;
  R[0] -= t;
  R[8] -= t;
  t = 2.0 * q.z * q.z;
  R[0] -= t;
  R[4] -= t;
  t = 2.0 * q.x * q.y;
  R[3] = t;
  R[1] = t;
  t = 2.0 * q.x * q.z;
  R[6] = t;
  R[2] = t;
  t = 2.0 * q.y * q.z;
  R[5] = t;
  R[7] = t;
  t = 2.0 * q.s * q.z;
  R[3] += t;
  R[1] -= t;
  t = 2.0 * q.s * q.y;
  R[6] -= t;
  R[2] += t;
  t = 2.0 * q.s * q.x;
  R[7] += t;
  R[5] -= t;
}

TFS_HD double dexp_fac(const double *u) {
  const double th2 = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
  const double th = sqrt(th2);
  if (th < 1e-5) return -1.0 / 12.0;
  return (0.5 * th * cos(0.5 * th) / sin(0.5 * th) - 1.0) / th2;
}

// sign = -1: dexpinv(u, v); sign = +1: its transpose.
TFS_HD void dexpinv_s(double *out, const double *u, const double *v, double sign) {
  const double c = dexp_fac(u);
  const double w[3] = {u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2],
                       u[0] * v[1] - u[1] * v[0]};
  out[0] = v[0] + sign * 0.5 * w[0] - c * (u[1] * w[2] - u[2] * w[1]);
  out[1] = v[1] + sign * 0.5 * w[1] - c * (u[2] * w[0] - u[0] * w[2]);
  out[2] = v[2] + sign * 0.5 * w[2] - c * (u[0] * w[1] - u[1] * w[0]);
}

// ---- 3x3 blocks (row-major) ------------------------------------------------
struct M3 {
  double a[9];
};

TFS_HD M3 m3_zero() {
  M3 m;
  for (int k = 0; k < 9; ++k) m.a[k] = 0.0;
  return m;
}
TFS_HD M3 m3_eye() {
  M3 m = m3_zero();
  m.a[0] = m.a[4] = m.a[8] = 1.0;
  return m;
}
// rcross(v): rcross(v) a = a x v
TFS_HD M3 rcross(const double *v) {
  M3 m;
  m.a[0] = 0.0;
  m.a[1] = v[2];
  m.a[2] = -v[1];
  m.a[3] = -v[2];
  m.a[4] = 0.0;
  m.a[5] = v[0];
  m.a[6] = v[1];
  m.a[7] = -v[0];
  m.a[8] = 0.0;
  return m;
}
TFS_HD M3 m3_mul(const M3 &x, const M3 &y) {
  M3 r;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double s = 0.0;
      for (int k = 0; k < 3; ++k) s += x.a[3 * i + k] * y.a[3 * k + j];
      r.a[3 * i + j] = s;
    }
  return r;
}
TFS_HD M3 m3_add(const M3 &x, const M3 &y) {
  M3 r;
  for (int k = 0; k < 9; ++k) r.a[k] = x.a[k] + y.a[k];
  return r;
}
TFS_HD M3 m3_sub(const M3 &x, const M3 &y) {
  M3 r;
  for (int k = 0; k < 9; ++k) r.a[k] = x.a[k] - y.a[k];
  return r;
}
TFS_HD M3 m3_scale(double s, const M3 &x) {
  M3 r;
  for (int k = 0; k < 9; ++k) r.a[k] = s * x.a[k];
  return r;
}
TFS_HD M3 m3_div(const M3 &x, double s) {
  M3 r;
  for (int k = 0; k < 9; ++k) r.a[k] = x.a[k] / s;
  return r;
}
TFS_HD M3 m3_from(const double *rm) {  // row-major 9 doubles
  M3 m;
  for (int k = 0; k < 9; ++k) m.a[k] = rm[k];
  return m;
}
TFS_HD void m3_vec(const M3 &m, const double *v, double *out) {
  for (int i = 0; i < 3; ++i) {
    double s = 0.0;
    for (int k = 0; k < 3; ++k) s += m.a[3 * i + k] * v[k];
    out[i] = s;
  }
}

// The 4x3 map psi(q) (quaternion.cpp psi_mat): row 0 = -v^T, rows 1..3 =
// rcross(v) + s I, all halved. Row-major 12 doubles.
TFS_HD void psi_mat(const Quat &q, double *P) {
  const double v[3] = {q.x, q.y, q.z};
  const M3 rc = rcross(v);
  P[0] = -q.x;
  P[1] = -q.y;
  P[2] = -q.z;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) P[3 * (i + 1) + j] = rc.a[3 * i + j] + (i == j ? q.s : 0.0);
  for (int k = 0; k < 12; ++k) P[k] *= 0.5;
}

// Left-multiplication matrix of q (4x4, row-major): [[s, -v^T], [v, s I - rcross(v)]].
TFS_HD void left_mult_mat(const Quat &q, double *L) {
  const double v[3] = {q.x, q.y, q.z};
  const M3 rc = rcross(v);
  L[0] = q.s;
  L[1] = -q.x;
  L[2] = -q.y;
  L[3] = -q.z;
  L[4] = q.x;
  L[8] = q.y;
  L[12] = q.z;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) L[4 * (i + 1) + (j + 1)] = -rc.a[3 * i + j] + (i == j ? q.s : 0.0);
}

// Body-frame bending/twisting moment of the link between two segments
// (filament::body_frame_moment): K (2 q_mid^* (q2 - q1)/DL - strain), with
// K = diag(kt, kb, kb).
TFS_HD void link_moment(const Quat &q1, const Quat &q2, double dl, double kb, double kt,
                        const double *strain, double *M) {
  const Quat mq = qconj(midpoint(q1, q2));
  const Quat dq{q2.s - q1.s, q2.x - q1.x, q2.y - q1.y, q2.z - q1.z};
  const Quat p = qmul(mq, dq);
  M[0] = kt * (2.0 * (p.x / dl) - strain[0]);
  M[1] = kb * (2.0 * (p.y / dl) - strain[1]);
  M[2] = kb * (2.0 * (p.z / dl) - strain[2]);
}

// Approximate derivative of the link moment with respect to the Lie algebra
// element of the upper (q2) or lower (q1) segment
// (filament.cpp body_frame_moment_lie_derivative).
TFS_HD M3 link_moment_lie_derivative(const Quat &q1, const Quat &q2, bool upper, double dl,
                                     double kb, double kt) {
  double A[12], L[16], D[12];
  psi_mat(upper ? q2 : q1, A);
  for (int k = 0; k < 12; ++k) A[k] = upper ? A[k] / dl : A[k] / -dl;
  left_mult_mat(qconj(midpoint(q1, q2)), L);
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 3; ++j) {
      double s = 0.0;
      for (int k = 0; k < 4; ++k) s += L[4 * i + k] * A[3 * k + j];
      D[3 * i + j] = s;
    }
  const Quat dq{(q2.s - q1.s) / dl, (q2.x - q1.x) / dl, (q2.y - q1.y) / dl, (q2.z - q1.z) / dl};
  left_mult_mat(dq, L);
  const double sB = upper ? 0.5 * dl : -0.5 * dl;
  for (int k = 0; k < 12; ++k) A[k] *= sB;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 3; ++j) {
      double s = 0.0;
      for (int k = 0; k < 4; ++k) s += L[4 * i + k] * A[3 * k + j];
      D[3 * i + j] += s;
    }
  M3 out;
  const double K[3] = {kt, kb, kb};
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) out.a[3 * i + j] = (2.0 * D[3 * (i + 1) + j]) * K[i];
  return out;
}

}  // namespace step
}  // namespace tfs
