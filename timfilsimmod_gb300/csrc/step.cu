// step.cu -- the implicit time step of one free swimmer with elastic
// filaments, device-resident: the loop of src/cilia/cilia_sim_main.cu:355-527
// (initial guess, internal forces, mobility solve, BDF residuals, the
// approximate-Jacobian Broyden iteration) for the configuration of elastic
// filaments tethered and clamped to a free rigid body (CILIA_TYPE 0,
// free body, GMRES linear solve).
//
// Unknowns per filament (6 NSEG, filament::update, filament.cpp:1896-1930):
//   [0, 3)          tether force,
//   [3 j, 3 j + 3)  inextensibility force of link j-1 (j = 1 .. NSEG-1),
//   [3 NSEG, +3)    clamping torque,
//   [3 (NSEG + j))  Lie-algebra increment of segment j (j = 1 .. NSEG-1);
// then six for the body (translation, rotation). Residuals use the same
// layout (mobility_solver.cpp:2661-2946): segment position and Lie-algebra
// BDF residuals per filament, then the body's.
//
// Work split. Segments and filaments live on the device: one thread per
// filament for the sequential parts (robot arm, internal forces), one CTA
// per filament for the approximate Jacobian (built in shared memory and
// inverted there by Gauss-Jordan with partial pivoting) and its products,
// one CTA per Broyden column for the low-rank update. The body's six degrees
// of freedom and the 6x6 Schur complement stay on the host (tens of
// numbers); the host drives the Broyden loop, reading back the convergence
// flag and the body's update once per iteration.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "step_math.cuh"
#include "tfs_solver.h"

using namespace tfs;
using namespace tfs::step;

namespace {

constexpr double kPiS = 3.14159265358979323846264338327950288;

struct StepDev {
  int nfil, nseg, ns, nbroy;
  double dl, dt, kb, kt, efm, mu, a, body_r, pert;
  int perturb;
  double *q, *qm1, *u, *um1, *xm1, *xm2;  // per segment
  double *x;                              // segment positions (the solver's x_segs)
  double *f;                              // internal forces and torques (6 per segment)
  double *fs;                             // the solver's f_segs (barrier forces get added there)
  double *lam, *lamm1, *lamm2;            // 3 (NSEG-1) per filament
  double *teth, *tethm1, *tethm2, *clamp, *clampm1, *clampm2;  // 3 per filament
  const double *fil_refs;                 // body-frame base offsets, 3 per filament
  double *jinv;                           // (6 NSEG)^2 per filament, row-major
  double *jb;                             // 6 x 6 NSEG per filament, row-major
  double *ecb;                            // the two 3x3 elastic clamping blocks per filament
  double *part;                           // per-filament partials (45)
};

struct BodyArgs {
  double x[3], xm1[3], xm2[3], u[3], um1[3];
  double R[9];       // rotation of the current body quaternion (row-major)
  double Q[9];       // rotation of the step's initial guess (Q_init)
  double BM[36];     // body mobility reference rotated by Q_init (row-major)
  double Dinv[9], DinvT[9], blc[9];
  double dt_fac;
};

// ---------------------------------------------------------------------------
// segment and filament mechanics
// ---------------------------------------------------------------------------

// segment::update: u += du, q = exp(u) qm1
__device__ void seg_update(const StepDev &d, int s, const double *du) {
  double *u = d.u + 3 * s;
  u[0] += du[0];
  u[1] += du[1];
  u[2] += du[2];
  store_q(d.q + 4 * s, qmul(lie_exp(u), load_q(d.qm1 + 4 * s)));
}

// BDF2 extrapolation of a multiplier from its last values (filament::initial_guess)
__device__ void extrapolate(double *v, double *m1, double *m2, int n, int nt) {
  for (int k = 0; k < n; ++k) {
    if (nt == 1) {
      m1[k] = v[k];
    } else if (nt == 2) {
      m2[k] = m1[k];
      m1[k] = v[k];
      v[k] = 2.0 * m1[k] - m2[k];
    } else if (nt > 2) {
      const double t = 3.0 * (v[k] - m1[k]) + m2[k];
      m2[k] = m1[k];
      m1[k] = v[k];
      v[k] = t;
    }
  }
}

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------

// The base segment at X + R ref and the robot arm
// x_j = x_{j-1} + DL/2 (t_{j-1} + t_j) (accept_state_from_rigid_body and
// robot_arm, filament.cpp:625-661), one warp per filament. In
// swimmer::update the reference runs the robot arm twice (after the base
// segment's update and after the whole filament's); the first result is
// overwritten by the second, which depends only on x_0 and the final
// orientations, so it runs once here, after every segment is updated.
constexpr int kFilWarps = 4;  // filaments (one warp each) per CTA of the per-filament kernels

__global__ void __launch_bounds__(32 * kFilWarps) k_robot_arm(StepDev d, BodyArgs b) {
  __shared__ double tan_s[kFilWarps][32][3];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int fil = blockIdx.x * kFilWarps + w;
  if (fil >= d.nfil) return;  // the whole warp
  const int s0 = fil * d.nseg;
  double xp[3] = {0.0, 0.0, 0.0}, t1[3] = {0.0, 0.0, 0.0};
  if (lane == 0) {
    const double *ref = d.fil_refs + 3 * fil;
    for (int i = 0; i < 3; ++i) {
      double s = 0.0;
      for (int k = 0; k < 3; ++k) s += b.R[3 * i + k] * ref[k];
      xp[i] = b.x[i] + s;
      d.x[3 * s0 + i] = xp[i];
    }
  }
  // the lanes form 32 segments' tangents at a time; lane 0 adds them up in
  // segment order
  for (int j0 = 0; j0 < d.nseg; j0 += 32) {
    if (j0 + lane < d.nseg) tangent(load_q(d.q + 4 * (s0 + j0 + lane)), tan_s[w][lane]);
    __syncwarp();
    if (lane == 0) {
      const int m = min(32, d.nseg - j0);
      for (int q = 0; q < m; ++q) {
        const double *t2 = tan_s[w][q];
        const int s = s0 + j0 + q;
        if (s > s0)
          for (int k = 0; k < 3; ++k) {
            xp[k] = xp[k] + 0.5 * d.dl * (t1[k] + t2[k]);
            d.x[3 * s + k] = xp[k];
          }
        for (int k = 0; k < 3; ++k) t1[k] = t2[k];
      }
    }
    __syncwarp();
  }
}

// swimmer::initial_guess, one thread per segment: segment::initial_guess
// (segment.cpp:38-76); for the base segment then the body's Lie algebra
// element (accept_state_from_rigid_body); multiplier extrapolation
// (filament.cpp:1275-1385): link j-1 by segment j, tether and clamp by the
// base segment. The robot arm follows (k_robot_arm).
__global__ void k_guess_segments(StepDev d, BodyArgs b, int nt) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= d.ns) return;
  const int fil = s / d.nseg, j = s - fil * d.nseg;
  for (int k = 0; k < 3; ++k) {
    d.xm2[3 * s + k] = d.xm1[3 * s + k];
    d.xm1[3 * s + k] = d.x[3 * s + k];
  }
  double *u = d.u + 3 * s, *um1 = d.um1 + 3 * s;
  for (int k = 0; k < 3; ++k) {
    if (nt <= 1) {
      um1[k] = u[k];
    } else {
      const double t = 2.0 * u[k] - um1[k];
      um1[k] = u[k];
      u[k] = t;
    }
  }
  const Quat q = load_q(d.q + 4 * s);
  store_q(d.qm1 + 4 * s, q);
  store_q(d.q + 4 * s, qmul(lie_exp(u), q));
  if (j == 0) {
    const double du[3] = {b.u[0] - u[0], b.u[1] - u[1], b.u[2] - u[2]};
    seg_update(d, s, du);
    extrapolate(d.teth + 3 * fil, d.tethm1 + 3 * fil, d.tethm2 + 3 * fil, 3, nt);
    extrapolate(d.clamp + 3 * fil, d.clampm1 + 3 * fil, d.clampm2 + 3 * fil, 3, nt);
  } else {
    const size_t l = (size_t)3 * ((d.nseg - 1) * fil + j - 1);
    extrapolate(d.lam + l, d.lamm1 + l, d.lamm2 + l, 3, nt);
  }
}

// swimmer::update, one thread per segment: the base segment takes the
// updated body's Lie algebra element (accept_state_from_rigid_body) and adds
// the tether and clamp increments; segment j >= 1 adds its link's
// inextensibility increment and its Lie algebra increment (filament::update,
// filament.cpp:1896-1930). The robot arm follows (k_robot_arm).
__global__ void k_update_segments(StepDev d, BodyArgs b, const double *__restrict__ upd) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= d.ns) return;
  const int n = d.nseg, fil = s / n, j = s - fil * n;
  const double *uf = upd + (size_t)6 * n * fil;
  if (j == 0) {
    const double *u0 = d.u + 3 * s;
    const double du[3] = {b.u[0] - u0[0], b.u[1] - u0[1], b.u[2] - u0[2]};
    seg_update(d, s, du);
    for (int k = 0; k < 3; ++k) {
      d.teth[3 * fil + k] += uf[k];
      d.clamp[3 * fil + k] += uf[3 * n + k];
    }
  } else {
    double *lam = d.lam + (size_t)3 * ((n - 1) * fil + j - 1);
    for (int k = 0; k < 3; ++k) lam[k] += uf[3 * j + k];
    seg_update(d, s, uf + 3 * (n + j));
  }
}

// filament::internal_forces_and_torques (filament.cpp:1467-1575), one thread
// per segment, accumulating in the reference's order: link j-1 (its
// inextensibility force, the torque of that force about the segment, minus
// the link's elastic moment), then link j (the same with the opposite
// signs), then the tether force and clamping torque (base segment), the tip
// follower force (last segment) and the step-0 perturbation (segment 4).
// Written to the internal force array and to the solver's f_segs.
__global__ void k_forces(StepDev d, int nt) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= d.ns) return;
  const int n = d.nseg, fil = s / n, j = s - fil * n;
  const double *lamf = d.lam + (size_t)3 * (n - 1) * fil;
  const double strain[3] = {0.0, 0.0, 0.0};
  const Quat qj = load_q(d.q + 4 * s);
  double t[3];
  tangent(qj, t);
  double f[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  if (j > 0) {  // link j-1: this segment is its upper end
    const double *lam = lamf + 3 * (j - 1);
    for (int k = 0; k < 3; ++k) f[k] += lam[k];
    f[3] -= 0.5 * d.dl * (t[1] * lam[2] - t[2] * lam[1]);
    f[4] -= 0.5 * d.dl * (t[2] * lam[0] - t[0] * lam[2]);
    f[5] -= 0.5 * d.dl * (t[0] * lam[1] - t[1] * lam[0]);
    const Quat qi = load_q(d.q + 4 * (s - 1));
    double R[9], Mb[3], M[3];
    rot_mat(midpoint(qi, qj), R);
    link_moment(qi, qj, d.dl, d.kb, d.kt, strain, Mb);
    m3_vec(m3_from(R), Mb, M);
    for (int k = 0; k < 3; ++k) f[3 + k] -= M[k];
  }
  if (j < n - 1) {  // link j: this segment is its lower end
    const double *lam = lamf + 3 * j;
    for (int k = 0; k < 3; ++k) f[k] -= lam[k];
    f[3] -= 0.5 * d.dl * (t[1] * lam[2] - t[2] * lam[1]);
    f[4] -= 0.5 * d.dl * (t[2] * lam[0] - t[0] * lam[2]);
    f[5] -= 0.5 * d.dl * (t[0] * lam[1] - t[1] * lam[0]);
    const Quat qk = load_q(d.q + 4 * (s + 1));
    double R[9], Mb[3], M[3];
    rot_mat(midpoint(qj, qk), R);
    link_moment(qj, qk, d.dl, d.kb, d.kt, strain, Mb);
    m3_vec(m3_from(R), Mb, M);
    for (int k = 0; k < 3; ++k) f[3 + k] += M[k];
  }
  if (j == 0)
    for (int k = 0; k < 3; ++k) f[k] += d.teth[3 * fil + k];
  if (j == n - 1)
    for (int k = 0; k < 3; ++k) f[k] -= d.efm * t[k];
  if (nt == 0 && d.perturb && j == 4) f[0] += d.pert;  // filament.cpp:1540-1555
  if (j == 0) {
    double ct[3];
    dexpinv_s(ct, d.u + 3 * s, d.clamp + 3 * fil, 1.0);
    for (int k = 0; k < 3; ++k) f[3 + k] += ct[k];
  }
  for (int k = 0; k < 6; ++k) {
    d.f[6 * (size_t)s + k] = f[k];
    d.fs[6 * (size_t)s + k] = f[k];
  }
}

// This filament's part of the swimmer force, -sum (f ; (x - X) x f + torque)
// in segment order (swimmer.cpp:469-529), one warp per filament: the lanes
// form 32 segments' terms at a time, lane 0 subtracts them in order.
__global__ void __launch_bounds__(32 * kFilWarps) k_swimmer_force(StepDev d, double bx0,
                                                                  double bx1, double bx2,
                                                                  double *__restrict__ swf_part) {
  __shared__ double term[kFilWarps][32][6];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int fil = blockIdx.x * kFilWarps + w;
  if (fil >= d.nfil) return;  // the whole warp
  const int n = d.nseg, s0 = fil * n;
  double sw[6] = {0, 0, 0, 0, 0, 0};
  for (int j0 = 0; j0 < n; j0 += 32) {
    if (j0 + lane < n) {
      const double *fm = d.f + 6 * (size_t)(s0 + j0 + lane);
      const double *xm = d.x + 3 * (size_t)(s0 + j0 + lane);
      double *t = term[w][lane];
      t[0] = fm[0];
      t[1] = fm[1];
      t[2] = fm[2];
      const double xd = xm[0] - bx0, yd = xm[1] - bx1, zd = xm[2] - bx2;
      t[3] = fm[3] + yd * fm[2] - zd * fm[1];
      t[4] = fm[4] + zd * fm[0] - xd * fm[2];
      t[5] = fm[5] + xd * fm[1] - yd * fm[0];
    }
    __syncwarp();
    if (lane == 0) {
      const int m = min(32, n - j0);
      for (int q = 0; q < m; ++q)
        for (int k = 0; k < 6; ++k) sw[k] -= term[w][q][k];
    }
    __syncwarp();
  }
  if (lane == 0)
    for (int k = 0; k < 6; ++k) swf_part[6 * fil + k] = sw[k];
}

// swimmer::f = the sum of the filaments' partial force and torque sums
// (swimmer.cpp:469-529): warp k adds component k over the
// filaments, lanes strided, then a fixed shuffle tree.
__global__ void k_swimmer_sum(const double *__restrict__ part, int nfil, double *__restrict__ out) {
  const int lane = threadIdx.x & 31, k = threadIdx.x >> 5;
  double s = 0.0;
  for (int i = lane; i < nfil; i += 32) s += part[6 * (size_t)i + k];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) out[k] = s;
}

// BDF residuals (mobility_solver.cpp:2661-2946), one thread per segment; the
// body's six entries by thread 0. Sets bit 0 of *flag if any entry exceeds
// the tolerance (TOL DL for positions, TOL for Lie-algebra elements) and
// bit 1 if any entry is not finite.
__global__ void k_errors(StepDev d, BodyArgs b, int nt, double tol, const double *__restrict__ v_segs,
                         const double *__restrict__ v_bodies, double *__restrict__ err,
                         int *__restrict__ flag) {
  const double c1 = -4.0 / 3.0, c2 = 1.0 / 3.0, c3 = -2.0 / 3.0;
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  bool big = false, bad = false;
  if (s < d.ns) {
    const int fil = s / d.nseg, j = s - fil * d.nseg;
    const double *v = v_segs + 6 * (size_t)s, *w = v + 3;
    const double *x = d.x + 3 * s, *xm1 = d.xm1 + 3 * s, *xm2 = d.xm2 + 3 * s;
    const size_t id = (size_t)6 * d.nseg * fil + 3 * j;
    for (int k = 0; k < 3; ++k) {
      const double e = nt < 1 ? x[k] - xm1[k] - d.dt * v[k]
                              : x[k] + c1 * xm1[k] + c2 * xm2[k] + c3 * d.dt * v[k];
      err[id + k] = e;
      big |= fabs(e) > d.dl * tol;
      bad |= !isfinite(e);
    }
    double W[3];
    const double *u = d.u + 3 * s, *um1 = d.um1 + 3 * s;
    dexpinv_s(W, u, w, -1.0);
    for (int k = 0; k < 3; ++k) {
      const double e = nt < 1 ? u[k] - d.dt * W[k] : u[k] - c2 * um1[k] + c3 * d.dt * W[k];
      err[id + 3 * d.nseg + k] = e;
      big |= fabs(e) > tol;
      bad |= !isfinite(e);
    }
  }
  if (s == 0) {
    const size_t id = (size_t)6 * d.ns;
    double w[3];
    dexpinv_s(w, b.u, v_bodies + 3, -1.0);
    for (int k = 0; k < 3; ++k) {
      const double ex = nt < 1 ? b.x[k] - b.xm1[k] - d.dt * v_bodies[k]
                               : b.x[k] + c1 * b.xm1[k] + c2 * b.xm2[k] + c3 * d.dt * v_bodies[k];
      const double eu = nt < 1 ? b.u[k] - d.dt * w[k] : b.u[k] - c2 * b.um1[k] + c3 * d.dt * w[k];
      err[id + k] = ex;
      err[id + 3 + k] = eu;
      big |= fabs(ex) > tol * d.dl;
      big |= fabs(eu) > tol;
      bad |= !isfinite(ex) || !isfinite(eu);
    }
  }
  const int bits = (__any_sync(0xffffffffu, big) ? 1 : 0) | (__any_sync(0xffffffffu, bad) ? 2 : 0);
  if (bits && (threadIdx.x & 31) == 0) atomicOr(flag, bits);
}

// ---------------------------------------------------------------------------
// approximate Jacobian (filament::invert_approx_jacobian, filament.cpp:1761-1894;
// jacobian_lie_algebra_block, :1577-1759) and the body coupling blocks
// (swimmer::prepare_jacobian_inv, swimmer.cpp:535-913)
// ---------------------------------------------------------------------------

struct SegFrame {
  Quat q;
  double t[3], n[3], b[3];
};

__device__ SegFrame seg_frame(const StepDev &d, int s) {
  SegFrame f;
  f.q = load_q(d.q + 4 * s);
  tangent(f.q, f.t);
  normal(f.q, f.n);
  binormal(f.q, f.b);
  return f;
}

// sign * 0.5 (K0 rcross(t) + K1 rcross(n) + K2 rcross(b))
__device__ M3 frame_comb(double sign, const double *K, const SegFrame &f) {
  const M3 a = m3_add(m3_add(m3_scale(K[0], rcross(f.t)), m3_scale(K[1], rcross(f.n))),
                      m3_scale(K[2], rcross(f.b)));
  return m3_scale(sign * 0.5, a);
}

// -tsf (dO - 0.5 (OM + L dO) + (rcross(OM u) + L OM + L L dO)/12)
__device__ M3 diag_block(double tsf, const M3 &dO, const M3 &OM, const M3 &L, const double *u) {
  double omu[3];
  m3_vec(OM, u, omu);
  const M3 LdO = m3_mul(L, dO);
  M3 t = m3_sub(dO, m3_scale(0.5, m3_add(OM, LdO)));
  const M3 r = m3_add(m3_add(rcross(omu), m3_mul(L, OM)), m3_mul(m3_mul(L, L), dO));
  t = m3_add(t, m3_div(r, 12.0));
  return m3_scale(-tsf, t);
}

// -tsf (dO - 0.5 L dO + L L dO / 12)
__device__ M3 off_block(double tsf, const M3 &dO, const M3 &L) {
  M3 t = m3_sub(dO, m3_mul(m3_scale(0.5, L), dO));
  t = m3_add(t, m3_div(m3_mul(m3_mul(L, L), dO), 12.0));
  return m3_scale(-tsf, t);
}

__device__ void put_block(double *J, int ld, int r0, int c0, const M3 &m) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) J[(size_t)(r0 + i) * ld + c0 + j] = m.a[3 * i + j];
}

// Row block k of the Lie-algebra block E (its diagonal including the
// identity, and the blocks to segments k-1 and k+1), written into J at
// rows 3 (N + k), columns 3 (N + k - 1 .. k + 1).
__device__ void lie_rows(const StepDev &d, int fil, int k, int nt, double *J) {
  const int n = d.nseg, n6 = 6 * n, s0 = fil * n;
  const double tsf = nt < 1 ? d.dt : 2.0 * d.dt / 3.0;
  const double Tfac = 1.0 / (8.0 * kPiS * d.mu * d.a * d.a * d.a);
  const double strain[3] = {0.0, 0.0, 0.0};
  const double *f = d.f + (size_t)6 * (s0 + k);
  const double *u = d.u + 3 * (s0 + k);
  const double *lam = d.lam + (size_t)3 * (n - 1) * fil;
  const SegFrame fk = seg_frame(d, s0 + k);
  const M3 L = m3_scale(-1.0, rcross(u));
  const double om[3] = {Tfac * f[3], Tfac * f[4], Tfac * f[5]};
  const M3 OM = rcross(om);
  const int r0 = 3 * (n + k);
  M3 diag_el = m3_zero();
  double lamvec[3];
  if (k == 0) {
    for (int c = 0; c < 3; ++c) lamvec[c] = lam[c];
  } else if (k == n - 1) {
    for (int c = 0; c < 3; ++c) lamvec[c] = lam[3 * (n - 2) + c];
  } else {
    for (int c = 0; c < 3; ++c) lamvec[c] = lam[3 * (k - 1) + c] + lam[3 * k + c];
  }
  const M3 constraint = m3_mul(m3_scale(-0.5 * d.dl, rcross(lamvec)), rcross(fk.t));
  if (k < n - 1) {  // the link to segment k+1
    const SegFrame fp = seg_frame(d, s0 + k + 1);
    double Kph[3], R[9];
    link_moment(fk.q, fp.q, d.dl, d.kb, d.kt, strain, Kph);
    rot_mat(midpoint(fk.q, fp.q), R);
    const M3 Rm = m3_from(R);
    M3 el = m3_add(frame_comb(1.0, Kph, fk),
                   m3_mul(Rm, link_moment_lie_derivative(fk.q, fp.q, false, d.dl, d.kb, d.kt)));
    diag_el = el;
    // right off-diagonal block
    el = m3_add(frame_comb(1.0, Kph, fp),
                m3_mul(Rm, link_moment_lie_derivative(fk.q, fp.q, true, d.dl, d.kb, d.kt)));
    put_block(J, n6, r0, r0 + 3, off_block(tsf, m3_scale(Tfac, el), L));
  }
  if (k > 0) {  // the link to segment k-1
    const SegFrame fm = seg_frame(d, s0 + k - 1);
    double Kmh[3], R[9];
    link_moment(fm.q, fk.q, d.dl, d.kb, d.kt, strain, Kmh);
    rot_mat(midpoint(fm.q, fk.q), R);
    const M3 Rm = m3_from(R);
    const M3 RL = m3_mul(Rm, link_moment_lie_derivative(fm.q, fk.q, true, d.dl, d.kb, d.kt));
    diag_el = k < n - 1 ? m3_sub(m3_add(diag_el, frame_comb(-1.0, Kmh, fk)), RL)
                        : m3_sub(frame_comb(-1.0, Kmh, fk), RL);

    // left off-diagonal block
    const M3 el = m3_sub(frame_comb(-1.0, Kmh, fm),
                m3_mul(Rm, link_moment_lie_derivative(fm.q, fk.q, false, d.dl, d.kb, d.kt)));
    put_block(J, n6, r0, r0 - 3, off_block(tsf, m3_scale(Tfac, el), L));
  }
  const M3 dO = m3_scale(Tfac, m3_add(diag_el, constraint));
  M3 blk = diag_block(tsf, dO, OM, L, u);
  blk.a[0] += 1.0;
  blk.a[4] += 1.0;
  blk.a[8] += 1.0;
  put_block(J, n6, r0, r0, blk);
}

// The RPY blocks between the body (a sphere of radius R) and segment m.
struct SphereBlocks {
  M3 tt, tr, rr, temp;
};

__device__ SphereBlocks sphere_blocks(const StepDev &d, const BodyArgs &b, int s) {
  SphereBlocks o;
  const double *x = d.x + 3 * s;
  double rh[3] = {x[0] - b.x[0], x[1] - b.x[1], x[2] - b.x[2]};
  const double r = sqrt(rh[0] * rh[0] + rh[1] * rh[1] + rh[2] * rh[2]);
  rh[0] /= r;
  rh[1] /= r;
  rh[2] /= r;
  M3 rr;
  rr.a[0] = rh[0] * rh[0];
  rr.a[4] = rh[1] * rh[1];
  rr.a[8] = rh[2] * rh[2];
  rr.a[1] = rr.a[3] = rh[0] * rh[1];
  rr.a[2] = rr.a[6] = rh[0] * rh[2];
  rr.a[5] = rr.a[7] = rh[2] * rh[1];
  const M3 I = m3_eye();
  const double R2a2 = d.body_r * d.body_r + d.a * d.a;
  o.tt = m3_div(m3_add(m3_scale(1.0 + R2a2 / (3.0 * r * r), I), m3_scale(1.0 - R2a2 / (r * r), rr)),
                8.0 * kPiS * d.mu * r);
  o.tr = m3_div(rcross(rh), 8.0 * kPiS * d.mu * r * r);
  o.rr = m3_div(m3_sub(m3_scale(3.0, rr), I), 16.0 * kPiS * d.mu * r * r * r);
  double t[3];
  tangent(load_q(d.q + 4 * s), t);
  o.temp = rcross(t);
  return o;
}

// Column block cb (3 columns) of the 6 x 6N coupling block B of the body's
// Lie-algebra equations to this filament's unknowns (swimmer.cpp:760-854),
// before the multiplication by the inverse Jacobian. top/bot = rows 0..2 / 3..5.
__device__ void body_block_column(const StepDev &d, const BodyArgs &b, int fil, int cb, M3 &top,
                                  M3 &bot) {
  const int n = d.nseg, s0 = fil * n;
  const double *ref = d.fil_refs + 3 * fil;
  double fbd[3];
  m3_vec(m3_from(b.Q), ref, fbd);
  double tl[3];
  tangent(load_q(d.q + 4 * (s0 + n - 1)), tl);
  const double eft[3] = {d.efm * tl[0], d.efm * tl[1], d.efm * tl[2]};
  const M3 Ef = rcross(eft);
  M3 t0 = m3_zero(), b0 = m3_zero();
  if (cb == 0) {
    t0 = m3_scale(-1.0, m3_eye());
    b0 = rcross(fbd);
  } else if (cb == n) {
    b0 = m3_scale(-1.0, m3_from(b.DinvT));
  } else if (cb == 2 * n - 1) {
    const double *xl = d.x + 3 * (s0 + n - 1);
    const double v[3] = {0.5 * d.dl * tl[0] - (xl[0] - b.x[0]), 0.5 * d.dl * tl[1] - (xl[1] - b.x[1]),
                         0.5 * d.dl * tl[2] - (xl[2] - b.x[2])};
    t0 = Ef;
    b0 = m3_mul(rcross(v), Ef);
  } else if (cb > n) {
    double t[3];
    tangent(load_q(d.q + 4 * (s0 + cb - n)), t);
    const double v[3] = {d.dl * t[0], d.dl * t[1], d.dl * t[2]};
    b0 = m3_mul(Ef, rcross(v));
  }
  // body mobility (rotated by the step's initial orientation) times the block
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double st = 0.0, sb = 0.0;
      for (int k = 0; k < 3; ++k) {
        st += b.BM[6 * i + k] * t0.a[3 * k + j];
        sb += b.BM[6 * (i + 3) + k] * t0.a[3 * k + j];
      }
      for (int k = 0; k < 3; ++k) {
        st += b.BM[6 * i + 3 + k] * b0.a[3 * k + j];
        sb += b.BM[6 * (i + 3) + 3 + k] * b0.a[3 * k + j];
      }
      top.a[3 * i + j] = st;
      bot.a[3 * i + j] = sb;
    }
  // sphere corrections from the RPY blocks of the segments involved
  const double hdl = 0.5 * d.dl;
  if (cb == 0) {
    const SphereBlocks m = sphere_blocks(d, b, s0);
    top = m3_add(top, m.tt);
    bot = m3_add(bot, m.tr);
  } else if (cb == n) {
    const SphereBlocks m = sphere_blocks(d, b, s0);
    const M3 DT = m3_from(b.DinvT);
    top = m3_add(top, m3_mul(m.tr, DT));
    bot = m3_add(bot, m3_mul(m.rr, DT));
  } else if (cb == 2 * n - 1) {
    const SphereBlocks m = sphere_blocks(d, b, s0 + n - 1);
    top = m3_add(top, m3_mul(m3_scale(-d.efm, m.tt), m.temp));
    bot = m3_add(bot, m3_mul(m3_scale(-d.efm, m.tr), m.temp));
  } else if (cb < n) {  // link cb - 1: segments cb - 1 (minus form) and cb (plus form)
    const SphereBlocks m1 = sphere_blocks(d, b, s0 + cb - 1);
    top = m3_add(top, m3_sub(m3_mul(m3_scale(hdl, m1.tr), m1.temp), m1.tt));
    bot = m3_add(bot, m3_sub(m3_mul(m3_scale(hdl, m1.rr), m1.temp), m1.tr));
    const SphereBlocks m2 = sphere_blocks(d, b, s0 + cb);
    top = m3_add(top, m3_add(m3_mul(m3_scale(hdl, m2.tr), m2.temp), m2.tt));
    bot = m3_add(bot, m3_add(m3_mul(m3_scale(hdl, m2.rr), m2.temp), m2.tr));
  }
  bot = m3_mul(m3_from(b.Dinv), bot);
  top = m3_scale(b.dt_fac, top);
  bot = m3_scale(b.dt_fac, bot);
}

__device__ M3 base_cross(const StepDev &d, const BodyArgs &b, int fil) {
  double fbd[3];
  m3_vec(m3_from(b.Q), d.fil_refs + 3 * fil, fbd);
  const double dn = sqrt(fbd[0] * fbd[0] + fbd[1] * fbd[1] + fbd[2] * fbd[2]);
  const double s = 0.5 * d.dl + dn;
  const double v[3] = {s * fbd[0] / dn, s * fbd[1] / dn, s * fbd[2] / dn};
  return rcross(v);
}

// JB A and the body's Lie-algebra self-dependence for filament fil, from the
// stored JB (after a CTA barrier).
__device__ void jac_tail(const StepDev &d, const BodyArgs &b, int fil, int n6, int n) {
  const int tid = threadIdx.x;
  const int s0 = fil * n;
  const double *jb = d.jb + (size_t)6 * n6 * fil;
  // JB A (6 x 6) with A = [I, D] per segment row block plus the elastic clamping blocks
  if (tid < 36) {
    const int r = tid / 6, c = tid % 6;
    const M3 D = base_cross(d, b, fil);
    const double *e1 = d.ecb + 18 * fil, *e2 = e1 + 9;
    const double *row = jb + (size_t)r * n6;
    double s = 0.0;
    for (int k = 0; k < 3 * n; ++k) {
      const int m = k % 3;
      s += row[k] * (c < 3 ? (m == c ? 1.0 : 0.0) : D.a[3 * m + c - 3]);
    }
    if (c >= 3) {
      for (int m = 0; m < 3; ++m) s += row[3 * n + m] * e1[3 * m + c - 3];
      for (int m = 0; m < 3; ++m) s += row[3 * n + 3 + m] * e2[3 * m + c - 3];
    }
    d.part[45 * fil + tid] = s;
  }
  if (tid == 64) {  // this filament's share of the body's Lie-algebra self-dependence
    double fbd[3];
    m3_vec(m3_from(b.Q), d.fil_refs + 3 * fil, fbd);
    const double *tl = d.teth + 3 * fil, *cl = d.clamp + 3 * fil;
    const double ucl[3] = {b.u[1] * cl[2] - b.u[2] * cl[1], b.u[2] * cl[0] - b.u[0] * cl[2],
                           b.u[0] * cl[1] - b.u[1] * cl[0]};
    M3 o = m3_scale(-1.0, m3_mul(rcross(tl), rcross(fbd)));
    o = m3_add(o, m3_sub(m3_scale(0.5, rcross(cl)),
                         m3_div(m3_add(rcross(ucl), m3_mul(m3_from(b.blc), rcross(cl))), 12.0)));
    double t[3];
    tangent(load_q(d.q + 4 * (s0 + n - 1)), t);
    const double et[3] = {d.efm * t[0], d.efm * t[1], d.efm * t[2]};
    o = m3_add(o, m3_mul(rcross(et), base_cross(d, b, fil)));
    for (int k = 0; k < 9; ++k) d.part[45 * fil + 36 + k] = o.a[k];
  }
}

// Element arithmetic of the low-precision inversion (FP32).
struct GjF32 {
  using E = float;
  static __device__ __forceinline__ E zero() { return 0.f; }
  static __device__ __forceinline__ float mag(E a) { return fabsf(a); }
  static __device__ __forceinline__ E recip(E a) { return 1.0f / a; }
  static __device__ __forceinline__ E mul(E a, E b) { return a * b; }
  static __device__ __forceinline__ E neg_mul(E c, E r) { return -(c * r); }
  static __device__ __forceinline__ E sub_mul(E x, E c, E r) { return fmaf(-c, r, x); }
  static __device__ __forceinline__ void acc(E &s, E a, E b) { s = fmaf(a, b, s); }
  static __device__ __forceinline__ E from(double v) { return (float)v; }
  static __device__ __forceinline__ double to(E a) { return (double)a; }
};

// Gauss-Jordan inversion in place of the n6 x n6 matrix in shared memory
// (row-major, elements of Ops), by the whole CTA. The same steps as the FP64
// elimination below: partial pivoting on the largest |entry| of the column
// at or below the diagonal (first index on ties), the pivot row scaled by
// 1/piv (its own entry becoming 1/piv), every other row i minus col_i times
// the pivot row (column k becoming -col_i / piv), and the columns
// unscrambled at the end.
template <class Ops>
__device__ void gj_invert_lo(typename Ops::E *J, int n6, typename Ops::E *col, int *perm) {
  using E = typename Ops::E;
  const int tid = threadIdx.x, nth = blockDim.x, warp = tid >> 5, lane = tid & 31;
  __shared__ E rp_s;
  __syncthreads();
  const int ng = nth / n6 > 0 ? nth / n6 : 1;
  const int g = tid / n6, jcol = g < ng ? tid - g * n6 : n6;
  for (int k = 0; k < n6; ++k) {
    if (warp == 0) {
      float best = -1.0f;
      int bi = k;
      for (int i = k + lane; i < n6; i += 32) {
        const float v = Ops::mag(J[(size_t)i * n6 + k]);
        if (v > best) {
          best = v;
          bi = i;
        }
      }
      for (int off = 16; off > 0; off >>= 1) {
        const float ov = __shfl_down_sync(0xffffffffu, best, off);
        const int oi = __shfl_down_sync(0xffffffffu, bi, off);
        if (ov > best || (ov == best && oi < bi)) {
          best = ov;
          bi = oi;
        }
      }
      if (lane == 0) perm[k] = bi;
    }
    __syncthreads();
    const int p = perm[k];
    if (p != k)
      for (int j = tid; j < n6; j += nth) {
        const E t = J[(size_t)k * n6 + j];
        J[(size_t)k * n6 + j] = J[(size_t)p * n6 + j];
        J[(size_t)p * n6 + j] = t;
      }
    __syncthreads();
    for (int i = tid; i < n6; i += nth) col[i] = i == k ? Ops::zero() : J[(size_t)i * n6 + k];
    if (tid == 0) rp_s = Ops::recip(J[(size_t)k * n6 + k]);
    __syncthreads();
    const E rp = rp_s;
    for (int j = tid; j < n6; j += nth)
      J[(size_t)k * n6 + j] = j == k ? rp : Ops::mul(J[(size_t)k * n6 + j], rp);
    __syncthreads();
    if (jcol < n6) {
      const E rk = J[k * n6 + jcol];
      E *q = J + g * n6 + jcol;  // rows g, g + ng, ... of column jcol
      const int st = ng * n6;
      if (jcol != k) {
        // col[k] = 0 leaves the pivot row as it is; four rows at a time,
        // their loads issued together
        int i = g;
        for (; i + 3 * ng < n6; i += 4 * ng, q += 4 * st) {
          const E c0 = col[i], c1 = col[i + ng], c2 = col[i + 2 * ng], c3 = col[i + 3 * ng];
          const E x0 = q[0], x1 = q[st], x2 = q[2 * st], x3 = q[3 * st];
          q[0] = Ops::sub_mul(x0, c0, rk);
          q[st] = Ops::sub_mul(x1, c1, rk);
          q[2 * st] = Ops::sub_mul(x2, c2, rk);
          q[3 * st] = Ops::sub_mul(x3, c3, rk);
        }
        for (; i < n6; i += ng, q += st) q[0] = Ops::sub_mul(q[0], col[i], rk);
      } else {
        for (int i = g; i < n6; i += ng, q += st)
          if (i != k) q[0] = Ops::neg_mul(col[i], rk);
      }
    }
    __syncthreads();
  }
  for (int k = n6 - 1; k >= 0; --k) {
    const int p = perm[k];
    if (p != k)
      for (int i = tid; i < n6; i += nth) {
        const E t = J[(size_t)i * n6 + k];
        J[(size_t)i * n6 + k] = J[(size_t)i * n6 + p];
        J[(size_t)i * n6 + p] = t;
      }
    __syncthreads();
  }
}

// One CTA per filament: assemble the approximate Jacobian in shared memory,
// invert it in place (Gauss-Jordan, partial pivoting), store the inverse,
// the product JB = B J^-1 and this filament's share of the Schur complement
// (JB A) and of the body's Lie-algebra self-dependence. With kFF (FP32C
// solvers) J and B are assembled in their global slots instead (no shared
// memory: launched with few threads, several CTAs share an SM and overlap
// the FP64 chains of the assembly) and k_jacobian_lo inverts.
template <bool kFF>
__global__ void __launch_bounds__(256) k_jacobian(StepDev d, BodyArgs b, int nt) {
  extern __shared__ double sm[];
  const int n = d.nseg, n6 = 6 * n, fil = blockIdx.x, tid = threadIdx.x, nth = blockDim.x;
  double *J = kFF ? d.jinv + (size_t)n6 * n6 * fil : sm;          // n6 * n6
  double *Bm = kFF ? d.jb + (size_t)6 * n6 * fil : J + (size_t)n6 * n6;  // 6 * n6
  double *col = kFF ? sm : Bm + 6 * n6;  // n6 (the inversion's; unused with kFF)
  double *red = col + n6;                  // 32 (pivot search) + 8
  int *perm = reinterpret_cast<int *>(red + 40);
  const int s0 = fil * n;
  for (int i = tid; i < n6 * n6; i += nth) J[i] = 0.0;
  __syncthreads();
  // position rows: multipliers (diagonal bands) and Lie-algebra columns
  const double fac = nt < 1 ? -d.dt / (6.0 * kPiS * d.mu * d.a) : -d.dt / (9.0 * kPiS * d.mu * d.a);
  for (int i = tid; i < 3 * n; i += nth) {
    J[(size_t)i * n6 + i] = fac;
    if (i < 3 * n - 3) J[(size_t)i * n6 + i + 3] = -fac;
  }
  const double fac2 = nt < 1 ? d.dl * d.dt / (16.0 * kPiS * d.mu * d.a * d.a * d.a)
                             : d.dl * d.dt / (24.0 * kPiS * d.mu * d.a * d.a * d.a);
  for (int j = tid; j < n; j += nth) {
    if (j >= 1) {
      double t[3];
      tangent(load_q(d.q + 4 * (s0 + j)), t);
      const M3 temp = m3_scale(d.dl, rcross(t));
      const int jpos = 3 * (n + j);
      put_block(J, n6, 3 * j, jpos, m3_scale(0.5, temp));
      for (int i = j + 1; i < n; ++i) put_block(J, n6, 3 * i, jpos, temp);
      if (j == n - 1) {
        const M3 e = m3_scale(fac * d.efm, rcross(t));
        for (int r = 0; r < 3; ++r)
          for (int c = 0; c < 3; ++c) J[(size_t)(3 * j + r) * n6 + jpos + c] -= e.a[3 * r + c];
      }
      // Lie rows of segments j-1 and j on the multiplier of link j-1
      for (int h = 0; h < 2; ++h) {
        const int sg = s0 + j - 1 + h;
        double tt[3];
        tangent(load_q(d.q + 4 * sg), tt);
        const M3 um = rcross(d.u + 3 * sg);
        const M3 tm = m3_scale(-1.0, rcross(tt));
        const M3 blk = m3_scale(
            fac2, m3_add(m3_add(tm, m3_mul(m3_scale(0.5, um), tm)), m3_div(m3_mul(m3_mul(um, um), tm), 12.0)));
        put_block(J, n6, 3 * (n + j - 1 + h), 3 * j, blk);
      }
    }
    lie_rows(d, fil, j, nt, J);
  }
  // coupling block B, column blocks in parallel
  for (int cb = tid; cb < 2 * n; cb += nth) {
    M3 top, bot;
    body_block_column(d, b, fil, cb, top, bot);
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) {
        Bm[r * n6 + 3 * cb + c] = top.a[3 * r + c];
        Bm[(r + 3) * n6 + 3 * cb + c] = bot.a[3 * r + c];
      }
  }
  __syncthreads();
  if (tid == 0) {  // the clamped base: keep the elastic blocks, replace the first Lie column
    double *ecb = d.ecb + 18 * fil;
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) {
        ecb[3 * r + c] = J[(size_t)(3 * n + r) * n6 + 3 * n + c];
        ecb[9 + 3 * r + c] = J[(size_t)(3 * n + 3 + r) * n6 + 3 * n + c];
      }
    const double fac3 = nt < 1 ? -d.dt / (8.0 * kPiS * d.mu * d.a * d.a * d.a)
                               : -d.dt / (12.0 * kPiS * d.mu * d.a * d.a * d.a);
    const M3 um = rcross(d.u + 3 * s0);
    const M3 uu12 = m3_div(m3_mul(um, um), 12.0);
    M3 blk = m3_add(m3_scale(0.5, um), uu12);
    M3 blkT = m3_add(m3_scale(-0.5, um), uu12);
    for (int c = 0; c < 3; ++c) {
      blk.a[4 * c] += 1.0;
      blkT.a[4 * c] += 1.0;
    }
    put_block(J, n6, 3 * n, 3 * n, m3_mul(m3_scale(fac3, blk), blkT));
    put_block(J, n6, 3 * n + 3, 3 * n, m3_zero());
  }
  __syncthreads();
  if constexpr (kFF) return;  // J and B are in global memory; k_jacobian_lo inverts
  // Gauss-Jordan inversion in place
  const int warp = tid >> 5, lane = tid & 31;
  const int ng = nth / n6 > 0 ? nth / n6 : 1;  // row groups
  const int g = tid / n6, jcol = g < ng ? tid - g * n6 : n6;
  for (int k = 0; k < n6; ++k) {
    if (warp == 0) {
      double best = -1.0;
      int bi = k;
      for (int i = k + lane; i < n6; i += 32) {
        const double v = fabs(J[(size_t)i * n6 + k]);
        if (v > best) {
          best = v;
          bi = i;
        }
      }
      for (int off = 16; off > 0; off >>= 1) {
        const double ov = __shfl_down_sync(0xffffffffu, best, off);
        const int oi = __shfl_down_sync(0xffffffffu, bi, off);
        if (ov > best || (ov == best && oi < bi)) {
          best = ov;
          bi = oi;
        }
      }
      if (lane == 0) perm[k] = bi;
    }
    __syncthreads();
    const int p = perm[k];
    if (p != k)
      for (int j = tid; j < n6; j += nth) {
        const double t = J[(size_t)k * n6 + j];
        J[(size_t)k * n6 + j] = J[(size_t)p * n6 + j];
        J[(size_t)p * n6 + j] = t;
      }
    __syncthreads();
    const double piv = J[(size_t)k * n6 + k];
    for (int i = tid; i < n6; i += nth) col[i] = i == k ? 0.0 : J[(size_t)i * n6 + k];
    __syncthreads();
    for (int j = tid; j < n6; j += nth) J[(size_t)k * n6 + j] = j == k ? 1.0 / piv : J[(size_t)k * n6 + j] / piv;
    __syncthreads();
    // thread (g, j) owns column j of rows g, g + ng, ...: the pivot row's
    // entry stays in a register and col[i] is a broadcast read
    if (jcol < n6) {
      const double rk = J[(size_t)k * n6 + jcol];
      if (jcol == k) {
        for (int i = g; i < n6; i += ng)
          if (i != k) J[(size_t)i * n6 + jcol] = -col[i] * rk;
      } else {
        for (int i = g; i < n6; i += ng)
          if (i != k) J[(size_t)i * n6 + jcol] -= col[i] * rk;
      }
    }
    __syncthreads();
  }
  for (int k = n6 - 1; k >= 0; --k) {
    const int p = perm[k];
    if (p != k)
      for (int i = tid; i < n6; i += nth) {
        const double t = J[(size_t)i * n6 + k];
        J[(size_t)i * n6 + k] = J[(size_t)i * n6 + p];
        J[(size_t)i * n6 + p] = t;
      }
    __syncthreads();
  }
  double *jinv = d.jinv + (size_t)n6 * n6 * fil;
  for (int i = tid; i < n6 * n6; i += nth) jinv[i] = J[i];
  // JB = B J^-1 (6 x n6)
  double *jb = d.jb + (size_t)6 * n6 * fil;
  for (int idx = tid; idx < 6 * n6; idx += nth) {
    const int r = idx / n6, c = idx - r * n6;
    double s = 0.0;
    for (int k = 0; k < n6; ++k) s += Bm[r * n6 + k] * J[(size_t)k * n6 + c];
    jb[idx] = s;
  }
  __syncthreads();
  jac_tail(d, b, fil, n6, n);
}

// The low-precision half of the FP32C approximate Jacobian: one CTA per
// filament of kJacLoThreads threads (a separate kernel, so that the
// elimination runs with many warps and few registers): J and B as k_jacobian
// left them in jinv and jb (FP64), J^-1 in place in Ops arithmetic,
// JB = B J^-1, then this filament's Schur and body partials. The inverse
// only seeds Broyden's method (its initial inverse Jacobian): FP32 elements
// keep the reference's Broyden iteration counts (tested at DT 1e-3 and at
// the reference's default DT) at a third of the float-float form's time.
constexpr int kJacLoThreads = 512;
constexpr int kJacAsmThreads = 64;  // k_jacobian<true>: assembly only
template <class Ops>
__global__ void __launch_bounds__(kJacLoThreads) k_jacobian_lo(StepDev d, BodyArgs b) {
  using E = typename Ops::E;
  extern __shared__ double sm[];
  const int n = d.nseg, n6 = 6 * n, fil = blockIdx.x, tid = threadIdx.x, nth = blockDim.x;
  E *J = reinterpret_cast<E *>(sm);   // n6 * n6
  E *Bf = J + (size_t)n6 * n6;        // 6 * n6
  E *col = Bf + 6 * n6;               // n6
  int *perm = reinterpret_cast<int *>(col + n6);
  double *jg = d.jinv + (size_t)n6 * n6 * fil, *bg = d.jb + (size_t)6 * n6 * fil;
  for (int i = tid; i < n6 * n6; i += nth) J[i] = Ops::from(jg[i]);
  for (int i = tid; i < 6 * n6; i += nth) Bf[i] = Ops::from(bg[i]);
  gj_invert_lo<Ops>(J, n6, col, perm);
  E *jo = reinterpret_cast<E *>(jg);  // J^-1 as E at the start of the filament's slot
  for (int i = tid; i < n6 * n6; i += nth) jo[i] = J[i];
  for (int idx = tid; idx < 6 * n6; idx += nth) {
    const int r = idx / n6, c = idx - r * n6;
    E s0 = Ops::zero(), s1 = Ops::zero();
    int k = 0;
    for (; k + 1 < n6; k += 2) {
      Ops::acc(s0, Bf[r * n6 + k], J[(size_t)k * n6 + c]);
      Ops::acc(s1, Bf[r * n6 + k + 1], J[(size_t)(k + 1) * n6 + c]);
    }
    if (k < n6) Ops::acc(s0, Bf[r * n6 + k], J[(size_t)k * n6 + c]);
    bg[idx] = Ops::to(s0) + Ops::to(s1);
  }
  __syncthreads();
  jac_tail(d, b, fil, n6, n);
}
using JacLoOps = GjF32;  // the arithmetic FP32C solvers invert in

// ---------------------------------------------------------------------------
// swimmer::jacobian_inv_mult (swimmer.cpp:915-1070), free-body branch:
//   b2 = in_body - sum_i JB_i in_i,  out_body = S^-1 b2,
//   out_i = J_i^-1 (in_i - A_i out_body)
// ---------------------------------------------------------------------------

// p6[6 fil + r] = (JB_i in_i)_r, one warp per row r
__global__ void k_jb_dot(StepDev d, const double *__restrict__ in, double *__restrict__ p6) {
  const int fil = blockIdx.x, r = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int n6 = 6 * d.nseg;
  const double *jb = d.jb + (size_t)6 * n6 * fil + (size_t)r * n6;
  const double *v = in + (size_t)n6 * fil;
  double s = 0.0;
  for (int k = lane; k < n6; k += 32) s += jb[k] * v[k];
  for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
  if (lane == 0) p6[6 * fil + r] = s;
}

// b2 = in_body - sum_i JB_i in_i and the body's part of the output
// S^-1 b2 (one CTA; the filament partials summed by a fixed tree)
__global__ void __launch_bounds__(256) k_body_solve(StepDev d, const double *__restrict__ in,
                                                    const double *__restrict__ p6,
                                                    const double *__restrict__ schur_inv,
                                                    double *__restrict__ out, double *__restrict__ ob) {
  __shared__ double sh[8][6];
  __shared__ double b2[6];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  double acc[6] = {0, 0, 0, 0, 0, 0};
  for (int i = tid; i < d.nfil; i += blockDim.x)
    for (int r = 0; r < 6; ++r) acc[r] += p6[6 * i + r];
  for (int r = 0; r < 6; ++r) {
    double v = acc[r];
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    if (lane == 0) sh[warp][r] = v;
  }
  __syncthreads();
  const size_t nb = (size_t)6 * d.ns;
  if (tid < 6) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sh[w][tid];
    b2[tid] = in[nb + tid] - t;
  }
  __syncthreads();
  if (tid < 6) {
    double v = 0.0;
    for (int c = 0; c < 6; ++c) v += schur_inv[6 * tid + c] * b2[c];
    out[nb + tid] = v;
    ob[tid] = v;
  }
}

// out_i = J_i^-1 (in_i - A_i ob), one CTA per filament, one warp per row
// J^-1 is stored as T per filament at the start of its (6N)^2-double slot
// (FP32 for FP32C solvers, whose inverse is computed in FP32).
template <typename T>
__global__ void k_jinv_apply(StepDev d, BodyArgs b, const double *__restrict__ in,
                             const double *__restrict__ ob_dev, double *__restrict__ out) {
  extern __shared__ double rhs_sm[];
  T *rhs = reinterpret_cast<T *>(rhs_sm);
  const int fil = blockIdx.x, n = d.nseg, n6 = 6 * n;
  const double *v = in + (size_t)n6 * fil;
  double ob[6];
  for (int k = 0; k < 6; ++k) ob[k] = ob_dev[k];
  const M3 D = base_cross(d, b, fil);
  const double *e1 = d.ecb + 18 * fil, *e2 = e1 + 9;
  for (int k = threadIdx.x; k < n6; k += blockDim.x) {
    double a = 0.0;
    if (k < 3 * n) {
      const int m = k % 3;
      a = ob[m] + D.a[3 * m] * ob[3] + D.a[3 * m + 1] * ob[4] + D.a[3 * m + 2] * ob[5];
    } else if (k < 3 * n + 6) {
      const double *e = k < 3 * n + 3 ? e1 + 3 * (k - 3 * n) : e2 + 3 * (k - 3 * n - 3);
      a = e[0] * ob[3] + e[1] * ob[4] + e[2] * ob[5];
    }
    rhs[k] = (T)(v[k] - a);
  }
  __syncthreads();
  const T *jinv = reinterpret_cast<const T *>(d.jinv + (size_t)n6 * n6 * fil);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int row = warp; row < n6; row += nw) {
    const T *jr = jinv + (size_t)row * n6;
    T s = 0;
    for (int k = lane; k < n6; k += 32) s += jr[k] * rhs[k];
    for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    if (lane == 0) out[(size_t)n6 * fil + row] = (double)s;
  }
}

// ---------------------------------------------------------------------------
// Broyden's low-rank update (broyden_solver.cpp:21-129); C and D are
// column-major nbroy x max_iter on the device.
// ---------------------------------------------------------------------------

constexpr int kRedThreads = 256;
constexpr int kNormBlocks = 128;
constexpr int kMaxDotChunks = 64;

__device__ double block_sum(double v, double *sh) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  if (lane == 0) sh[warp] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x < 32) {
    t = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
    for (int off = 16; off > 0; off >>= 1) t += __shfl_xor_sync(0xffffffffu, t, off);
  }
  return t;  // valid in thread 0
}

// part[i * nchunk + c] = a . D_i over rows of chunk c (grid nchunk x ncols)
__global__ void __launch_bounds__(kRedThreads) k_col_dots(const double *__restrict__ a,
                                                          const double *__restrict__ Dm, long nbroy,
                                                          long rows_per_chunk,
                                                          double *__restrict__ part) {
  __shared__ double sh[32];
  const double *col = Dm + (size_t)blockIdx.y * nbroy;
  const long r0 = blockIdx.x * rows_per_chunk;
  const long r1 = r0 + rows_per_chunk < nbroy ? r0 + rows_per_chunk : nbroy;
  double s = 0.0;
  for (long r = r0 + threadIdx.x; r < r1; r += blockDim.x) s += a[r] * col[r];
  s = block_sum(s, sh);
  if (threadIdx.x == 0) part[(size_t)blockIdx.y * gridDim.x + blockIdx.x] = s;
}

// coef[i] = sum over chunks of part[i * nchunk + c] (one warp per column)
__global__ void k_col_dots_final(const double *__restrict__ part, int nchunk,
                                 double *__restrict__ coef) {
  double s = 0.0;
  for (int c = threadIdx.x; c < nchunk; c += 32) s += part[(size_t)blockIdx.x * nchunk + c];
  for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
  if (threadIdx.x == 0) coef[blockIdx.x] = s;
}

// v = -conf v - sum_i coef[i] C_i
__global__ void k_scale_sub_cols(double *__restrict__ v, const double *__restrict__ Cm,
                                 const double *__restrict__ coef, int ncols, double conf, long nbroy) {
  for (long r = blockIdx.x * (long)blockDim.x + threadIdx.x; r < nbroy; r += (long)gridDim.x * blockDim.x) {
    double acc = v[r] * -conf;
    for (int i = 0; i < ncols; ++i) acc -= coef[i] * Cm[(size_t)i * nbroy + r];
    v[r] = acc;
  }
}

// D_it = nerr - err, with per-block partial sums of squares
__global__ void __launch_bounds__(kRedThreads) k_diff(const double *__restrict__ nerr,
                                                      const double *__restrict__ err,
                                                      double *__restrict__ dcol, long nbroy,
                                                      double *__restrict__ partial) {
  __shared__ double sh[32];
  double s = 0.0;
  for (long r = blockIdx.x * (long)blockDim.x + threadIdx.x; r < nbroy; r += (long)gridDim.x * blockDim.x) {
    const double v = nerr[r] - err[r];
    dcol[r] = v;
    s += v * v;
  }
  s = block_sum(s, sh);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

// C_it /= |D_it|, D_it /= |D_it|
__global__ void __launch_bounds__(kRedThreads) k_div2(double *__restrict__ ccol, double *__restrict__ dcol,
                                                      long nbroy, const double *__restrict__ partial) {
  __shared__ double sh[32];
  __shared__ double delta;
  double s = threadIdx.x < kNormBlocks ? partial[threadIdx.x] : 0.0;
  s = block_sum(s, sh);
  if (threadIdx.x == 0) delta = sqrt(s);
  __syncthreads();
  const double dl = delta;
  for (long r = blockIdx.x * (long)blockDim.x + threadIdx.x; r < nbroy; r += (long)gridDim.x * blockDim.x) {
    ccol[r] /= dl;
    dcol[r] /= dl;
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

struct tfs_stepper {
  tfs_solver *s = nullptr;
  tfs_step_config cfg{};
  StepDev d{};
  // body state (rigid_body::x, xm1, xm2, u, um1, q, qm1, Q_init)
  double bx[3], bxm1[3], bxm2[3], bu[3], bum1[3], bq[4], bqm1[4];
  double Qinit[9];
  double schur_inv[36];   // row-major
  double *schur_dev = nullptr;
  double *err = nullptr, *nerr = nullptr, *upd = nullptr, *tin = nullptr, *tout = nullptr;
  double *Cm = nullptr, *Dm = nullptr, *coef = nullptr, *dotpart = nullptr;
  double *p6 = nullptr, *ob = nullptr, *partial = nullptr, *swpart = nullptr;
  int *flag = nullptr;
  double *hbuf = nullptr;  // pinned: max(45, 6) nfil + 8
  int *hflag = nullptr;    // pinned
  int iter = 0;
  int jac_ready = 0;
  size_t jac_smem = 0, jac_ff_smem = 0;
  bool jinv_f32 = false;  // the stored J^-1 is FP32 (FP32C solvers)
  long nbroy = 0;
  // the straight start (for tfs_stepper_reset): unit directions, base
  // quaternions, body frame references; the solver's warm start as it was
  // when the stepper was created
  std::vector<double> dirs, q0, refs;
  double *warm = nullptr;  // 3 nblob + 6
};

namespace {

using tfs::fail;
using tfs::cuda_fail;

#define ST_CUDA(call, what)                                  \
  do {                                                       \
    cudaError_t e_ = (call);                                 \
    if (e_ != cudaSuccess) return tfs::cuda_fail(e_, what);  \
  } while (0)

#define ST_LAUNCH(what)                                      \
  do {                                                       \
    tfs::count_launch();                                     \
    cudaError_t e_ = cudaGetLastError();                     \
    if (e_ != cudaSuccess) return tfs::cuda_fail(e_, what);  \
  } while (0)

void rot_rm(const double *q, double *R) { rot_mat(load_q(q), R); }

// Q B Q^T for each 3x3 block of the column-major 6x6 body mobility, row-major out
// (swimmer.cpp:731-736)
void rotated_body_mobility(const double *bm_cm, const double *Q, double *out) {
  for (int bi = 0; bi < 2; ++bi)
    for (int bj = 0; bj < 2; ++bj) {
      M3 B;
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) B.a[3 * i + j] = bm_cm[(3 * bi + i) + 6 * (3 * bj + j)];
      const M3 Qm = m3_from(Q);
      M3 Qt;
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) Qt.a[3 * i + j] = Q[3 * j + i];
      const M3 r = m3_mul(m3_mul(Qm, B), Qt);
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) out[6 * (3 * bi + i) + 3 * bj + j] = r.a[3 * i + j];
    }
}

// Gauss-Jordan with partial pivoting, row-major n x n, in place; false if singular.
bool invert_rm(double *A, int n) {
  std::vector<int> perm(n);
  for (int k = 0; k < n; ++k) {
    int p = k;
    for (int i = k + 1; i < n; ++i)
      if (std::fabs(A[i * n + k]) > std::fabs(A[p * n + k])) p = i;
    perm[k] = p;
    if (A[p * n + k] == 0.0) return false;
    if (p != k)
      for (int j = 0; j < n; ++j) std::swap(A[k * n + j], A[p * n + j]);
    const double piv = A[k * n + k];
    for (int j = 0; j < n; ++j) A[k * n + j] = j == k ? 1.0 / piv : A[k * n + j] / piv;
    for (int i = 0; i < n; ++i) {
      if (i == k) continue;
      const double ci = A[i * n + k];
      for (int j = 0; j < n; ++j) A[i * n + j] = j == k ? -ci * A[k * n + k] : A[i * n + j] - ci * A[k * n + j];
    }
  }
  for (int k = n - 1; k >= 0; --k)
    if (perm[k] != k)
      for (int i = 0; i < n; ++i) std::swap(A[i * n + k], A[i * n + perm[k]]);
  return true;
}

BodyArgs body_args(const tfs_stepper *st, int nt) {
  BodyArgs b{};
  for (int k = 0; k < 3; ++k) {
    b.x[k] = st->bx[k];
    b.xm1[k] = st->bxm1[k];
    b.xm2[k] = st->bxm2[k];
    b.u[k] = st->bu[k];
    b.um1[k] = st->bum1[k];
  }
  rot_rm(st->bq, b.R);
  std::memcpy(b.Q, st->Qinit, sizeof b.Q);
  rotated_body_mobility(st->s->body_mob_ref, st->Qinit, b.BM);
  const M3 blc = m3_scale(-1.0, rcross(st->bu));
  const M3 bb12 = m3_div(m3_mul(blc, blc), 12.0);
  const M3 I = m3_eye();
  const M3 Dinv = m3_add(I, m3_sub(bb12, m3_scale(0.5, blc)));
  const M3 DinvT = m3_add(I, m3_add(bb12, m3_scale(0.5, blc)));
  std::memcpy(b.Dinv, Dinv.a, sizeof b.Dinv);
  std::memcpy(b.DinvT, DinvT.a, sizeof b.DinvT);
  std::memcpy(b.blc, blc.a, sizeof b.blc);
  b.dt_fac = nt < 1 ? -st->cfg.dt : -2.0 * st->cfg.dt / 3.0;
  return b;
}

int grid_for(long n, int threads) {
  long g = (n + threads - 1) / threads;
  if (g > 4096) g = 4096;
  return (int)(g < 1 ? 1 : g);
}

// out = jacobian_inv_mult(in), device to device
int jinv_mult_dev(tfs_stepper *st, int nt, const double *in, double *out) {
  const StepDev &d = st->d;
  cudaStream_t str = st->s->stream;
  const BodyArgs b = body_args(st, nt);
  k_jb_dot<<<d.nfil, 192, 0, str>>>(d, in, st->p6);
  ST_LAUNCH("jacobian_inv_mult (JB in)");
  k_body_solve<<<1, 256, 0, str>>>(d, in, st->p6, st->schur_dev, out, st->ob);
  ST_LAUNCH("jacobian_inv_mult (body)");
  if (st->jinv_f32) k_jinv_apply<float><<<d.nfil, 256, sizeof(double) * 6 * d.nseg, str>>>(d, b, in, st->ob, out);
  else k_jinv_apply<double><<<d.nfil, 256, sizeof(double) * 6 * d.nseg, str>>>(d, b, in, st->ob, out);
  ST_LAUNCH("jacobian_inv_mult (filaments)");
  return TFS_OK;
}

// v = -conf v - sum_{i < ncols} (a . D_i) C_i
int low_rank(tfs_stepper *st, const double *a, double *v, int ncols) {
  cudaStream_t str = st->s->stream;
  if (ncols > 0) {
    long nchunk = (st->nbroy + 4095) / 4096;
    if (nchunk > kMaxDotChunks) nchunk = kMaxDotChunks;
    const long rows = (st->nbroy + nchunk - 1) / nchunk;
    k_col_dots<<<dim3((unsigned)nchunk, (unsigned)ncols), kRedThreads, 0, str>>>(a, st->Dm, st->nbroy,
                                                                               rows, st->dotpart);
    ST_LAUNCH("Broyden column dots");
    k_col_dots_final<<<ncols, 32, 0, str>>>(st->dotpart, (int)nchunk, st->coef);
    ST_LAUNCH("Broyden column dots (sum)");
  }
  k_scale_sub_cols<<<grid_for(st->nbroy, 256), 256, 0, str>>>(v, st->Cm, st->coef, ncols,
                                                              st->cfg.jacobian_confidence, st->nbroy);
  ST_LAUNCH("Broyden low-rank update");
  return TFS_OK;
}

// The straight start (filament::initial_setup, filament.cpp:219-346): the
// body at rest at its configured pose, filaments along their directions from
// the bases X + R ref, all multipliers and histories zero. With rot (3 values
// per segment) each segment is first turned by exp(rot) and the positions
// follow from the robot arm; without it they are base + j DL dir, accumulated
// as the reference does.
int load_start(tfs_stepper *st, const double *rot) {
  const StepDev &d = st->d;
  const tfs_step_config *cfg = &st->cfg;
  const size_t ns = d.ns, nf = d.nfil, nl = 3 * (size_t)(d.nseg - 1) * nf;
  for (int k = 0; k < 3; ++k) st->bx[k] = st->bxm1[k] = st->bxm2[k] = cfg->body_x[k];
  for (int k = 0; k < 3; ++k) st->bu[k] = st->bum1[k] = 0.0;
  for (int k = 0; k < 4; ++k) st->bq[k] = st->bqm1[k] = cfg->body_q[k];
  rot_rm(st->bq, st->Qinit);
  std::vector<double> hx(3 * ns), hq(4 * ns), hu(3 * ns, 0.0), zero(std::max(nl, 6 * ns), 0.0);
  for (size_t i = 0; i < nf; ++i) {
    const double *ud = &st->dirs[3 * i];
    const Quat q0 = load_q(&st->q0[4 * i]);
    double pos[3];
    for (int k = 0; k < 3; ++k) {
      double r = 0.0;
      for (int c = 0; c < 3; ++c) r += st->Qinit[3 * k + c] * st->refs[3 * i + c];
      pos[k] = st->bx[k] + r;
    }
    double tprev[3] = {0.0, 0.0, 0.0};
    for (int j = 0; j < d.nseg; ++j) {
      const size_t sg = i * d.nseg + j;
      const Quat q = rot ? qmul(lie_exp(rot + 3 * sg), q0) : q0;
      store_q(&hq[4 * sg], q);
      if (rot) {
        double t[3];
        tangent(q, t);
        if (j > 0)
          for (int k = 0; k < 3; ++k) pos[k] = pos[k] + 0.5 * d.dl * (tprev[k] + t[k]);
        for (int k = 0; k < 3; ++k) tprev[k] = t[k];
        for (int k = 0; k < 3; ++k) hx[3 * sg + k] = pos[k];
      } else {
        for (int k = 0; k < 3; ++k) hx[3 * sg + k] = pos[k];
        for (int k = 0; k < 3; ++k) pos[k] += d.dl * ud[k];
      }
    }
  }
  cudaStream_t str = st->s->stream;
  struct C {
    double *dst;
    const double *src;
    size_t n;
  } copies[] = {{d.x, hx.data(), 3 * ns},    {d.xm1, hx.data(), 3 * ns}, {d.xm2, hx.data(), 3 * ns},
                {d.q, hq.data(), 4 * ns},    {d.qm1, hq.data(), 4 * ns}, {d.u, hu.data(), 3 * ns},
                {d.um1, hu.data(), 3 * ns},  {d.f, zero.data(), 6 * ns}, {d.lam, zero.data(), nl},
                {d.lamm1, zero.data(), nl},  {d.lamm2, zero.data(), nl}, {d.teth, zero.data(), 3 * nf},
                {d.tethm1, zero.data(), 3 * nf}, {d.tethm2, zero.data(), 3 * nf},
                {d.clamp, zero.data(), 3 * nf}, {d.clampm1, zero.data(), 3 * nf},
                {d.clampm2, zero.data(), 3 * nf}, {const_cast<double *>(d.fil_refs), st->refs.data(), 3 * nf}};
  for (auto &c : copies)
    ST_CUDA(cudaMemcpyAsync(c.dst, c.src, sizeof(double) * c.n, cudaMemcpyHostToDevice, str),
            "stepper state");
  ST_CUDA(cudaStreamSynchronize(str), "stepper state");
  st->iter = 0;
  st->jac_ready = 0;
  st->s->origin_dirty = true;
  return TFS_OK;
}

}  // namespace

extern "C" {

int tfs_step_config_default(tfs_step_config *cfg, int nfil, int nseg) {
  if (cfg == nullptr) return fail(TFS_EINVAL, "null config");
  std::memset(cfg, 0, sizeof *cfg);
  cfg->nfil = nfil;
  cfg->nseg = nseg;
  cfg->seg_sep = 2.2;
  cfg->dt = 36.3833 / 300.0;
  cfg->tol = 1e-4;
  cfg->max_broyden_iter = 400;
  cfg->kb = 1800.0;
  cfg->kt = 1800.0;
  cfg->end_force_magnitude = nseg > 0 ? 220.0 * 1800.0 / (2.6 * 2.6 * (double)nseg * (double)nseg) : 0.0;
  cfg->jacobian_confidence = 0.1;
  cfg->body_radius = 1.0;
  cfg->perturb_first_step = 1;
  cfg->body_q[0] = 1.0;
  return TFS_OK;
}

int tfs_stepper_destroy(tfs_stepper *st) {
  if (st == nullptr) return TFS_OK;
  StepDev &d = st->d;
  double *bufs[] = {d.q,     d.qm1,  d.u,       d.um1,    d.xm1,    d.xm2,     d.f,       d.lam,
                    d.lamm1, d.lamm2, d.teth,   d.tethm1, d.tethm2, d.clamp,   d.clampm1, d.clampm2,
                    d.jinv,  d.jb,   d.ecb,     d.part,   st->schur_dev, st->err, st->nerr, st->upd,
                    st->tin, st->tout, st->Cm,  st->Dm,   st->coef, st->dotpart, st->p6,    st->ob,    st->partial,
                    st->swpart};
  for (double *p : bufs)
    if (p) cudaFree(p);
  if (d.fil_refs) cudaFree(const_cast<double *>(d.fil_refs));
  if (st->flag) cudaFree(st->flag);
  if (st->warm) cudaFree(st->warm);
  if (st->hbuf) cudaFreeHost(st->hbuf);
  if (st->hflag) cudaFreeHost(st->hflag);
  delete st;
  return TFS_OK;
}

int tfs_stepper_create(tfs_solver *s, const tfs_step_config *cfg, const double *fil_refs,
                       const double *fil_dirs, tfs_stepper **out) {
  TFS_CHECK_SOLVER(s);
  if (cfg == nullptr || fil_refs == nullptr || fil_dirs == nullptr || out == nullptr)
    return fail(TFS_EINVAL, "null argument");
  *out = nullptr;
  if (s->cfg.nswim != 1) return fail(TFS_EINVAL, "the stepper advances one swimmer per solver");
  if (cfg->nfil != s->cfg.nfil || cfg->nseg != s->cfg.nseg)
    return fail(TFS_EINVAL, "step sizes (%d x %d) differ from the solver's (%d x %d)", cfg->nfil,
                cfg->nseg, s->cfg.nfil, s->cfg.nseg);
  if (cfg->nfil < 1) return fail(TFS_EINVAL, "at least one filament");
  if (cfg->nseg < 3) return fail(TFS_EINVAL, "at least three segments per filament");
  if (!s->have_refs) return fail(TFS_ESTATE, "set the blob references first");
  if (!(cfg->dt > 0) || !(cfg->tol > 0) || cfg->max_broyden_iter < 1 || !(cfg->seg_sep > 0) ||
      !(cfg->body_radius > 0))
    return fail(TFS_EINVAL, "dt, tol, seg_sep, body_radius must be > 0 and max_broyden_iter >= 1");
  const int n6 = 6 * cfg->nseg;
  const size_t smem = sizeof(double) * ((size_t)n6 * n6 + 7 * (size_t)n6 + 40) + sizeof(int) * n6;
  int dev = 0, optin = 0;
  ST_CUDA(cudaGetDevice(&dev), "device");
  ST_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev), "attribute");
  if (smem > (size_t)optin)
    return fail(TFS_EINVAL, "nseg %d: the approximate Jacobian (%zu bytes) does not fit in shared memory",
                cfg->nseg, smem);
  ST_CUDA(cudaFuncSetAttribute(k_jacobian<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
          "jacobian shared memory");
  const size_t ff_smem = sizeof(typename JacLoOps::E) * ((size_t)n6 * n6 + 7 * (size_t)n6) + sizeof(int) * n6;
  ST_CUDA(cudaFuncSetAttribute(k_jacobian_lo<JacLoOps>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ff_smem),
          "jacobian shared memory");
  ST_CUDA(cudaFuncSetAttribute(k_jacobian<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
          "jacobian shared memory");
  tfs_stepper *st = new (std::nothrow) tfs_stepper();
  if (st == nullptr) return fail(TFS_ENOMEM, "host allocation");
  st->s = s;
  st->cfg = *cfg;
  st->jac_smem = smem;
  st->jac_ff_smem = ff_smem;
  StepDev &d = st->d;
  d.nfil = cfg->nfil;
  d.nseg = cfg->nseg;
  d.ns = d.nfil * d.nseg;
  d.nbroy = 6 * (d.ns + 1);
  st->nbroy = d.nbroy;
  d.dl = cfg->seg_sep;
  d.dt = cfg->dt;
  d.kb = cfg->kb;
  d.kt = cfg->kt;
  d.efm = cfg->end_force_magnitude;
  d.mu = s->cfg.mu;
  d.a = s->cfg.a_seg;
  d.body_r = cfg->body_radius;
  d.pert = 0.01 * cfg->end_force_magnitude;
  d.perturb = cfg->perturb_first_step;
  d.x = s->x_segs;
  d.fs = s->f_segs;
  const size_t ns = d.ns, nf = d.nfil, nl = 3 * (size_t)(d.nseg - 1) * nf;
  const size_t mi = cfg->max_broyden_iter;
  struct A {
    double **p;
    size_t n;
  } allocs[] = {{&d.q, 4 * ns},        {&d.qm1, 4 * ns},       {&d.u, 3 * ns},
                {&d.um1, 3 * ns},      {&d.xm1, 3 * ns},       {&d.xm2, 3 * ns},
                {&d.f, 6 * ns},        {&d.lam, nl},           {&d.lamm1, nl},
                {&d.lamm2, nl},        {&d.teth, 3 * nf},      {&d.tethm1, 3 * nf},
                {&d.tethm2, 3 * nf},   {&d.clamp, 3 * nf},     {&d.clampm1, 3 * nf},
                {&d.clampm2, 3 * nf},  {&d.jinv, (size_t)n6 * n6 * nf},
                {&d.jb, 6 * (size_t)n6 * nf}, {&d.ecb, 18 * nf}, {&d.part, 45 * nf},
                {&st->schur_dev, 36},  {&st->err, (size_t)d.nbroy}, {&st->nerr, (size_t)d.nbroy},
                {&st->upd, (size_t)d.nbroy}, {&st->tin, (size_t)d.nbroy}, {&st->tout, (size_t)d.nbroy},
                {&st->Cm, (size_t)d.nbroy * mi}, {&st->Dm, (size_t)d.nbroy * mi},
                {&st->coef, mi},       {&st->dotpart, mi * kMaxDotChunks},
                {&st->p6, 6 * nf},     {&st->ob, 8},
                {&st->partial, kNormBlocks}, {&st->swpart, 6 * nf}};
  for (auto &a : allocs) {
    if (cudaMalloc(reinterpret_cast<void **>(a.p), sizeof(double) * a.n) != cudaSuccess) {
      cudaGetLastError();
      tfs_stepper_destroy(st);
      return fail(TFS_ENOMEM, "stepper device allocation (%zu doubles)", a.n);
    }
  }
  double *refs_dev = nullptr;
  if (cudaMalloc(&refs_dev, sizeof(double) * 3 * nf) != cudaSuccess ||
      cudaMalloc(&st->flag, sizeof(int)) != cudaSuccess ||
      cudaMallocHost(&st->hbuf, sizeof(double) * (45 * nf + 64)) != cudaSuccess ||
      cudaMallocHost(&st->hflag, sizeof(int)) != cudaSuccess) {
    cudaGetLastError();
    if (refs_dev) cudaFree(refs_dev);
    tfs_stepper_destroy(st);
    return fail(TFS_ENOMEM, "stepper allocation");
  }
  d.fil_refs = refs_dev;
  st->dirs.resize(3 * nf);
  st->q0.resize(4 * nf);
  st->refs.assign(fil_refs, fil_refs + 3 * nf);
  for (size_t i = 0; i < nf; ++i) {
    const double *dir = fil_dirs + 3 * i;
    const double dn = std::sqrt(dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]);
    if (!(dn > 0.0)) {
      tfs_stepper_destroy(st);
      return fail(TFS_EINVAL, "filament %zu: zero direction", i);
    }
    for (int k = 0; k < 3; ++k) st->dirs[3 * i + k] = dir[k] / dn;
    store_q(&st->q0[4 * i], along_direction(dir));
  }
  {
    double nq = 0.0;
    for (int k = 0; k < 4; ++k) nq += cfg->body_q[k] * cfg->body_q[k];
    if (!(nq > 0.0)) {
      tfs_stepper_destroy(st);
      return fail(TFS_EINVAL, "zero body quaternion");
    }
  }
  int rc = load_start(st, nullptr);
  if (rc != TFS_OK) {
    tfs_stepper_destroy(st);
    return rc;
  }
  tfs::solver_reset_history(s);
  // the warm start of the first solve, restored by tfs_stepper_reset
  const size_t nw = 3 * (size_t)s->nb + 6;
  if (cudaMalloc(&st->warm, sizeof(double) * nw) != cudaSuccess) {
    cudaGetLastError();
    tfs_stepper_destroy(st);
    return fail(TFS_ENOMEM, "stepper allocation");
  }
  cudaError_t e = cudaMemcpyAsync(st->warm, s->f_blobs, sizeof(double) * 3 * s->nb,
                                  cudaMemcpyDeviceToDevice, s->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(st->warm + 3 * s->nb, s->v_bodies, sizeof(double) * 6,
                        cudaMemcpyDeviceToDevice, s->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  if (e != cudaSuccess) {
    tfs_stepper_destroy(st);
    return cuda_fail(e, "stepper warm start");
  }
  s->origin_dirty = true;
  *out = st;
  return TFS_OK;
}

#define TFS_CHECK_STEPPER(st)                                                   \
  do {                                                                          \
    if ((st) == nullptr) return tfs::fail(TFS_EINVAL, "null stepper handle");    \
  } while (0)

int tfs_stepper_initial_guess(tfs_stepper *st, int nt) {
  TFS_CHECK_STEPPER(st);
  const int hrc = tfs::solver_new_step(st->s);
  if (hrc != TFS_OK) return hrc;
  // rigid_body::initial_guess (rigid_body.cpp:395-480)
  double gx[3], gu[3];
  for (int k = 0; k < 3; ++k) {
    if (nt <= 1) {
      gx[k] = 2.0 * st->bx[k] - st->bxm1[k];
      gu[k] = st->bu[k];
    } else {
      gx[k] = 3.0 * (st->bx[k] - st->bxm1[k]) + st->bxm2[k];
      gu[k] = 2.0 * st->bu[k] - st->bum1[k];
    }
  }
  for (int k = 0; k < 3; ++k) {
    st->bxm2[k] = st->bxm1[k];
    st->bxm1[k] = st->bx[k];
    st->bx[k] = gx[k];
    st->bum1[k] = st->bu[k];
    st->bu[k] = gu[k];
  }
  std::memcpy(st->bqm1, st->bq, sizeof st->bq);
  store_q(st->bq, qmul(lie_exp(st->bu), load_q(st->bqm1)));
  rot_rm(st->bq, st->Qinit);
  st->jac_ready = 0;
  const BodyArgs b = body_args(st, nt);
  k_guess_segments<<<(st->d.ns + 63) / 64, 64, 0, st->s->stream>>>(st->d, b, nt);
  ST_LAUNCH("initial guess");
  k_robot_arm<<<(st->d.nfil + kFilWarps - 1) / kFilWarps, 32 * kFilWarps, 0, st->s->stream>>>(
      st->d, b);
  ST_LAUNCH("robot arm");
  st->s->origin_dirty = true;
  return TFS_OK;
}

int tfs_stepper_forces(tfs_stepper *st, int nt, double *swimmer_f) {
  TFS_CHECK_STEPPER(st);
  const StepDev &d = st->d;
  cudaStream_t str = st->s->stream;
  k_forces<<<(d.ns + 63) / 64, 64, 0, str>>>(d, nt);
  ST_LAUNCH("internal forces");
  k_swimmer_force<<<(d.nfil + kFilWarps - 1) / kFilWarps, 32 * kFilWarps, 0, str>>>(
      d, st->bx[0], st->bx[1], st->bx[2], st->swpart);
  ST_LAUNCH("swimmer force");
  // swimmer::f on the device, where compute_velocities reads it
  k_swimmer_sum<<<1, 6 * 32, 0, str>>>(st->swpart, d.nfil, st->s->swimmer_f);
  ST_LAUNCH("swimmer force sum");
  if (swimmer_f) {
    ST_CUDA(cudaMemcpyAsync(st->hbuf, st->s->swimmer_f, sizeof(double) * 6, cudaMemcpyDeviceToHost,
                            str),
            "swimmer force");
    ST_CUDA(cudaStreamSynchronize(str), "internal forces");
    std::memcpy(swimmer_f, st->hbuf, sizeof(double) * 6);
  }
  return TFS_OK;
}

namespace {

// The solve of one Broyden iteration at the current pose, on the swimmer
// force the last forces call left on the device; no host wait at the end.
int stepper_velocities(tfs_stepper *st, int *gmres_iters) {
  int rc = tfs_set_body_pose(st->s, st->bx, st->bq);
  if (rc != TFS_OK) return rc;
  st->s->origin_dirty = true;
  return tfs::compute_velocities_dev(st->s, gmres_iters);
}

}  // namespace

int tfs_stepper_compute_velocities(tfs_stepper *st, int nt, int *gmres_iters) {
  TFS_CHECK_STEPPER(st);
  (void)nt;
  const int rc = stepper_velocities(st, gmres_iters);
  if (rc != TFS_OK) return rc;
  ST_CUDA(cudaStreamSynchronize(st->s->stream), "compute_velocities");
  return TFS_OK;
}

int tfs_stepper_compute_errors(tfs_stepper *st, int nt, int which, double *err_host, int *too_large) {
  TFS_CHECK_STEPPER(st);
  const StepDev &d = st->d;
  cudaStream_t str = st->s->stream;
  double *e = which ? st->nerr : st->err;
  ST_CUDA(cudaMemsetAsync(st->flag, 0, sizeof(int), str), "error flag");
  const BodyArgs b = body_args(st, nt);
  k_errors<<<(d.ns + 63) / 64, 64, 0, str>>>(d, b, nt, st->cfg.tol, st->s->v_segs, st->s->v_bodies,
                                                 e, st->flag);
  ST_LAUNCH("residuals");
  ST_CUDA(cudaMemcpyAsync(st->hflag, st->flag, sizeof(int), cudaMemcpyDeviceToHost, str), "error flag");
  if (err_host)
    ST_CUDA(cudaMemcpyAsync(err_host, e, sizeof(double) * d.nbroy, cudaMemcpyDeviceToHost, str),
            "residuals");
  ST_CUDA(cudaStreamSynchronize(str), "residuals");
  if (too_large) *too_large = (*st->hflag & 1) != 0;
  if (*st->hflag & 2) return fail(TFS_ENAN, "non-finite residual (Broyden's method diverged)");
  return TFS_OK;
}

int tfs_stepper_prepare_jacobian_inv(tfs_stepper *st, int nt, double *schur_inv) {
  TFS_CHECK_STEPPER(st);
  const StepDev &d = st->d;
  cudaStream_t str = st->s->stream;
  const BodyArgs b = body_args(st, nt);
  // FP32C: the inverse in FP32 (it only seeds Broyden's method, and FP64 is
  // this GPU's slowest pipe)
  st->jinv_f32 = st->s->cfg.precision == TFS_FP32C;
  if (st->jinv_f32) {
    k_jacobian<true><<<d.nfil, kJacAsmThreads, 0, str>>>(d, b, nt);
    ST_LAUNCH("approximate Jacobian");
    k_jacobian_lo<JacLoOps><<<d.nfil, kJacLoThreads, st->jac_ff_smem, str>>>(d, b);
  } else {
    k_jacobian<false><<<d.nfil, 256, st->jac_smem, str>>>(d, b, nt);
  }
  ST_LAUNCH("approximate Jacobian");
  ST_CUDA(cudaMemcpyAsync(st->hbuf, d.part, sizeof(double) * 45 * d.nfil, cudaMemcpyDeviceToHost, str),
          "Schur parts");
  ST_CUDA(cudaStreamSynchronize(str), "approximate Jacobian");
  // the 6x6 Schur complement of the body equations (swimmer.cpp:684-913)
  const double dtf = b.dt_fac;
  const M3 blc = m3_from(b.blc);
  const M3 cbo = m3_div(m3_scale(-1.0, blc), dtf);
  double S[36] = {0};
  for (int k = 0; k < 6; ++k) S[7 * k] = 1.0;
  auto add_rr = [&](const M3 &m) {
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) S[6 * (3 + i) + 3 + j] += m.a[3 * i + j];
  };
  add_rr(m3_scale(dtf, m3_sub(m3_div(m3_mul(blc, cbo), 12.0), m3_scale(0.5, cbo))));
  M3 old = m3_zero();
  for (int i = 0; i < d.nfil; ++i) old = m3_add(old, m3_from(st->hbuf + 45 * i + 36));
  M3 BMrr;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) BMrr.a[3 * i + j] = b.BM[6 * (3 + i) + 3 + j];
  old = m3_mul(BMrr, old);
  add_rr(m3_scale(dtf, m3_add(m3_sub(old, m3_mul(m3_scale(0.5, blc), old)),
                              m3_div(m3_mul(m3_mul(blc, blc), old), 12.0))));
  for (int i = 0; i < d.nfil; ++i)
    for (int k = 0; k < 36; ++k) S[k] -= st->hbuf[45 * i + k];
  if (!invert_rm(S, 6)) return fail(TFS_ENAN, "singular Schur complement");
  std::memcpy(st->schur_inv, S, sizeof S);
  ST_CUDA(cudaMemcpyAsync(st->schur_dev, st->schur_inv, sizeof S, cudaMemcpyHostToDevice, str), "Schur");
  ST_CUDA(cudaStreamSynchronize(str), "Schur");
  st->jac_ready = 1;
  if (schur_inv)
    for (int i = 0; i < 6; ++i)
      for (int j = 0; j < 6; ++j) schur_inv[i + 6 * j] = S[6 * i + j];
  return TFS_OK;
}

int tfs_stepper_inverse_jacobian(tfs_stepper *st, int fil, double *out) {
  TFS_CHECK_STEPPER(st);
  if (out == nullptr || fil < 0 || fil >= st->d.nfil) return fail(TFS_EINVAL, "bad filament or output");
  if (!st->jac_ready) return fail(TFS_ESTATE, "prepare_jacobian_inv has not run this step");
  const int n6 = 6 * st->d.nseg;
  std::vector<double> h((size_t)n6 * n6);
  if (st->jinv_f32) {
    std::vector<float> hf(h.size());
    ST_CUDA(cudaMemcpyAsync(hf.data(), st->d.jinv + (size_t)n6 * n6 * fil, sizeof(float) * hf.size(),
                            cudaMemcpyDeviceToHost, st->s->stream),
            "inverse Jacobian");
    ST_CUDA(cudaStreamSynchronize(st->s->stream), "inverse Jacobian");
    for (size_t i = 0; i < h.size(); ++i) h[i] = hf[i];
  } else {
    ST_CUDA(cudaMemcpyAsync(h.data(), st->d.jinv + (size_t)n6 * n6 * fil, sizeof(double) * h.size(),
                            cudaMemcpyDeviceToHost, st->s->stream),
            "inverse Jacobian");
    ST_CUDA(cudaStreamSynchronize(st->s->stream), "inverse Jacobian");
  }
  for (int i = 0; i < n6; ++i)
    for (int j = 0; j < n6; ++j) out[i + (size_t)n6 * j] = h[(size_t)n6 * i + j];
  return TFS_OK;
}

int tfs_stepper_jacobian_inv_mult(tfs_stepper *st, int nt, const double *in, double *out) {
  TFS_CHECK_STEPPER(st);
  if (in == nullptr || out == nullptr) return fail(TFS_EINVAL, "null vector");
  if (!st->jac_ready) return fail(TFS_ESTATE, "prepare_jacobian_inv has not run this step");
  cudaStream_t str = st->s->stream;
  const size_t bytes = sizeof(double) * st->nbroy;
  ST_CUDA(cudaMemcpyAsync(st->tin, in, bytes, cudaMemcpyHostToDevice, str), "jacobian_inv_mult input");
  int rc = jinv_mult_dev(st, nt, st->tin, st->tout);
  if (rc != TFS_OK) return rc;
  ST_CUDA(cudaMemcpyAsync(out, st->tout, bytes, cudaMemcpyDeviceToHost, str), "jacobian_inv_mult output");
  ST_CUDA(cudaStreamSynchronize(str), "jacobian_inv_mult");
  return TFS_OK;
}

int tfs_stepper_broyden_reset(tfs_stepper *st) {
  TFS_CHECK_STEPPER(st);
  st->iter = 0;
  return TFS_OK;
}

int tfs_stepper_find_update(tfs_stepper *st, int nt, double *update) {
  TFS_CHECK_STEPPER(st);
  if (!st->jac_ready) return fail(TFS_ESTATE, "prepare_jacobian_inv has not run this step");
  int rc = jinv_mult_dev(st, nt, st->err, st->upd);
  if (rc != TFS_OK) return rc;
  if ((rc = low_rank(st, st->err, st->upd, st->iter)) != TFS_OK) return rc;
  if (update) {
    ST_CUDA(cudaMemcpyAsync(update, st->upd, sizeof(double) * st->nbroy, cudaMemcpyDeviceToHost,
                            st->s->stream),
            "update");
    ST_CUDA(cudaStreamSynchronize(st->s->stream), "update");
  }
  return TFS_OK;
}

int tfs_stepper_apply_update(tfs_stepper *st, int nt) {
  TFS_CHECK_STEPPER(st);
  cudaStream_t str = st->s->stream;
  // rigid_body::update (rigid_body.cpp:502-529) on the host, then the filaments
  ST_CUDA(cudaMemcpyAsync(st->hbuf, st->upd + 6 * (size_t)st->d.ns, sizeof(double) * 6,
                          cudaMemcpyDeviceToHost, str),
          "body update");
  ST_CUDA(cudaStreamSynchronize(str), "body update");
  for (int k = 0; k < 3; ++k) {
    st->bx[k] += st->hbuf[k];
    st->bu[k] += st->hbuf[3 + k];
  }
  store_q(st->bq, qmul(lie_exp(st->bu), load_q(st->bqm1)));
  const BodyArgs b = body_args(st, nt);
  k_update_segments<<<(st->d.ns + 63) / 64, 64, 0, str>>>(st->d, b, st->upd);
  ST_LAUNCH("apply update");
  k_robot_arm<<<(st->d.nfil + kFilWarps - 1) / kFilWarps, 32 * kFilWarps, 0, str>>>(st->d, b);
  ST_LAUNCH("robot arm");
  st->s->origin_dirty = true;
  return tfs_stepper_forces(st, nt, nullptr);
}

int tfs_stepper_end_of_iter(tfs_stepper *st, int nt, int too_large) {
  TFS_CHECK_STEPPER(st);
  const int maxit = st->cfg.max_broyden_iter;
  if (too_large && st->iter < maxit - 1) {
    cudaStream_t str = st->s->stream;
    double *ccol = st->Cm + (size_t)st->iter * st->nbroy;
    double *dcol = st->Dm + (size_t)st->iter * st->nbroy;
    int rc = jinv_mult_dev(st, nt, st->nerr, ccol);
    if (rc != TFS_OK) return rc;
    if ((rc = low_rank(st, st->nerr, ccol, st->iter)) != TFS_OK) return rc;
    k_diff<<<kNormBlocks, kRedThreads, 0, str>>>(st->nerr, st->err, dcol, st->nbroy, st->partial);
    ST_LAUNCH("Broyden difference");
    k_div2<<<grid_for(st->nbroy, kRedThreads), kRedThreads, 0, str>>>(ccol, dcol, st->nbroy, st->partial);
    ST_LAUNCH("Broyden normalisation");
    std::swap(st->err, st->nerr);
  }
  st->iter++;
  return TFS_OK;
}

int tfs_stepper_step(tfs_stepper *st, int nt, int *broyden_iters, int *gmres_iters) {
  TFS_CHECK_STEPPER(st);
  int rc, it = 0, total = 0, big = 0;
  if ((rc = tfs_stepper_initial_guess(st, nt)) != TFS_OK) return rc;
  if ((rc = tfs_stepper_forces(st, nt, nullptr)) != TFS_OK) return rc;
  if ((rc = stepper_velocities(st, &it)) != TFS_OK) return rc;
  total += it;
  if ((rc = tfs_stepper_compute_errors(st, nt, 0, nullptr, &big)) != TFS_OK) return rc;
  if (big && (rc = tfs_stepper_prepare_jacobian_inv(st, nt, nullptr)) != TFS_OK) return rc;
  st->iter = 0;
  while (big && st->iter < st->cfg.max_broyden_iter) {
    if ((rc = tfs_stepper_find_update(st, nt, nullptr)) != TFS_OK) return rc;
    if ((rc = tfs_stepper_apply_update(st, nt)) != TFS_OK) return rc;
    if ((rc = stepper_velocities(st, &it)) != TFS_OK) return rc;
    total += it;
    if ((rc = tfs_stepper_compute_errors(st, nt, 1, nullptr, &big)) != TFS_OK) return rc;
    if ((rc = tfs_stepper_end_of_iter(st, nt, big)) != TFS_OK) return rc;
  }
  if (broyden_iters) *broyden_iters = st->iter;
  if (gmres_iters) *gmres_iters = total;
  if (big) return fail(TFS_ENOTCONV, "step %d: Broyden's method reached %d iterations", nt, st->iter);
  return TFS_OK;
}

int tfs_stepper_state(tfs_stepper *st, double *x, double *q, double *u, double *lambda, double *tether,
                      double *clamp, double *body_x, double *body_q, double *body_u) {
  TFS_CHECK_STEPPER(st);
  const StepDev &d = st->d;
  cudaStream_t str = st->s->stream;
  const size_t ns = d.ns, nf = d.nfil, nl = 3 * (size_t)(d.nseg - 1) * nf;
  struct C {
    double *dst;
    const double *src;
    size_t n;
  } copies[] = {{x, d.x, 3 * ns},        {q, d.q, 4 * ns},         {u, d.u, 3 * ns},
                {lambda, d.lam, nl},    {tether, d.teth, 3 * nf}, {clamp, d.clamp, 3 * nf}};
  for (auto &c : copies)
    if (c.dst) ST_CUDA(cudaMemcpyAsync(c.dst, c.src, sizeof(double) * c.n, cudaMemcpyDeviceToHost, str), "state");
  ST_CUDA(cudaStreamSynchronize(str), "state");
  if (body_x) std::memcpy(body_x, st->bx, sizeof st->bx);
  if (body_q) std::memcpy(body_q, st->bq, sizeof st->bq);
  if (body_u) std::memcpy(body_u, st->bu, sizeof st->bu);
  return TFS_OK;
}

int tfs_stepper_reset(tfs_stepper *st, const double *seg_rotation) {
  if (st != nullptr) tfs::solver_reset_history(st->s);
  TFS_CHECK_STEPPER(st);
  int rc = load_start(st, seg_rotation);
  if (rc != TFS_OK) return rc;
  tfs_solver *s = st->s;
  ST_CUDA(cudaMemcpyAsync(s->f_blobs, st->warm, sizeof(double) * 3 * s->nb, cudaMemcpyDeviceToDevice,
                          s->stream),
          "warm start");
  ST_CUDA(cudaMemcpyAsync(s->v_bodies, st->warm + 3 * s->nb, sizeof(double) * 6,
                          cudaMemcpyDeviceToDevice, s->stream),
          "warm start");
  ST_CUDA(cudaStreamSynchronize(s->stream), "warm start");
  return TFS_OK;
}

}  // extern "C"

namespace tfs {
// The reference's backup record of one swimmer (filament::write_backup,
// filament.cpp:1952-2037, then rigid_body::write_backup, rigid_body.cpp:
// 556-579): per filament, per segment q, x, xm1, xm2, u, um1; tether, clamp
// multipliers with their two previous values; per link the multiplier and
// its two previous values; then the body's q, x, xm1, xm2, u, um1.
size_t backup_values(const tfs_stepper *st) {
  return (size_t)st->d.nfil * (9 + 28 * (size_t)st->d.nseg) + 19;
}

int stepper_backup(tfs_stepper *st, std::vector<double> &out) {
  const StepDev &d = st->d;
  const size_t ns = d.ns, nf = d.nfil, nl = 3 * (size_t)(d.nseg - 1) * nf;
  std::vector<double> q(4 * ns), x(3 * ns), xm1(3 * ns), xm2(3 * ns), u(3 * ns), um1(3 * ns),
      t0(3 * nf), t1(3 * nf), t2(3 * nf), c0(3 * nf), c1(3 * nf), c2(3 * nf), l0(nl), l1(nl), l2(nl);
  struct C {
    double *dst;
    const double *src;
    size_t n;
  } copies[] = {{q.data(), d.q, 4 * ns},         {x.data(), d.x, 3 * ns},
                {xm1.data(), d.xm1, 3 * ns},     {xm2.data(), d.xm2, 3 * ns},
                {u.data(), d.u, 3 * ns},         {um1.data(), d.um1, 3 * ns},
                {t0.data(), d.teth, 3 * nf},     {t1.data(), d.tethm1, 3 * nf},
                {t2.data(), d.tethm2, 3 * nf},   {c0.data(), d.clamp, 3 * nf},
                {c1.data(), d.clampm1, 3 * nf},  {c2.data(), d.clampm2, 3 * nf},
                {l0.data(), d.lam, nl},          {l1.data(), d.lamm1, nl},
                {l2.data(), d.lamm2, nl}};
  cudaStream_t str = st->s->stream;
  for (auto &c : copies)
    ST_CUDA(cudaMemcpyAsync(c.dst, c.src, sizeof(double) * c.n, cudaMemcpyDeviceToHost, str), "backup");
  ST_CUDA(cudaStreamSynchronize(str), "backup");
  out.clear();
  out.reserve(backup_values(st));
  auto put3 = [&](const std::vector<double> &v, size_t i) {
    out.push_back(v[3 * i]);
    out.push_back(v[3 * i + 1]);
    out.push_back(v[3 * i + 2]);
  };
  for (size_t f = 0; f < nf; ++f) {
    for (int j = 0; j < d.nseg; ++j) {
      const size_t sg = f * d.nseg + j;
      for (int k = 0; k < 4; ++k) out.push_back(q[4 * sg + k]);
      put3(x, sg);
      put3(xm1, sg);
      put3(xm2, sg);
      put3(u, sg);
      put3(um1, sg);
    }
    put3(t0, f);
    put3(t1, f);
    put3(t2, f);
    put3(c0, f);
    put3(c1, f);
    put3(c2, f);
    for (int j = 0; j < d.nseg - 1; ++j) {
      const size_t l = f * (d.nseg - 1) + j;
      put3(l0, l);
      put3(l1, l);
      put3(l2, l);
    }
  }
  for (int k = 0; k < 4; ++k) out.push_back(st->bq[k]);
  for (int k = 0; k < 3; ++k) out.push_back(st->bx[k]);
  for (int k = 0; k < 3; ++k) out.push_back(st->bxm1[k]);
  for (int k = 0; k < 3; ++k) out.push_back(st->bxm2[k]);
  for (int k = 0; k < 3; ++k) out.push_back(st->bu[k]);
  for (int k = 0; k < 3; ++k) out.push_back(st->bum1[k]);
  return TFS_OK;
}

// Restore a backup record (as filament::initial_setup and
// rigid_body::initial_setup read one, filament.cpp:140-215,
// rigid_body.cpp:16-60: q^{n-1} = q); Broyden's memory is cleared and the
// solver's warm start is the one it had when the stepper was created.
int stepper_load(tfs_stepper *st, const double *v) {
  solver_reset_history(st->s);
  const StepDev &d = st->d;
  const size_t ns = d.ns, nf = d.nfil, nl = 3 * (size_t)(d.nseg - 1) * nf;
  std::vector<double> q(4 * ns), x(3 * ns), xm1(3 * ns), xm2(3 * ns), u(3 * ns), um1(3 * ns),
      t0(3 * nf), t1(3 * nf), t2(3 * nf), c0(3 * nf), c1(3 * nf), c2(3 * nf), l0(nl), l1(nl), l2(nl);
  size_t p = 0;
  auto get3 = [&](std::vector<double> &w, size_t i) {
    w[3 * i] = v[p++];
    w[3 * i + 1] = v[p++];
    w[3 * i + 2] = v[p++];
  };
  for (size_t f = 0; f < nf; ++f) {
    for (int j = 0; j < d.nseg; ++j) {
      const size_t sg = f * d.nseg + j;
      for (int k = 0; k < 4; ++k) q[4 * sg + k] = v[p++];
      get3(x, sg);
      get3(xm1, sg);
      get3(xm2, sg);
      get3(u, sg);
      get3(um1, sg);
    }
    get3(t0, f);
    get3(t1, f);
    get3(t2, f);
    get3(c0, f);
    get3(c1, f);
    get3(c2, f);
    for (int j = 0; j < d.nseg - 1; ++j) {
      const size_t l = f * (d.nseg - 1) + j;
      get3(l0, l);
      get3(l1, l);
      get3(l2, l);
    }
  }
  for (int k = 0; k < 4; ++k) st->bq[k] = st->bqm1[k] = v[p++];
  for (int k = 0; k < 3; ++k) st->bx[k] = v[p++];
  for (int k = 0; k < 3; ++k) st->bxm1[k] = v[p++];
  for (int k = 0; k < 3; ++k) st->bxm2[k] = v[p++];
  for (int k = 0; k < 3; ++k) st->bu[k] = v[p++];
  for (int k = 0; k < 3; ++k) st->bum1[k] = v[p++];
  rot_rm(st->bq, st->Qinit);
  struct C {
    double *dst;
    const double *src;
    size_t n;
  } copies[] = {{d.q, q.data(), 4 * ns},        {d.qm1, q.data(), 4 * ns},
                {d.x, x.data(), 3 * ns},        {d.xm1, xm1.data(), 3 * ns},
                {d.xm2, xm2.data(), 3 * ns},    {d.u, u.data(), 3 * ns},
                {d.um1, um1.data(), 3 * ns},    {d.teth, t0.data(), 3 * nf},
                {d.tethm1, t1.data(), 3 * nf},  {d.tethm2, t2.data(), 3 * nf},
                {d.clamp, c0.data(), 3 * nf},   {d.clampm1, c1.data(), 3 * nf},
                {d.clampm2, c2.data(), 3 * nf}, {d.lam, l0.data(), nl},
                {d.lamm1, l1.data(), nl},       {d.lamm2, l2.data(), nl}};
  tfs_solver *s = st->s;
  for (auto &c : copies)
    ST_CUDA(cudaMemcpyAsync(c.dst, c.src, sizeof(double) * c.n, cudaMemcpyHostToDevice, s->stream),
            "restore");
  ST_CUDA(cudaMemcpyAsync(s->f_blobs, st->warm, sizeof(double) * 3 * s->nb, cudaMemcpyDeviceToDevice,
                          s->stream),
          "warm start");
  ST_CUDA(cudaMemcpyAsync(s->v_bodies, st->warm + 3 * s->nb, sizeof(double) * 6,
                          cudaMemcpyDeviceToDevice, s->stream),
          "warm start");
  ST_CUDA(cudaStreamSynchronize(s->stream), "restore");
  st->iter = 0;
  st->jac_ready = 0;
  s->origin_dirty = true;
  return TFS_OK;
}

// Internal forces (the reference's f_segs_host, before barrier forces) to the host.
int stepper_internal_forces(tfs_stepper *st, double *f) {
  ST_CUDA(cudaMemcpyAsync(f, st->d.f, sizeof(double) * 6 * st->d.ns, cudaMemcpyDeviceToHost,
                          st->s->stream),
          "internal forces");
  ST_CUDA(cudaStreamSynchronize(st->s->stream), "internal forces");
  return TFS_OK;
}

int stepper_dims(const tfs_stepper *st, int *nfil, int *nseg) {
  *nfil = st->d.nfil;
  *nseg = st->d.nseg;
  return TFS_OK;
}

tfs_solver *stepper_solver(tfs_stepper *st) { return st ? st->s : nullptr; }
long stepper_segments(const tfs_stepper *st) { return st ? (long)st->d.ns : 0; }
}  // namespace tfs

namespace tfs {
// Device bytes of a stepper (tfs_stepper_create's allocations).
size_t stepper_bytes_estimate(int nfil, int nseg, int max_broyden_iter) {
  const size_t nf = nfil, ns = (size_t)nfil * nseg, n6 = 6 * (size_t)nseg;
  const size_t nbroy = 6 * (ns + 1);
  const size_t doubles = 31 * ns + 12 * nf * nseg + nf * (n6 * n6 + 6 * n6 + 18 + 45 + 6 + 6 + 3) +
                         nbroy * (5 + 2 * (size_t)max_broyden_iter) +
                         (size_t)max_broyden_iter * (1 + kMaxDotChunks) + 256;
  return 8 * doubles;
}
}  // namespace tfs
