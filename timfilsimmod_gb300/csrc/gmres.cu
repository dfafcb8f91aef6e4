// gmres.cu -- device-resident solve of the free-body saddle-point system of
// one swimmer (the reference's solve_linear_system, mobility_solver.cpp:
// 2092-2570, with apply_preconditioner_new :1437-1509 and
// system_matrix_mult_new :2027-2084, free-body branches).
//
// Unknowns x = [lambda (3 Nb blob forces); U, Omega], n = 3 Nb + 6:
//   A x     = [ M_bb lambda - (U + Omega x d_m) ; -sum_m (lambda_m ; d_m x lambda_m) ]
//   P^-1 x  = [ 6 pi mu a (lambda_m + U' + Omega' x d_m) ; (U', Omega') ]
//             with (U', Omega') = KTKinv b - N V,  b = -sum_m (lambda_m ; d_m x lambda_m),
//             N and KTKinv the body mobility and (K^T K)^-1 rotated to the body's
//             current orientation,
// where d_m = R ref_m. Right-preconditioned GMRES without restarts, warm
// started from the previous (lambda, U, Omega), modified Gram-Schmidt Arnoldi
// and the reference's Givens sign convention, stopping when
// |beta_k| / ||rhs|| <= tol or after min(n, max_iter) steps.
//
// Every vector and scalar of the iteration lives on the device. The small
// per-instance work (preconditioner, K/K^T, Gram-Schmidt, Givens, back
// solve) runs in single-CTA kernels; the blob-blob product M_bb runs on the
// tile kernel (rpy_kernels.cu) between them. A `done` flag in device memory
// makes every later kernel of the sequence return at once, so the host can
// launch the iteration in chunks (or replay it as a CUDA graph) and only
// poll the flag between chunks.
#include <cuda_runtime.h>

#include "gmres.h"
#include "tfs_kernels.h"

namespace tfs {

constexpr double kPiD = 3.14159265358979323846264338327950288;
constexpr int kSolveThreads = 1024;

// Deterministic block sum of one double per thread (all threads get it).
__device__ double block_sum(double v, double *red) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  if (wid == 0) {
    double t = lane < nw ? red[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
    if (lane == 0) red[32] = t;
  }
  __syncthreads();
  return red[32];
}

// Six simultaneous block sums in one pass (red holds >= 33 * 6 doubles):
// per-warp shuffle sums, then thread k adds the warps' partials of value k in
// warp order (deterministic).
__device__ void block_sum6(double (&v)[6], double *red) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int k = 0; k < 6; ++k)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
  __syncthreads();
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < 6; ++k) red[6 * wid + k] = v[k];
  __syncthreads();
  if (threadIdx.x < 6) {
    double t = 0.0;
    for (int w = 0; w < nw; ++w) t += red[6 * w + threadIdx.x];
    red[6 * 32 + threadIdx.x] = t;
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < 6; ++k) v[k] = red[6 * 32 + k];
}

__device__ void matvec6(double *out, const double *M, const double *v) {
  for (int i = 0; i < 6; ++i) {
    double s = 0.0;
    for (int k = 0; k < 6; ++k) s += M[i + 6 * k] * v[k];
    out[i] = s;
  }
}

// Pack blob forces f[3 nb] (with blob positions x) into the source-record
// formats the tile kernel reads: FP64 {x,y,z,fx,fy,fz}; FP32 (centred)
// {x,y,z,fx,fy,fz,0,0}; FP32x2 {-x,-x,-y,-y,-z,-z,fx,fx,fy,fy,fz,fz}.
__device__ void pack_blob_records(const GmresArgs &a, const double *f, int m) {
  const double *x = a.x_blobs + 3 * (size_t)m;
  if (!a.fp32) {
    double *r = reinterpret_cast<double *>(a.rec64) + 6 * (size_t)m;
    r[0] = x[0]; r[1] = x[1]; r[2] = x[2];
    r[3] = f[0]; r[4] = f[1]; r[5] = f[2];
  } else {
    const double *o = a.origin;
    float *r = reinterpret_cast<float *>(a.rec32) + 8 * (size_t)m;
    r[0] = float(x[0] - o[0]); r[1] = float(x[1] - o[1]); r[2] = float(x[2] - o[2]);
    r[3] = float(f[0]); r[4] = float(f[1]); r[5] = float(f[2]); r[6] = 0.f; r[7] = 0.f;
    float *q = reinterpret_cast<float *>(a.rec32x2) + 12 * (size_t)m;
    for (int k = 0; k < 3; ++k) {
      const float mk = float(o[k] - x[k]);
      q[2 * k] = mk;
      q[2 * k + 1] = mk;
      const float fk = float(f[k]);
      q[6 + 2 * k] = fk;
      q[6 + 2 * k + 1] = fk;
    }
  }
}

// out = P^-1 in (all n entries); `in` and `out` may not alias.
__device__ void precondition(const GmresArgs &a, double *out, const double *in, double *red,
                             double *sh6) {
  const int nb = a.nb, vel = 3 * nb;
  double b[6] = {0, 0, 0, 0, 0, 0};
  for (int m = threadIdx.x; m < nb; m += blockDim.x) {
    const double *d = a.diff + 3 * (size_t)m;
    const double *l = in + 3 * (size_t)m;
    b[0] -= l[0];
    b[1] -= l[1];
    b[2] -= l[2];
    b[3] -= d[1] * l[2] - d[2] * l[1];
    b[4] -= d[2] * l[0] - d[0] * l[2];
    b[5] -= d[0] * l[1] - d[1] * l[0];
  }
  block_sum6(b, red);
  if (threadIdx.x == 0) {
    double t1[6], t2[6];
    matvec6(t1, a.mats + 36, b);     // rotated KTKinv
    matvec6(t2, a.mats, in + vel);   // rotated body mobility
    for (int k = 0; k < 6; ++k) sh6[k] = t1[k] - t2[k];
  }
  __syncthreads();
  const double minv = 6.0 * kPiD * a.mu * a.a_blob;
  for (int m = threadIdx.x; m < nb; m += blockDim.x) {
    const double *d = a.diff + 3 * (size_t)m;
    const double *l = in + 3 * (size_t)m;
    double blk0 = l[0] + sh6[0], blk1 = l[1] + sh6[1], blk2 = l[2] + sh6[2];
    blk0 += sh6[4] * d[2] - sh6[5] * d[1];
    blk1 += sh6[5] * d[0] - sh6[3] * d[2];
    blk2 += sh6[3] * d[1] - sh6[4] * d[0];
    out[3 * (size_t)m] = minv * blk0;
    out[3 * (size_t)m + 1] = minv * blk1;
    out[3 * (size_t)m + 2] = minv * blk2;
  }
  if (threadIdx.x < 6) out[vel + threadIdx.x] = sh6[threadIdx.x];
  __syncthreads();
}

// w = A x given v = M_bb x_lambda (all n entries of w).
__device__ void finish_system_mult(const GmresArgs &a, double *w, const double *x,
                                   const double *v, double *red) {
  const int nb = a.nb, vel = 3 * nb;
  const double U0 = x[vel], U1 = x[vel + 1], U2 = x[vel + 2];
  const double W0 = x[vel + 3], W1 = x[vel + 4], W2 = x[vel + 5];
  double s[6] = {0, 0, 0, 0, 0, 0};
  for (int m = threadIdx.x; m < nb; m += blockDim.x) {
    const double *d = a.diff + 3 * (size_t)m;
    const double *l = x + 3 * (size_t)m;
    s[0] -= l[0];
    s[1] -= l[1];
    s[2] -= l[2];
    s[3] -= d[1] * l[2] - d[2] * l[1];
    s[4] -= d[2] * l[0] - d[0] * l[2];
    s[5] -= d[0] * l[1] - d[1] * l[0];
    const double *vv = v + 3 * (size_t)m;
    w[3 * (size_t)m] = -(U0 - d[1] * W2 + d[2] * W1) + vv[0];
    w[3 * (size_t)m + 1] = -(U1 - d[2] * W0 + d[0] * W2) + vv[1];
    w[3 * (size_t)m + 2] = -(U2 - d[0] * W1 + d[1] * W0) + vv[2];
  }
  block_sum6(s, red);
  if (threadIdx.x < 6) w[vel + threadIdx.x] = s[threadIdx.x];
  __syncthreads();
}

__device__ double block_dot(const double *x, const double *y, int n, double *red) {
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += x[i] * y[i];
  return block_sum(s, red);
}

// ---------------------------------------------------------------------------
// Phase kernels (one CTA per solve).
// ---------------------------------------------------------------------------

// Start: ||rhs||, zero-rhs exit, soln = warm start, pack soln_lambda for M_bb.
__global__ void __launch_bounds__(kSolveThreads) gmres_start_kernel(GmresArgs a) {
  __shared__ double red[6 * 33];
  GmresScalars *st = a.st;
  const int n = a.n, vel = 3 * a.nb;
  double ss = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) ss += a.rhs[i] * a.rhs[i];
  const double nr = sqrt(block_sum(ss, red));
  if (threadIdx.x == 0) {
    st->norm_rhs = nr;
    st->iter = 0;
    st->done = 0;
    st->iters = 0;
    st->status = 0;
    st->rel = 0.0;
  }
  if (nr == 0.0) {
    // the solution is zero (mobility_solver.cpp:2158-2170)
    for (int i = threadIdx.x; i < vel; i += blockDim.x) a.f_blobs[i] = 0.0;
    if (threadIdx.x < 6) a.v_bodies[threadIdx.x] = 0.0;
    if (threadIdx.x == 0) st->done = 1;
    return;
  }
  for (int i = threadIdx.x; i < vel; i += blockDim.x) a.soln[i] = a.f_blobs[i];
  if (threadIdx.x < 6) a.soln[vel + threadIdx.x] = a.v_bodies[threadIdx.x];
  __syncthreads();
  for (int m = threadIdx.x; m < a.nb; m += blockDim.x) pack_blob_records(a, a.soln + 3 * m, m);
}

// r0 = rhs - A soln, the warm-start tests, Q_0 = r0 / beta_0.
__global__ void __launch_bounds__(kSolveThreads) gmres_residual_kernel(GmresArgs a) {
  __shared__ double red[6 * 33];
  GmresScalars *st = a.st;
  if (st->done) return;
  const int n = a.n;
  double *q0 = a.Q;
  finish_system_mult(a, q0, a.soln, a.v, red);  // q0 = A soln
  double ss = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double r = a.rhs[i] - q0[i];
    q0[i] = r;
    ss += r * r;
  }
  double beta0 = sqrt(block_sum(ss, red));
  const double nr = st->norm_rhs;
  if (fabs(beta0) <= a.tol * nr) {
    // the warm start already solves the system (mobility_solver.cpp:2304-2307)
    if (threadIdx.x == 0) st->done = 1;
    return;
  }
  if (fabs(beta0) > nr) {
    // discard a poor warm start (:2313-2320)
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      a.soln[i] = 0.0;
      q0[i] = a.rhs[i];
    }
    beta0 = nr;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) q0[i] /= beta0;
  if (threadIdx.x == 0) {
    a.beta[0] = beta0;
    st->iter = 1;
  }
}

// z = P^-1 Q_{k-1}; pack z_lambda for M_bb.
__global__ void __launch_bounds__(kSolveThreads) gmres_precond_kernel(GmresArgs a) {
  __shared__ double red[6 * 33];
  __shared__ double sh6[6];
  GmresScalars *st = a.st;
  if (st->done) return;
  const int k = st->iter;
  precondition(a, a.z, a.Q + (size_t)(k - 1) * a.n, red, sh6);
  for (int m = threadIdx.x; m < a.nb; m += blockDim.x) pack_blob_records(a, a.z + 3 * m, m);
}

// Q_k = A z (from v = M_bb z_lambda), modified Gram-Schmidt, Givens
// rotations, convergence; on exit the back solve, x = x0 + P^-1 Q y and the
// solution written to (f_blobs, v_bodies).
//
// The new basis vector w is kept in shared memory when it fits (dynamic
// shared memory of n doubles; otherwise it lives in its Q column) and every
// thread owns the same entries throughout, so the Gram-Schmidt steps need no
// barrier beyond their reductions. Each step fuses the previous step's update
// w -= h_{i-1} q_{i-1} with the next dot product <w, q_i>: the operations on
// w are those of modified Gram-Schmidt, in the same order.
__global__ void __launch_bounds__(kSolveThreads) gmres_arnoldi_kernel(GmresArgs a) {
  __shared__ double red[6 * 33];
  __shared__ double sh6[6];
  __shared__ int finish;
  extern __shared__ double wsm[];
  GmresScalars *st = a.st;
  if (st->done) return;
  const int n = a.n, k = st->iter, ld = a.max_iter + 1;
  double *qk = a.Q + (size_t)k * n;
  double *H = a.H;
  double *w = a.w_in_smem ? wsm : qk;
  finish_system_mult(a, w, a.z, a.v, red);
  double hprev = 0.0;
  const double *qprev = nullptr;
  for (int i = 0; i < k; ++i) {
    const double *qi = a.Q + (size_t)i * n;
    double part = 0.0;
    for (int t = threadIdx.x; t < n; t += blockDim.x) {
      double wt = w[t];
      if (qprev) wt -= hprev * qprev[t];
      w[t] = wt;
      part += wt * qi[t];
    }
    const double h = block_sum(part, red);
    if (threadIdx.x == 0) H[i + (size_t)(k - 1) * ld] = h;
    hprev = h;
    qprev = qi;
  }
  double part = 0.0;
  for (int t = threadIdx.x; t < n; t += blockDim.x) {
    double wt = w[t];
    if (qprev) wt -= hprev * qprev[t];
    w[t] = wt;
    part += wt * wt;
  }
  const double qn = sqrt(block_sum(part, red));
  for (int t = threadIdx.x; t < n; t += blockDim.x) qk[t] = w[t] / qn;
  if (threadIdx.x == 0) {
    double *cs = a.cs, *sn = a.sn, *beta = a.beta;
#define HH(i, j) H[(i) + (size_t)(j) * ld]
    HH(k, k - 1) = qn;
    for (int i = 1; i < k; ++i) {
      const double t = cs[i - 1] * HH(i - 1, k - 1) + sn[i - 1] * HH(i, k - 1);
      HH(i, k - 1) = cs[i - 1] * HH(i, k - 1) - sn[i - 1] * HH(i - 1, k - 1);
      HH(i - 1, k - 1) = t;
    }
    const double hd = HH(k - 1, k - 1), hs = HH(k, k - 1);
    if (hs == 0.0) {
      cs[k - 1] = 1.0;
      sn[k - 1] = 0.0;
    } else if (fabs(hs) > fabs(hd)) {
      const double t = hd / hs;
      sn[k - 1] = (2.0 * (double)(hs > 0) - 1.0) / sqrt(1.0 + t * t);
      cs[k - 1] = t * sn[k - 1];
    } else {
      const double t = hs / hd;
      cs[k - 1] = (2.0 * (double)(hd > 0) - 1.0) / sqrt(1.0 + t * t);
      sn[k - 1] = t * cs[k - 1];
    }
    HH(k - 1, k - 1) = cs[k - 1] * hd + sn[k - 1] * hs;
    HH(k, k - 1) = 0.0;
    beta[k] = -sn[k - 1] * beta[k - 1];
    beta[k - 1] = cs[k - 1] * beta[k - 1];
    const double rel = fabs(beta[k]) / st->norm_rhs;
    st->rel = rel;
    finish = (rel <= a.tol || k == a.max_iter) ? 1 : 0;
    if (!(rel == rel)) {  // NaN: stop and report
      finish = 1;
      st->status = 1;
    }
    if (finish) {
      double *y = a.y;
      y[k - 1] = beta[k - 1] / HH(k - 1, k - 1);
      for (int i = k - 2; i >= 0; --i) {
        double yi = beta[i];
        for (int j = k - 1; j > i; --j) yi -= HH(i, j) * y[j];
        y[i] = yi / HH(i, i);
      }
    }
#undef HH
  }
  __syncthreads();
  if (!finish) {
    if (threadIdx.x == 0) st->iter = k + 1;
    return;
  }
  // tmp = Q_{0..k-1} y; soln += P^-1 tmp
  for (int t = threadIdx.x; t < n; t += blockDim.x) {
    double s = 0.0;
    for (int i = 0; i < k; ++i) s += a.y[i] * a.Q[(size_t)i * n + t];
    a.tmp[t] = s;
  }
  __syncthreads();
  precondition(a, a.z, a.tmp, red, sh6);
  const int vel = 3 * a.nb;
  for (int t = threadIdx.x; t < n; t += blockDim.x) {
    const double x = a.soln[t] + a.z[t];
    a.soln[t] = x;
    if (t < vel) a.f_blobs[t] = x;
    else a.v_bodies[t - vel] = x;
  }
  if (threadIdx.x == 0) {
    st->iters = k;
    st->done = 1;
  }
}

// ---------------------------------------------------------------------------
// Iterative refinement (FP32C): the outer FP64 residual and update.
// ---------------------------------------------------------------------------

// r = rhs - A x (v = M_bb x_lambda in FP64), rel = ||r|| / ||rhs||; done when
// rel <= tol (or rhs = 0, where x = 0). Zeroes the correction dx.
__global__ void __launch_bounds__(kSolveThreads) refine_residual_kernel(GmresArgs a,
                                                                        const double *x,
                                                                        double *r, double *dx,
                                                                        int outer) {
  __shared__ double red[6 * 33];
  GmresScalars *st = a.st;
  const int n = a.n;
  finish_system_mult(a, r, x, a.v, red);  // r = A x
  double rr = 0.0, bb = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double b = a.rhs[i];
    const double t = b - r[i];
    r[i] = t;
    rr += t * t;
    bb += b * b;
    dx[i] = 0.0;
  }
  const double nr = sqrt(block_sum(rr, red));
  const double nb = sqrt(block_sum(bb, red));
  if (threadIdx.x == 0) {
    if (outer == 0) st->status = 0;
    st->norm_rhs = nb;
    st->rel = nb > 0.0 ? nr / nb : 0.0;
    st->iter = outer;
    st->done = (nb == 0.0 || nr <= a.tol * nb) ? 1 : 0;
    if (!(nr == nr)) {
      st->done = 1;
      st->status = 1;
    }
  }
  if (nb == 0.0)
    for (int i = threadIdx.x; i < n; i += blockDim.x) r[i] = 0.0;
}

__global__ void axpy_kernel(double *x, const double *d, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    x[i] += d[i];
}

cudaError_t launch_refine_residual(const GmresArgs &a, const double *x, double *r, double *dx,
                                   int outer, cudaStream_t st) {
  refine_residual_kernel<<<1, kSolveThreads, 0, st>>>(a, x, r, dx, outer);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_axpy(double *x, const double *d, int n, cudaStream_t st) {
  axpy_kernel<<<(n + 255) / 256, 256, 0, st>>>(x, d, n);
  count_launch();
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Small helpers of the compute_velocities sequence.
// ---------------------------------------------------------------------------

// x_blobs = body_x + R ref_m, diff_m = R ref_m (rigid_body::blob_positions).
__global__ void blob_positions_kernel(double *x_blobs, double *diff, const double *refs, int nb,
                                      BodyPose pose) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= nb) return;
  const double *r = refs + 3 * (size_t)m;
  for (int i = 0; i < 3; ++i) {
    const double d = pose.R[i] * r[0] + pose.R[i + 3] * r[1] + pose.R[i + 6] * r[2];
    diff[3 * (size_t)m + i] = d;
    x_blobs[3 * (size_t)m + i] = pose.x[i] + d;
  }
}

// swimmer_f += sum_m (frep_m ; d_m x frep_m) (mobility_solver.cpp:208-234),
// then rhs = [-v_blobs ; -swimmer_f] (assemble_rhs :439-570).
__global__ void __launch_bounds__(kSolveThreads) rhs_kernel(const double *frep,
                                                             const double *diff,
                                                             const double *v_blobs, int nb,
                                                             double *swimmer_f, double *rhs) {
  __shared__ double red[6 * 33];
  double s[6] = {0, 0, 0, 0, 0, 0};
  for (int m = threadIdx.x; m < nb; m += blockDim.x) {
    const double *r = diff + 3 * (size_t)m, *f = frep + 3 * (size_t)m;
    s[0] += f[0];
    s[1] += f[1];
    s[2] += f[2];
    s[3] += r[1] * f[2] - r[2] * f[1];
    s[4] += r[2] * f[0] - r[0] * f[2];
    s[5] += r[0] * f[1] - r[1] * f[0];
  }
  block_sum6(s, red);
  for (int i = threadIdx.x; i < 3 * nb; i += blockDim.x) rhs[i] = -v_blobs[i];
  if (threadIdx.x < 6) {
    const double f = swimmer_f[threadIdx.x] + s[threadIdx.x];
    swimmer_f[threadIdx.x] = f;
    rhs[3 * nb + threadIdx.x] = -f;
  }
}

// rhs = -e_{n-1-j} (make_body_reference_matrices, mobility_solver.cpp:2996-3000)
__global__ void unit_rhs_kernel(double *rhs, int n, int j) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    rhs[i] = (i == n - 1 - j) ? -1.0 : 0.0;
}

// column 5-j of the body mobility = v_bodies
__global__ void store_body_column_kernel(double *body_mob, const double *v_bodies, int j) {
  if (threadIdx.x < 6) body_mob[threadIdx.x + 6 * (5 - j)] = v_bodies[threadIdx.x];
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
cudaError_t launch_gmres_start(const GmresArgs &a, cudaStream_t st) {
  gmres_start_kernel<<<1, kSolveThreads, 0, st>>>(a);
  count_launch();
  return cudaGetLastError();
}
cudaError_t launch_gmres_residual(const GmresArgs &a, cudaStream_t st) {
  gmres_residual_kernel<<<1, kSolveThreads, 0, st>>>(a);
  count_launch();
  return cudaGetLastError();
}
cudaError_t launch_gmres_precond(const GmresArgs &a, cudaStream_t st) {
  gmres_precond_kernel<<<1, kSolveThreads, 0, st>>>(a);
  count_launch();
  return cudaGetLastError();
}
// Largest basis vector kept in shared memory by the Arnoldi kernel.
constexpr int kMaxSmemVector = 24 * 1024;  // doubles (192 KB)

bool gmres_w_fits_smem(int n) { return n <= kMaxSmemVector; }

cudaError_t launch_gmres_arnoldi(const GmresArgs &a, cudaStream_t st) {
  static bool configured = false;
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(gmres_arnoldi_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)(sizeof(double) * kMaxSmemVector));
    if (e != cudaSuccess) return e;
    configured = true;
  }
  const size_t smem = a.w_in_smem ? sizeof(double) * a.n : 0;
  gmres_arnoldi_kernel<<<1, kSolveThreads, smem, st>>>(a);
  count_launch();
  return cudaGetLastError();
}
cudaError_t launch_blob_positions(double *x_blobs, double *diff, const double *refs, int nb,
                                  const BodyPose &pose, cudaStream_t st) {
  if (nb <= 0) return cudaSuccess;
  blob_positions_kernel<<<(nb + 255) / 256, 256, 0, st>>>(x_blobs, diff, refs, nb, pose);
  count_launch();
  return cudaGetLastError();
}
cudaError_t launch_rhs(const double *frep, const double *diff, const double *v_blobs, int nb,
                       double *swimmer_f, double *rhs, cudaStream_t st) {
  rhs_kernel<<<1, kSolveThreads, 0, st>>>(frep, diff, v_blobs, nb, swimmer_f, rhs);
  count_launch();
  return cudaGetLastError();
}
cudaError_t launch_unit_rhs(double *rhs, int n, int j, cudaStream_t st) {
  unit_rhs_kernel<<<(n + 255) / 256, 256, 0, st>>>(rhs, n, j);
  count_launch();
  return cudaGetLastError();
}
cudaError_t launch_store_body_column(double *body_mob, const double *v_bodies, int j,
                                     cudaStream_t st) {
  store_body_column_kernel<<<1, 32, 0, st>>>(body_mob, v_bodies, j);
  count_launch();
  return cudaGetLastError();
}

}  // namespace tfs
