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
// started from the previous (lambda, U, Omega), the reference's Givens sign
// convention, stopping when |beta_k| / ||rhs|| <= tol or after
// min(n, max_iter) steps.
//
// Work split. GB300 issues 2 FP64 FMAs per clock per SM, so the FP64 vector
// work of an Arnoldi step (~4 k n FMAs at step k) is spread over the SMs: the
// blobs are cut into G contiguous slices, one CTA each (the last CTA also owns
// the 6 body rows). Every reduction (the preconditioner's and K^T's 6-vectors,
// the Gram-Schmidt dot products, norms) is finished by the last CTA to
// arrive: each CTA writes its partial sums, and the CTA that takes the last
// ticket of the kernel's counter adds them in CTA order (deterministic),
// does the scalar work (6x6 products, Givens rotations, convergence test) and
// resets the counter. Orthogonalisation is classical Gram-Schmidt applied
// twice (CGS2: the second pass re-orthogonalises against the same basis),
// two reductions per step instead of one per basis vector.
//
// Every vector and scalar lives on the device; the blob-blob product M_bb
// runs on the tile kernel (rpy_kernels.cu) between the phases. A `done` flag
// in device memory makes the iteration kernels return at once, so the host
// launches steps in chunks and polls the flag between chunks.
#include <cuda_runtime.h>

#include <algorithm>

#include "gmres.h"
#include "tfs_kernels.h"

namespace tfs {

constexpr double kPiD = 3.14159265358979323846264338327950288;
constexpr int kGT = 128;  // threads per CTA of the GMRES kernels

// ---------------------------------------------------------------------------
// helpers
// ---------------------------------------------------------------------------

struct Slice {
  int m0, m1;  // blobs [m0, m1)
  bool body;   // this CTA owns the six body rows
};

__device__ __forceinline__ Slice my_slice(const GmresArgs &a) {
  Slice s;
  s.m0 = min(a.nb, (int)blockIdx.x * a.blobs_per_cta);
  s.m1 = min(a.nb, s.m0 + a.blobs_per_cta);
  s.body = blockIdx.x == gridDim.x - 1;
  return s;
}

// Block sum of L values per thread into sh[0..L); all threads get them.
// red holds >= 32 * L doubles.
template <int L>
__device__ void block_sum_vec(double (&v)[L], double *red, double *sh) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int k = 0; k < L; ++k)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
  __syncthreads();
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < L; ++k) red[L * wid + k] = v[k];
  __syncthreads();
  if (threadIdx.x < L) {
    double t = 0.0;
    for (int w = 0; w < nw; ++w) t += red[L * w + threadIdx.x];
    sh[threadIdx.x] = t;
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < L; ++k) v[k] = sh[k];
}

// Sum of n strided per-CTA partials p[c * stride], c < n, by one warp: lanes
// take c = lane (mod 32), then a fixed shuffle tree, so every lane gets the
// same bits. (GB300 issues an FP64 warp instruction in ~19 SM cycles: a
// single thread adding G partials in sequence costs microseconds.)
__device__ __forceinline__ double warp_sum_strided(const double *p, int n, size_t stride) {
  double t = 0.0;
  for (int c = threadIdx.x & 31; c < n; c += 32) t += __ldcg(p + (size_t)c * stride);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  return t;
}

// The rows of a slice: its blobs' rows, then (last CTA) the six body rows.
__device__ __forceinline__ int slice_rows(const Slice &sl) {
  return 3 * (sl.m1 - sl.m0) + (sl.body ? 6 : 0);
}
__device__ __forceinline__ int slice_row(const GmresArgs &a, const Slice &sl, int r) {
  const int nblob_rows = 3 * (sl.m1 - sl.m0);
  return r < nblob_rows ? 3 * sl.m0 + r : 3 * a.nb + (r - nblob_rows);
}

// k dot products <w, Q_i> over this CTA's rows (blob rows only when
// with_body is false) into part[blockIdx.x * stride + i]. red holds >= 32*64.
__device__ void block_dots(const GmresArgs &a, const Slice &sl, bool with_body, const double *w,
                           int k, double *part, int stride, double *red) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int rows = 3 * (sl.m1 - sl.m0) + (with_body && sl.body ? 6 : 0);
  for (int i = 0; i < k; ++i) {
    const double *qi = a.Q + (size_t)i * a.n;
    double v = 0.0;
    for (int r = threadIdx.x; r < rows; r += blockDim.x) {
      const int t = slice_row(a, sl, r);
      v += w[t] * qi[t];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) red[wid * 64 + (i & 63)] = v;
    if ((i & 63) == 63 || i == k - 1) {
      __syncthreads();
      const int base = i & ~63;
      if ((int)threadIdx.x <= i - base) {
        double t = 0.0;
        for (int ww = 0; ww < nw; ++ww) t += red[ww * 64 + threadIdx.x];
        part[(size_t)blockIdx.x * stride + base + threadIdx.x] = t;
      }
      __syncthreads();
    }
  }
}

// Last-CTA election: every CTA calls this after writing its partials; it
// returns true in exactly one CTA (the last to arrive), which then sees all
// partials and must reset the counter. The last CTA reads the other CTAs'
// partials with ld.global.cg (__ldcg, L2): L1 is not coherent across SMs, and
// a line of the partial array cached by an earlier launch's last CTA on the
// same SM could otherwise be read stale while other streams keep the SM busy.
__device__ bool last_cta(unsigned *counter) {
  __shared__ bool last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(counter, 1u) == gridDim.x - 1;
  __syncthreads();
  if (last) __threadfence();
  return last;
}

__device__ void matvec6(double *out, const double *M, const double *v) {
  for (int i = 0; i < 6; ++i) {
    double s = 0.0;
    for (int k = 0; k < 6; ++k) s += M[i + 6 * k] * v[k];
    out[i] = s;
  }
}

// Blob force records for the M_bb product (FP64 / FP32 / FP32x2 formats).
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

// sum over this CTA's blobs of (l_m ; d_m x l_m) into part6[blockIdx.x]
__device__ void kt_partial(const GmresArgs &a, const Slice &sl, const double *l, double *part6,
                           double *red, double *sh) {
  double s[6] = {0, 0, 0, 0, 0, 0};
  for (int m = sl.m0 + threadIdx.x; m < sl.m1; m += blockDim.x) {
    const double *d = a.diff + 3 * (size_t)m;
    const double *v = l + 3 * (size_t)m;
    s[0] += v[0];
    s[1] += v[1];
    s[2] += v[2];
    s[3] += d[1] * v[2] - d[2] * v[1];
    s[4] += d[2] * v[0] - d[0] * v[2];
    s[5] += d[0] * v[1] - d[1] * v[0];
  }
  block_sum_vec<6>(s, red, sh);
  if (threadIdx.x < 6) part6[6 * blockIdx.x + threadIdx.x] = s[threadIdx.x];
}

// sum over CTAs (in order) of part6, by the last CTA; result in sh[0..6)
__device__ void sum_part6(const double *part6, int G, double *sh) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int k = wid; k < 6; k += nw) {
    const double t = warp_sum_strided(part6 + k, G, 6);
    if (lane == 0) sh[k] = t;
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
// preconditioner: out = P^-1 in, in two kernels
// ---------------------------------------------------------------------------

// (1) b = -sum_m (in_m ; d_m x in_m); the last CTA forms the body rows
//     out_vel = KTKinv b - N in_vel. use_iter: in = Q_{k-1}.
__global__ void __launch_bounds__(kGT) precond_reduce_kernel(GmresArgs a, const double *in_base,
                                                             double *out, int use_iter) {
  __shared__ double red[32 * 8], sh[8];
  GmresScalars *st = a.st;
  if (use_iter && st->done) return;
  const double *in = use_iter ? in_base + (size_t)(st->iter - 1) * a.n : in_base;
  const Slice sl = my_slice(a);
  kt_partial(a, sl, in, a.part6, red, sh);
  if (!last_cta(a.counters + 0)) return;
  sum_part6(a.part6, gridDim.x, sh);
  if (threadIdx.x == 0) {
    double b[6], t1[6], t2[6];
    for (int k = 0; k < 6; ++k) b[k] = -sh[k];
    matvec6(t1, a.mats + 36, b);         // rotated KTKinv
    matvec6(t2, a.mats, in + 3 * a.nb);  // rotated body mobility
    for (int k = 0; k < 6; ++k) out[3 * a.nb + k] = t1[k] - t2[k];
    a.counters[0] = 0;
  }
}

// (2) out_m = 6 pi mu a (in_m + U' + Omega' x d_m); optionally pack out_lambda
//     as blob records for M_bb.
__global__ void __launch_bounds__(kGT) precond_apply_kernel(GmresArgs a, const double *in_base,
                                                            double *out, int use_iter,
                                                            int pack) {
  GmresScalars *st = a.st;
  if (use_iter && st->done) return;
  const double *in = use_iter ? in_base + (size_t)(st->iter - 1) * a.n : in_base;
  const Slice sl = my_slice(a);
  const double *U = out + 3 * a.nb;
  const double u0 = U[0], u1 = U[1], u2 = U[2], w0 = U[3], w1 = U[4], w2 = U[5];
  const double minv = 6.0 * kPiD * a.mu * a.a_blob;
  for (int m = sl.m0 + threadIdx.x; m < sl.m1; m += blockDim.x) {
    const double *d = a.diff + 3 * (size_t)m;
    const double *l = in + 3 * (size_t)m;
    double b0 = l[0] + u0, b1 = l[1] + u1, b2 = l[2] + u2;
    b0 += w1 * d[2] - w2 * d[1];
    b1 += w2 * d[0] - w0 * d[2];
    b2 += w0 * d[1] - w1 * d[0];
    double *o = out + 3 * (size_t)m;
    o[0] = minv * b0;
    o[1] = minv * b1;
    o[2] = minv * b2;
    if (pack) pack_blob_records(a, o, m);
  }
}

// ---------------------------------------------------------------------------
// start and residual
// ---------------------------------------------------------------------------

// ||rhs|| (last CTA), soln = warm start, pack soln_lambda for M_bb.
__global__ void __launch_bounds__(kGT) gmres_start_kernel(GmresArgs a) {
  __shared__ double red[32 * 8], sh[8];
  GmresScalars *st = a.st;
  const Slice sl = my_slice(a);
  const int vel = 3 * a.nb;
  double ss[1] = {0.0};
  for (int t = 3 * sl.m0 + threadIdx.x; t < 3 * sl.m1; t += blockDim.x) {
    ss[0] += a.rhs[t] * a.rhs[t];
    a.soln[t] = a.f_blobs[t];
  }
  for (int m = sl.m0 + threadIdx.x; m < sl.m1; m += blockDim.x)
    pack_blob_records(a, a.f_blobs + 3 * (size_t)m, m);
  if (sl.body && threadIdx.x < 6) {
    ss[0] += a.rhs[vel + threadIdx.x] * a.rhs[vel + threadIdx.x];
    a.soln[vel + threadIdx.x] = a.v_bodies[threadIdx.x];
  }
  block_sum_vec<1>(ss, red, sh);
  if (threadIdx.x == 0) a.part[blockIdx.x] = ss[0];
  if (!last_cta(a.counters + 1)) return;
  const double tsum = threadIdx.x < 32 ? warp_sum_strided(a.part, gridDim.x, 1) : 0.0;
  if (threadIdx.x == 0) {
    const double t = tsum;
    st->norm_rhs = sqrt(t);
    st->iter = 0;
    st->done = 0;
    st->iters = 0;
    st->status = 0;
    st->rel = 0.0;
    st->flag = 0;
    a.counters[1] = 0;
  }
}

// r0 = rhs - A soln into Q_0 (blob rows per CTA; body rows by the last CTA),
// beta_0 = ||r0||, and the warm-start tests (mobility_solver.cpp:2279-2320):
// flag 1 = the warm start already solves the system (done), 2 = discard it,
// 3 = zero right-hand side (the solution is zero, :2158-2170).
__global__ void __launch_bounds__(kGT) gmres_residual_kernel(GmresArgs a) {
  __shared__ double red[32 * 8], sh[8];
  GmresScalars *st = a.st;
  const Slice sl = my_slice(a);
  const int vel = 3 * a.nb;
  double *q0 = a.Q;
  const double *x = a.soln;
  const double u0 = x[vel], u1 = x[vel + 1], u2 = x[vel + 2];
  const double w0 = x[vel + 3], w1 = x[vel + 4], w2 = x[vel + 5];
  double ss[1] = {0.0};
  for (int m = sl.m0 + threadIdx.x; m < sl.m1; m += blockDim.x) {
    const double *d = a.diff + 3 * (size_t)m;
    const double *v = a.v + 3 * (size_t)m;
    const double *b = a.rhs + 3 * (size_t)m;
    const double r0 = b[0] - (-(u0 - d[1] * w2 + d[2] * w1) + v[0]);
    const double r1 = b[1] - (-(u1 - d[2] * w0 + d[0] * w2) + v[1]);
    const double r2 = b[2] - (-(u2 - d[0] * w1 + d[1] * w0) + v[2]);
    q0[3 * (size_t)m] = r0;
    q0[3 * (size_t)m + 1] = r1;
    q0[3 * (size_t)m + 2] = r2;
    ss[0] += r0 * r0 + r1 * r1 + r2 * r2;
  }
  kt_partial(a, sl, x, a.part6, red, sh);
  block_sum_vec<1>(ss, red, sh);
  if (threadIdx.x == 0) a.part[blockIdx.x] = ss[0];
  if (!last_cta(a.counters + 2)) return;
  sum_part6(a.part6, gridDim.x, sh);
  const double tsum = threadIdx.x < 32 ? warp_sum_strided(a.part, gridDim.x, 1) : 0.0;
  if (threadIdx.x == 0) {
    double t = tsum;
    for (int k = 0; k < 6; ++k) {
      const double r = a.rhs[vel + k] - (-sh[k]);
      q0[vel + k] = r;
      t += r * r;
    }
    const double nr = st->norm_rhs;
    double beta0 = sqrt(t);
    int flag = 0;
    if (nr == 0.0) {
      flag = 3;
    } else if (fabs(beta0) <= a.tol * nr) {
      flag = 1;
    } else if (fabs(beta0) > nr) {
      flag = 2;
      beta0 = nr;
    }
    a.beta[0] = beta0;
    st->flag = flag;
    if (flag == 1 || flag == 3) st->done = 1;
    else st->iter = 1;
    a.counters[2] = 0;
  }
}

// Q_0 /= beta_0 (or Q_0 = rhs / ||rhs|| and soln = 0 for a discarded warm
// start); for a zero right-hand side, f_blobs = v_bodies = 0.
__global__ void __launch_bounds__(kGT) gmres_residual_scale_kernel(GmresArgs a) {
  GmresScalars *st = a.st;
  const Slice sl = my_slice(a);
  const int flag = st->flag;
  const double beta0 = a.beta[0];
  if (flag == 1) return;
  const int rows = slice_rows(sl);
  for (int r = threadIdx.x; r < rows; r += blockDim.x) {
    const int t = slice_row(a, sl, r);
    if (flag == 3) {
      if (t < 3 * a.nb) a.f_blobs[t] = 0.0;
      else a.v_bodies[t - 3 * a.nb] = 0.0;
    } else if (flag == 2) {
      a.soln[t] = 0.0;
      a.Q[t] = a.rhs[t] / beta0;
    } else {
      a.Q[t] /= beta0;
    }
  }
}

// ---------------------------------------------------------------------------
// Arnoldi step k: w = A z into Q_k, CGS2 against Q_0..Q_{k-1}, norm, Givens.
// ---------------------------------------------------------------------------

// w_blob = M_bb z_lambda - (U + Omega x d_m) (v = M_bb z from the tile
// kernel); first-pass dots over blob rows; the last CTA adds the body rows
// w_vel = -sum (z_m ; d_m x z_m) and their dot terms: h1.
__global__ void __launch_bounds__(kGT) arnoldi_dot1_kernel(GmresArgs a) {
  __shared__ double red[32 * 64], sh[8];
  GmresScalars *st = a.st;
  if (st->done) return;
  const int k = st->iter, n = a.n, vel = 3 * a.nb;
  const Slice sl = my_slice(a);
  double *w = a.Q + (size_t)k * n;
  const double *z = a.z;
  const double u0 = z[vel], u1 = z[vel + 1], u2 = z[vel + 2];
  const double w0 = z[vel + 3], w1 = z[vel + 4], w2 = z[vel + 5];
  for (int m = sl.m0 + threadIdx.x; m < sl.m1; m += blockDim.x) {
    const double *d = a.diff + 3 * (size_t)m;
    const double *v = a.v + 3 * (size_t)m;
    w[3 * (size_t)m] = -(u0 - d[1] * w2 + d[2] * w1) + v[0];
    w[3 * (size_t)m + 1] = -(u1 - d[2] * w0 + d[0] * w2) + v[1];
    w[3 * (size_t)m + 2] = -(u2 - d[0] * w1 + d[1] * w0) + v[2];
  }
  kt_partial(a, sl, z, a.part6, red, sh);
  __syncthreads();
  block_dots(a, sl, false, w, k, a.part, a.part_stride, red);
  if (!last_cta(a.counters + 3)) return;
  sum_part6(a.part6, gridDim.x, sh);
  if (threadIdx.x < 6) w[vel + threadIdx.x] = -sh[threadIdx.x];
  __syncthreads();
  for (int i = threadIdx.x >> 5; i < k; i += blockDim.x >> 5) {
    double t = warp_sum_strided(a.part + i, gridDim.x, a.part_stride);
    if ((threadIdx.x & 31) == 0) {
      const double *qi = a.Q + (size_t)i * n;
      for (int j = 0; j < 6; ++j) t += w[vel + j] * qi[vel + j];
      a.h1[i] = t;
    }
  }
  if (threadIdx.x == 0) a.counters[3] = 0;
}

// w -= sum_i h1_i Q_i (this CTA's rows), then second-pass dots: h2, and
// H(:, k-1) = h1 + h2.
__global__ void __launch_bounds__(kGT) arnoldi_dot2_kernel(GmresArgs a) {
  __shared__ double red[32 * 64];
  GmresScalars *st = a.st;
  if (st->done) return;
  const int k = st->iter, n = a.n;
  const Slice sl = my_slice(a);
  double *w = a.Q + (size_t)k * n;
  const int rows = slice_rows(sl);
  for (int r = threadIdx.x; r < rows; r += blockDim.x) {
    const int t = slice_row(a, sl, r);
    double wt = w[t];
    for (int i = 0; i < k; ++i) wt -= a.h1[i] * a.Q[(size_t)i * n + t];
    w[t] = wt;
  }
  __syncthreads();
  block_dots(a, sl, true, w, k, a.part, a.part_stride, red);
  if (!last_cta(a.counters + 4)) return;
  const int ld = a.max_iter + 1;
  for (int i = threadIdx.x >> 5; i < k; i += blockDim.x >> 5) {
    const double t = warp_sum_strided(a.part + i, gridDim.x, a.part_stride);
    if ((threadIdx.x & 31) == 0) {
      a.h2[i] = t;
      a.H[i + (size_t)(k - 1) * ld] = a.h1[i] + t;
    }
  }
  if (threadIdx.x == 0) a.counters[4] = 0;
}

// w -= sum_i h2_i Q_i, ||w||; the last CTA applies the Givens rotations
// (mobility_solver.cpp:2370-2413), tests convergence and, when finishing,
// back-solves for y (:2419-2438).
__global__ void __launch_bounds__(kGT) arnoldi_norm_kernel(GmresArgs a) {
  __shared__ double red[32 * 8], sh[8];
  GmresScalars *st = a.st;
  if (st->done) return;
  const int k = st->iter, n = a.n;
  const Slice sl = my_slice(a);
  double *w = a.Q + (size_t)k * n;
  const int rows = slice_rows(sl);
  double ss[1] = {0.0};
  for (int r = threadIdx.x; r < rows; r += blockDim.x) {
    const int t = slice_row(a, sl, r);
    double wt = w[t];
    for (int i = 0; i < k; ++i) wt -= a.h2[i] * a.Q[(size_t)i * n + t];
    w[t] = wt;
    ss[0] += wt * wt;
  }
  block_sum_vec<1>(ss, red, sh);
  if (threadIdx.x == 0) a.part[blockIdx.x] = ss[0];
  if (!last_cta(a.counters + 5)) return;
  const double tsum = threadIdx.x < 32 ? warp_sum_strided(a.part, gridDim.x, 1) : 0.0;
  if (threadIdx.x == 0) {
    const double t = tsum;
    const double qn = sqrt(t);
    st->qnorm = qn;
    const int ld = a.max_iter + 1;
    double *H = a.H, *cs = a.cs, *sn = a.sn, *beta = a.beta;
#define HH(i, j) H[(i) + (size_t)(j) * ld]
    HH(k, k - 1) = qn;
    for (int i = 1; i < k; ++i) {
      const double tt = cs[i - 1] * HH(i - 1, k - 1) + sn[i - 1] * HH(i, k - 1);
      HH(i, k - 1) = cs[i - 1] * HH(i, k - 1) - sn[i - 1] * HH(i - 1, k - 1);
      HH(i - 1, k - 1) = tt;
    }
    const double hd = HH(k - 1, k - 1), hs = HH(k, k - 1);
    if (hs == 0.0) {
      cs[k - 1] = 1.0;
      sn[k - 1] = 0.0;
    } else if (fabs(hs) > fabs(hd)) {
      const double tt = hd / hs;
      sn[k - 1] = (2.0 * (double)(hs > 0) - 1.0) / sqrt(1.0 + tt * tt);
      cs[k - 1] = tt * sn[k - 1];
    } else {
      const double tt = hs / hd;
      cs[k - 1] = (2.0 * (double)(hd > 0) - 1.0) / sqrt(1.0 + tt * tt);
      sn[k - 1] = tt * cs[k - 1];
    }
    HH(k - 1, k - 1) = cs[k - 1] * hd + sn[k - 1] * hs;
    HH(k, k - 1) = 0.0;
    beta[k] = -sn[k - 1] * beta[k - 1];
    beta[k - 1] = cs[k - 1] * beta[k - 1];
    const double rel = fabs(beta[k]) / st->norm_rhs;
    st->rel = rel;
    bool finish = rel <= a.tol || k == a.max_iter;
    if (!(rel == rel)) {  // NaN: stop and report
      finish = true;
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
      st->iters = k;
      st->done = 1;
    } else {
      st->iter = k + 1;
    }
#undef HH
    a.counters[5] = 0;
  }
}

// Q_k = w / ||w|| (the step was not the last one).
__global__ void __launch_bounds__(kGT) arnoldi_scale_kernel(GmresArgs a) {
  GmresScalars *st = a.st;
  if (st->done) return;
  const int k = st->iter - 1, n = a.n;
  const Slice sl = my_slice(a);
  double *w = a.Q + (size_t)k * n;
  const double qn = st->qnorm;
  const int rows = slice_rows(sl);
  for (int r = threadIdx.x; r < rows; r += blockDim.x) {
    const int t = slice_row(a, sl, r);
    w[t] = w[t] / qn;
  }
}

// ---------------------------------------------------------------------------
// finish: tmp = Q y; z = P^-1 tmp; soln += z -> (f_blobs, v_bodies)
// (mobility_solver.cpp:2440-2563)
// ---------------------------------------------------------------------------

__global__ void __launch_bounds__(kGT) finish_qy_kernel(GmresArgs a) {
  const int k = a.st->iters, n = a.n;
  const Slice sl = my_slice(a);
  const int rows = slice_rows(sl);
  for (int r = threadIdx.x; r < rows; r += blockDim.x) {
    const int t = slice_row(a, sl, r);
    double s = 0.0;
    for (int i = 0; i < k; ++i) s += a.y[i] * a.Q[(size_t)i * n + t];
    a.tmp[t] = s;
  }
}

__global__ void __launch_bounds__(kGT) finish_update_kernel(GmresArgs a) {
  const int vel = 3 * a.nb;
  const Slice sl = my_slice(a);
  const int rows = slice_rows(sl);
  for (int r = threadIdx.x; r < rows; r += blockDim.x) {
    const int t = slice_row(a, sl, r);
    const double x = a.soln[t] + a.z[t];
    a.soln[t] = x;
    if (t < vel) a.f_blobs[t] = x;
    else a.v_bodies[t - vel] = x;
  }
}

// ---------------------------------------------------------------------------
// Iterative refinement (FP32C): the outer FP64 residual and update.
// ---------------------------------------------------------------------------

// r = rhs - A x (v = M_bb x_lambda in FP64), rel = ||r|| / ||rhs||; done when
// rel <= tol (or rhs = 0, where x = 0). Zeroes the correction dx.
__global__ void __launch_bounds__(kGT) refine_residual_kernel(GmresArgs a, const double *x,
                                                              double *r, double *dx,
                                                              int outer) {
  __shared__ double red[32 * 8], sh[8];
  GmresScalars *st = a.st;
  const Slice sl = my_slice(a);
  const int vel = 3 * a.nb;
  const double u0 = x[vel], u1 = x[vel + 1], u2 = x[vel + 2];
  const double w0 = x[vel + 3], w1 = x[vel + 4], w2 = x[vel + 5];
  double ss[2] = {0.0, 0.0};
  for (int m = sl.m0 + threadIdx.x; m < sl.m1; m += blockDim.x) {
    const double *d = a.diff + 3 * (size_t)m;
    const double *v = a.v + 3 * (size_t)m;
    const double *b = a.rhs + 3 * (size_t)m;
    const double ax[3] = {-(u0 - d[1] * w2 + d[2] * w1) + v[0],
                          -(u1 - d[2] * w0 + d[0] * w2) + v[1],
                          -(u2 - d[0] * w1 + d[1] * w0) + v[2]};
    for (int j = 0; j < 3; ++j) {
      const double rr = b[j] - ax[j];
      r[3 * (size_t)m + j] = rr;
      dx[3 * (size_t)m + j] = 0.0;
      ss[0] += rr * rr;
      ss[1] += b[j] * b[j];
    }
  }
  kt_partial(a, sl, x, a.part6, red, sh);
  block_sum_vec<2>(ss, red, sh);
  if (threadIdx.x == 0) {
    a.part[2 * blockIdx.x] = ss[0];
    a.part[2 * blockIdx.x + 1] = ss[1];
  }
  if (!last_cta(a.counters + 6)) return;
  sum_part6(a.part6, gridDim.x, sh);
  // warp 0: sum of r^2, warp 1: sum of b^2 over the CTAs' partials
  if (threadIdx.x < 64) {
    const double t = warp_sum_strided(a.part + (threadIdx.x >> 5), gridDim.x, 2);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = t;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double rr = red[0], bb = red[1];
    for (int k = 0; k < 6; ++k) {
      const double b = a.rhs[vel + k];
      const double t = b - (-sh[k]);
      r[vel + k] = t;
      dx[vel + k] = 0.0;
      rr += t * t;
      bb += b * b;
    }
    const double nr = sqrt(rr), nb = sqrt(bb);
    if (outer == 0) st->status = 0;
    st->norm_rhs = nb;
    st->rel = nb > 0.0 ? nr / nb : 0.0;
    st->iter = outer;
    st->done = (nb == 0.0 || nr <= a.tol * nb) ? 1 : 0;
    if (!(nr == nr)) {
      st->done = 1;
      st->status = 1;
    }
    a.counters[6] = 0;
  }
}

__global__ void axpy_kernel(double *x, const double *d, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    x[i] += d[i];
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
__global__ void __launch_bounds__(kGT) rhs_kernel(GmresArgs a, const double *frep,
                                                  const double *v_blobs, double *swimmer_f,
                                                  double *rhs) {
  __shared__ double red[32 * 8], sh[8];
  const Slice sl = my_slice(a);
  const int vel = 3 * a.nb;
  for (int t = 3 * sl.m0 + threadIdx.x; t < 3 * sl.m1; t += blockDim.x) rhs[t] = -v_blobs[t];
  kt_partial(a, sl, frep, a.part6, red, sh);
  if (!last_cta(a.counters + 7)) return;
  sum_part6(a.part6, gridDim.x, sh);
  if (threadIdx.x < 6) {
    const double f = swimmer_f[threadIdx.x] + sh[threadIdx.x];
    swimmer_f[threadIdx.x] = f;
    rhs[vel + threadIdx.x] = -f;
  }
  if (threadIdx.x == 0) a.counters[7] = 0;
}

// rhs = -e_{n-1-j} (make_body_reference_matrices, mobility_solver.cpp:2996-3000)
__global__ void unit_rhs_kernel(double *rhs, int n, int j) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    rhs[i] = (i == n - 1 - j) ? -1.0 : 0.0;
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------

// CTAs of the kernel-sequence GMRES: at least 32 blobs per CTA. Its kernels
// are latency-bound (a few grid-wide reductions per Arnoldi step); fewer CTAs
// shorten each last-CTA reduction and leave SMs to other swimmers' streams
// (measured on GB300: 32 blobs per CTA beats 4 by ~20% per step for 642 and
// 2562 blobs, results unchanged).
int gmres_grid(int nb, int sms, int *blobs_per_cta) {
  int G = std::max(1, std::min(sms, (nb + 31) / 32));
  int per = std::max(1, (nb + G - 1) / G);
  G = std::max(1, (nb + per - 1) / per);
  *blobs_per_cta = per;
  return G;
}

cudaError_t launch_gmres_start(const GmresArgs &a, cudaStream_t st) {
  gmres_start_kernel<<<a.G, kGT, 0, st>>>(a);
  count_launch();
  return cudaGetLastError();
}
cudaError_t launch_gmres_residual(const GmresArgs &a, cudaStream_t st) {
  gmres_residual_kernel<<<a.G, kGT, 0, st>>>(a);
  count_launch();
  gmres_residual_scale_kernel<<<a.G, kGT, 0, st>>>(a);
  count_launch();
  return cudaGetLastError();
}
cudaError_t launch_gmres_precond(const GmresArgs &a, cudaStream_t st) {
  precond_reduce_kernel<<<a.G, kGT, 0, st>>>(a, a.Q, a.z, 1);
  count_launch();
  precond_apply_kernel<<<a.G, kGT, 0, st>>>(a, a.Q, a.z, 1, 1);
  count_launch();
  return cudaGetLastError();
}
cudaError_t launch_gmres_arnoldi(const GmresArgs &a, cudaStream_t st) {
  arnoldi_dot1_kernel<<<a.G, kGT, 0, st>>>(a);
  count_launch();
  arnoldi_dot2_kernel<<<a.G, kGT, 0, st>>>(a);
  count_launch();
  arnoldi_norm_kernel<<<a.G, kGT, 0, st>>>(a);
  count_launch();
  arnoldi_scale_kernel<<<a.G, kGT, 0, st>>>(a);
  count_launch();
  return cudaGetLastError();
}
cudaError_t launch_gmres_finish(const GmresArgs &a, cudaStream_t st) {
  finish_qy_kernel<<<a.G, kGT, 0, st>>>(a);
  count_launch();
  precond_reduce_kernel<<<a.G, kGT, 0, st>>>(a, a.tmp, a.z, 0);
  count_launch();
  precond_apply_kernel<<<a.G, kGT, 0, st>>>(a, a.tmp, a.z, 0, 0);
  count_launch();
  finish_update_kernel<<<a.G, kGT, 0, st>>>(a);
  count_launch();
  return cudaGetLastError();
}
cudaError_t launch_refine_residual(const GmresArgs &a, const double *x, double *r, double *dx,
                                   int outer, cudaStream_t st) {
  refine_residual_kernel<<<a.G, kGT, 0, st>>>(a, x, r, dx, outer);
  count_launch();
  return cudaGetLastError();
}
cudaError_t launch_axpy(double *x, const double *d, int n, cudaStream_t st) {
  axpy_kernel<<<(n + 255) / 256, 256, 0, st>>>(x, d, n);
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
cudaError_t launch_rhs(const GmresArgs &a, const double *frep, const double *v_blobs,
                       double *swimmer_f, double *rhs, cudaStream_t st) {
  rhs_kernel<<<a.G, kGT, 0, st>>>(a, frep, v_blobs, swimmer_f, rhs);
  count_launch();
  return cudaGetLastError();
}
cudaError_t launch_unit_rhs(double *rhs, int n, int j, cudaStream_t st) {
  unit_rhs_kernel<<<(n + 255) / 256, 256, 0, st>>>(rhs, n, j);
  count_launch();
  return cudaGetLastError();
}

}  // namespace tfs
