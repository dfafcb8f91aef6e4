// prescribed.cu -- the prescribed-cilia mobility solve of one swimmer on the
// device: the reference's mobility_solver compute_velocities under
// PRESCRIBED_CILIA (mobility_solver.cpp:2574-2596), with assemble_rhs
// (:282-437), solve_linear_system (:2092-2570), apply_preconditioner_new
// (:1040-1436), system_matrix_mult_new (:1806-2026) and
// swimmer::make_precon_mat (swimmer.cpp:1154-1322).
//
// Unknowns, in the reference's order: segment forces (3 Ns), blob forces
// (3 Nb), body U and Omega (6, free body), phase rates (nfil, dynamic phase),
// shape-rotation rates (nfil, dynamic shape rotation). The operator is the
// translational RPY mobility of every particle (the reference's kernels under
// PRESCRIBED_CILIA use rpy_interaction<3,3> for all four blocks, and Mbs_mult
// adds to Mbb_mult's result; Msf_mult replaces the segment block for the
// weakly coupled filaments) minus the rigid-body and phase/angle couplings
// K and plus their transposes -K^T.
//
// Layout and kernels. The pair products run on the work-queue kernel
// (rpy_queue.cuh) as 3x3 jobs -- segments and blobs as "blob-like" 3-force
// records -- each into its own output, added in the reference's order by the
// combine kernel; the weakly coupled segment block runs on msf_kernel
// (weak.cu). Everything else is O(N) and works per filament (one warp: the
// segment rows of one filament, the phase/angle dot products, the Schur
// corrections) or per 32 blobs (one warp), with the swimmer-wide 6-vectors
// (K^T rows, the preconditioner's body block) summed by the last CTA to
// arrive, in warp order (deterministic). GMRES is right-preconditioned,
// warm started from the previous solution, orthogonalised by classical
// Gram-Schmidt applied twice (two reductions per step; the reference uses
// modified Gram-Schmidt, equal in exact arithmetic), with the reference's
// Givens sign convention and stopping test; its vectors and Hessenberg
// matrix live on the device. The step kernels read the step index from the
// device scalars and skip once the solve is finished, so the Arnoldi steps
// run in chunks replayed as a CUDA graph, the host polling one flag per
// chunk. FP64, as the reference's FIL_USE_DOUBLE_PRECISION build, or FP32C
// (inner solves on FP32 pair sums refined on float-float or FP64 residuals).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/tfs_gb300.h"
#include "tfs_kernels.h"
#include "tfs_solver.h"

namespace tfs {

namespace {

constexpr double kPiP = 3.14159265358979323846264338327950288;
constexpr int kPT = 128;         // threads per CTA of the O(N) kernels
constexpr int kPW = kPT / 32;    // warps per CTA
// threads per CTA of the GMRES vector kernels (one CTA per SM at the medium
// swimmer's sizes: eight warps to cover the L2 latency of their row loads)
constexpr int kGT = 256;
constexpr int kGW = kGT / 32;
constexpr int kFilC = 16;        // per-filament constants (below)
constexpr int kPresMaxIter = 350;  // MAX_LINEAR_SYSTEM_ITER (config.hpp:312)
constexpr int kPresChunk = 4;      // Arnoldi steps launched between polls of the done flag
// FP32C: the deepest relative reduction an inner solve is asked for. Its
// Krylov vectors are FP64 and only the pair sums are FP32 (compensated,
// ~1e-7 relative), so below this the correction's own error dominates.
constexpr double kPresInnerFloor = 1e-7;

// Per filament m (swimmer.cpp:1255-1287, mobility_solver.cpp:1060-1100):
// [0] c11 = K_phi.K_phi, [1] c22 = K_th.K_th, [2] c12 = K_phi.K_th,
// [3..5] v_phi = sum_k K_phi, [6..8] v_th, [9..11] u_phi = sum_k d_k x K_phi,
// [12..14] u_th; d_k = x_k - body x.
enum { FC11 = 0, FC22 = 1, FC12 = 2, FVPHI = 3, FVTH = 6, FUPHI = 9, FUTH = 12 };

struct PresScalars {
  double norm_rhs, beta0, qnorm, rel;
  double tol;  // stopping test of the running GMRES: |beta_k| <= tol norm_rhs
  int iter;    // the Arnoldi step being built (k, from 1)
  int flag;    // warm-start test: 1 accepted, 2 discarded, 3 zero right-hand side
  int done;    // 1: converged or out of steps
  int iters;   // Arnoldi steps taken
  int status;  // 0 ok, 1 non-finite residual, 2 singular body block
};

}  // namespace

// Device state of the prescribed-cilia solve (one per solver, made by
// tfs_prescribed_setup).
struct PresState {
  tfs_prescribed_config cfg{};
  int nfil = 0, nseg = 0, ns = 0, nb = 0, n = 0;
  int o_body = 0, o_phase = 0, o_angle = 0;
  bool free_body = false, phase = false, angle = false, weak = false;
  bool have_kin = false, have_x = false;
  int max_iter = kPresMaxIter;
  // kinematics
  double *kphi = nullptr, *kth = nullptr;          // 3 Ns
  double *phase_v = nullptr, *omega0 = nullptr, *angle_v = nullptr, *pdot = nullptr;  // nfil
  double *vbody = nullptr;                         // 6: prescribed body velocities
  double *tab_p = nullptr, *tab_a = nullptr;       // generalised-force tables
  int n_tab_p = 0, n_tab_a = 0;
  double *fil = nullptr;                           // kFilC nfil
  double *m6inv = nullptr;                         // 36, column-major
  double body_x[3] = {0, 0, 0};
  // vectors
  double *b = nullptr, *x = nullptr, *z = nullptr, *tmp = nullptr;  // n
  double *Q = nullptr, *H = nullptr, *beta = nullptr, *cs = nullptr, *sn = nullptr, *y = nullptr;
  double *h1 = nullptr, *h2 = nullptr;
  double *part = nullptr;                          // G x pstride
  double *part6 = nullptr;                         // 6 x warps of the O(N) kernels
  unsigned *cnt = nullptr;                         // last-CTA counters
  PresScalars *st = nullptr, *st_host = nullptr;
  int G = 1, rows = 1, pstride = 1;
  // products
  double *rec_s = nullptr, *rec_b = nullptr;       // FP64 3-force records
  double *f6 = nullptr, *v6 = nullptr;             // weakly coupled: 6-stride forces, velocities
  double *v_ss = nullptr, *v_sb = nullptr, *v_bb = nullptr, *v_bs = nullptr;
  double *qpart = nullptr;                         // job partial sums
  unsigned *qcnt = nullptr;                        // [2] launch counters, arrival counters
  QueueJob jobs[4];
  int n_jobs = 0;
  QueueJob *jobs_dev = nullptr;  // four slots; weakly coupled: the fourth holds hook_ss
  QueueJob hook_ss{};            // weakly coupled: the seg <- seg job of the block hook
  // FP32C: FP32 3-force records (origin-relative positions) and their jobs
  float *rec_s32 = nullptr, *rec_b32 = nullptr;
  QueueJob jobs32[4];
  QueueJob *jobs32_dev = nullptr;
  long long fallbacks = 0;  // FP32C refinements that stalled and finished in FP64
  // FP32C residuals in float-float arithmetic (rpy_ff.cu) when every
  // particle has the same radius and no block is the weakly coupled one: the
  // translational mobility of all particles is then one equal-radius
  // product over the concatenated positions (segments, then blobs)
  bool use_ff = false;
  double *x_all = nullptr, *v_all = nullptr;  // 3 (Ns + Nb)
  void *rec_ff = nullptr;
  double *body_dev = nullptr;  // [3] body position of the kinematics set last
  // Arnoldi steps run in chunks of kPresChunk, device-driven: the step
  // kernels read the step from the scalars and skip once finished, and the
  // products' jobs skip through *skip = st->done (jobs_it, jobs32_it); each
  // chunk replays a CUDA graph captured once per precision
  QueueJob *jobs_it_dev = nullptr, *jobs32_it_dev = nullptr;
  cudaGraphExec_t graph[2] = {nullptr, nullptr};
  long long graph_kernels[2] = {0, 0};
  int graph_variant[2] = {-1, -1};
  bool graphs_ok = true;
};

namespace {

// ---------------------------------------------------------------------------
// device helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ double pw_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Sum over c < n of p[c * stride] by one warp: lane l adds the terms c = l,
// l + 32, l + 64, ... in that order, then a fixed shuffle tree, so every lane
// gets the same bits. The terms are loaded eight per lane at a time: one L2
// round trip covers 256 of them.
__device__ __forceinline__ double pw_sum_strided(const double *p, int n, size_t stride) {
  const int lane = threadIdx.x & 31;
  double t = 0.0;
  for (int c0 = 0; c0 < n; c0 += 256) {
    double v[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int c = c0 + lane + 32 * j;
      v[j] = c < n ? __ldcg(p + (size_t)c * stride) : 0.0;
    }
#pragma unroll
    for (int j = 0; j < 8; ++j)
      if (c0 + lane + 32 * j < n) t += v[j];
  }
  return pw_sum(t);
}

// Warp sums of eight values a lane by a reduce-scatter butterfly: at each of
// the first three levels a lane keeps half of its columns and adds its
// partner's half of them, then two plain levels; 9 FP64 adds a lane instead
// of the 40 of eight shuffle trees (the FP64 pipe bounds these kernels on
// this part). Lanes 4c .. 4c+3 return the same bits: column c's sum.
__device__ __forceinline__ double pw_sum8(const double v[8]) {
  const int lane = threadIdx.x & 31;
  const bool b4 = lane & 16, b3 = lane & 8, b2 = lane & 4;
  double w[4], x[2];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const double keep = b4 ? v[4 + j] : v[j], send = b4 ? v[j] : v[4 + j];
    w[j] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
  }
#pragma unroll
  for (int j = 0; j < 2; ++j) {
    const double keep = b3 ? w[2 + j] : w[j], send = b3 ? w[j] : w[2 + j];
    x[j] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
  }
  double y = (b2 ? x[1] : x[0]) + __shfl_xor_sync(0xffffffffu, b2 ? x[0] : x[1], 4);
  y += __shfl_xor_sync(0xffffffffu, y, 2);
  y += __shfl_xor_sync(0xffffffffu, y, 1);
  return y;
}

// The same for four values a lane (6 adds instead of 20): lanes 8c .. 8c+7
// return column c's sum.
__device__ __forceinline__ double pw_sum4(const double v[4]) {
  const int lane = threadIdx.x & 31;
  const bool b4 = lane & 16, b3 = lane & 8;
  double w[2];
#pragma unroll
  for (int j = 0; j < 2; ++j) {
    const double keep = b4 ? v[2 + j] : v[j], send = b4 ? v[j] : v[2 + j];
    w[j] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
  }
  double y = (b3 ? w[1] : w[0]) + __shfl_xor_sync(0xffffffffu, b3 ? w[0] : w[1], 8);
  y += __shfl_xor_sync(0xffffffffu, y, 4);
  y += __shfl_xor_sync(0xffffffffu, y, 2);
  y += __shfl_xor_sync(0xffffffffu, y, 1);
  return y;
}

// Four adjacent columns at once: the sum over c < n of p[c * stride + j] for
// j < m (m <= 4), lane l adding the terms c = l, l + 32, ... in that order,
// then pw_sum4 (lanes 8j .. 8j+7 return column j's sum), with the loads of
// all four columns for 128 terms in flight together.
__device__ __forceinline__ double pw_sum_strided4(const double *p, int n, size_t stride, int m) {
  const int lane = threadIdx.x & 31;
  double t[4] = {0.0, 0.0, 0.0, 0.0};
  for (int c0 = 0; c0 < n; c0 += 128) {
    double v[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      const int c = c0 + lane + 32 * a;
#pragma unroll
      for (int j = 0; j < 4; ++j)
        v[a][j] = (c < n && j < m) ? __ldcg(p + (size_t)c * stride + j) : 0.0;
    }
#pragma unroll
    for (int a = 0; a < 4; ++a)
      if (c0 + lane + 32 * a < n)
#pragma unroll
        for (int j = 0; j < 4; ++j) t[j] += v[a][j];
  }
  return pw_sum4(t);
}

// True in exactly one CTA, the last to arrive after writing its partials
// (which then must reset the counter).
__device__ bool pres_last_cta(unsigned *counter) {
  __shared__ bool last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(counter, 1u) == gridDim.x - 1;
  __syncthreads();
  if (last) __threadfence();
  return last;
}

__device__ __forceinline__ void cross3(const double *a, const double *b, double *o) {
  o[0] = a[1] * b[2] - a[2] * b[1];
  o[1] = a[2] * b[0] - a[0] * b[2];
  o[2] = a[0] * b[1] - a[1] * b[0];
}

// cyclic_cubic_spline_interpolation (mobility_solver.cpp:240-279).
__device__ double pres_spline(double phase, const double *in, int n) {
  double p = 0.5 * phase / kPiP;
  p -= floor(p);
  p *= n;
  if (!(p >= 0.0 && p <= (double)n)) return nan("");  // non-finite phase: no table read
  const int lo = (int)p;
  if (lo == n) return in[0];
  const int hi = lo == n - 1 ? 0 : lo + 1;
  const double ql = in[lo], qu = in[hi];
  const double dql = lo == 0 ? in[1] - in[0] : 0.5 * (in[hi] - in[lo - 1]);
  const double dqu = hi == 0 ? in[0] - in[n - 1] : 0.5 * (in[hi == n - 1 ? 0 : hi + 1] - in[lo]);
  const double t = p - lo, t2 = t * t, t3 = t2 * t;
  return ql * (2.0 * t3 - 3.0 * t2 + 1.0) + dql * (t3 - 2.0 * t2 + t) + qu * (3.0 * t2 - 2.0 * t3) +
         dqu * (t3 - t2);
}

// Arguments of the O(N) kernels.
struct PA {
  int ns, nb, nfil, nseg, n, o_body, o_phase, o_angle;
  int free_body, phase, angle, weak;
  double c, cb;
  const double *body;  // device [3]: the body position
  const double *x_segs, *d_blobs, *kphi, *kth, *fil, *m6inv;
  double *part6;
  unsigned *cnt;
  int fil_warps, blob_warps;  // warps [0, fil_warps) per filament, then per 32 blobs
};

__device__ __forceinline__ int pa_warp() {
  return (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
}

__device__ __forceinline__ void seg_d(const PA &a, int i, double *d) {
  d[0] = a.x_segs[3 * (size_t)i] - a.body[0];
  d[1] = a.x_segs[3 * (size_t)i + 1] - a.body[1];
  d[2] = a.x_segs[3 * (size_t)i + 2] - a.body[2];
}

// Sum of the warps' partial 6-vectors (warp order), by the last CTA: result
// in sh[0..6).
__device__ void sum_part6_warps(const PA &a, double *sh) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int W = a.fil_warps + a.blob_warps;
  for (int k = wid; k < 6; k += kPW) {
    const double t = pw_sum_strided(a.part6 + k, W, 6);
    if (lane == 0) sh[k] = t;
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
// kinematics: per-filament constants and the free body's 6x6 block
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kPT) pres_fil_kernel(PA a, double *fil) {
  const int m = pa_warp(), lane = threadIdx.x & 31;
  if (m >= a.nfil) return;
  double v[15];
#pragma unroll
  for (int q = 0; q < 15; ++q) v[q] = 0.0;
  for (int k = lane; k < a.nseg; k += 32) {
    const int i = m * a.nseg + k;
    double d[3], kp[3], kt[3], u[3];
    seg_d(a, i, d);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      kp[c] = a.kphi[3 * (size_t)i + c];
      kt[c] = a.angle ? a.kth[3 * (size_t)i + c] : 0.0;
    }
    v[FC11] += kp[0] * kp[0] + kp[1] * kp[1] + kp[2] * kp[2];
    v[FC22] += kt[0] * kt[0] + kt[1] * kt[1] + kt[2] * kt[2];
    v[FC12] += kp[0] * kt[0] + kp[1] * kt[1] + kp[2] * kt[2];
    cross3(d, kp, u);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      v[FVPHI + c] += kp[c];
      v[FVTH + c] += kt[c];
      v[FUPHI + c] += u[c];
    }
    cross3(d, kt, u);
#pragma unroll
    for (int c = 0; c < 3; ++c) v[FUTH + c] += u[c];
  }
#pragma unroll
  for (int q = 0; q < 15; ++q) v[q] = pw_sum(v[q]);
  if (lane < 15) {
    double t = v[0];
#pragma unroll
    for (int q = 1; q < 15; ++q)
      if (lane == q) t = v[q];
    fil[(size_t)kFilC * m + lane] = t;
  }
}

// M (row r, column c) of the free body's preconditioner block
// (swimmer.cpp:1154-1322), then its inverse: one CTA. st->status = 2 if M is
// singular.
__global__ void __launch_bounds__(256) pres_m6_kernel(PA a, double *m6inv, PresScalars *st) {
  // per thread: S1 = sum f rcross(d) (9), S2 = sum f rcross(d)^2 (9),
  // C11, C21, C22 (27) of the phase/angle Schur terms
  double acc[45];
#pragma unroll
  for (int q = 0; q < 45; ++q) acc[q] = 0.0;
  for (int p = threadIdx.x; p < a.ns + a.nb; p += blockDim.x) {
    double d[3];
    double f;
    if (p < a.ns) {
      seg_d(a, p, d);
      f = a.c;
    } else {
      const double *db = a.d_blobs + 3 * (size_t)(p - a.ns);
      d[0] = db[0]; d[1] = db[1]; d[2] = db[2];
      f = a.cb;
    }
    // rcross(d) (matrix.cpp:665-679): rows {0, d2, -d1}, {-d2, 0, d0}, {d1, -d0, 0}
    const double R[9] = {0.0, d[2], -d[1], -d[2], 0.0, d[0], d[1], -d[0], 0.0};
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        acc[3 * r + c] += f * R[3 * r + c];
        double s = 0.0;
#pragma unroll
        for (int k = 0; k < 3; ++k) s += R[3 * r + k] * R[3 * k + c];
        acc[9 + 3 * r + c] += f * s;
      }
  }
  if (a.phase) {
    for (int m = threadIdx.x; m < a.nfil; m += blockDim.x) {
      const double *F = a.fil + (size_t)kFilC * m;
      const double *vp = F + FVPHI, *vt = F + FVTH, *up = F + FUPHI, *ut = F + FUTH;
      double i11, i22, i12;
      if (a.angle) {
        const double det = F[FC11] * F[FC22] - F[FC12] * F[FC12];
        i11 = F[FC22] / det;
        i22 = F[FC11] / det;
        i12 = -F[FC12] / det;
      } else {
        i11 = 1.0 / F[FC11];
        i22 = i12 = 0.0;
      }
#pragma unroll
      for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          acc[18 + 3 * r + c] += vp[r] * vp[c] * i11 + vp[r] * vt[c] * i12 + vt[r] * vp[c] * i12 +
                                 vt[r] * vt[c] * i22;
          acc[27 + 3 * r + c] += up[r] * vp[c] * i11 + up[r] * vt[c] * i12 + ut[r] * vp[c] * i12 +
                                 ut[r] * vt[c] * i22;
          acc[36 + 3 * r + c] += up[r] * up[c] * i11 + up[r] * ut[c] * i12 + ut[r] * up[c] * i12 +
                                 ut[r] * ut[c] * i22;
        }
    }
  }
  __shared__ double red[8][45];
  __shared__ double M[6][12];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < 45; ++q) {
    const double t = pw_sum(acc[q]);
    if (lane == 0) red[wid][q] = t;
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  double S[45];
  for (int q = 0; q < 45; ++q) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w][q];
    S[q] = t;
  }
  const double eye = (double)a.ns * a.c + (double)a.nb * a.cb;
  for (int r = 0; r < 6; ++r)
    for (int c = 0; c < 12; ++c) M[r][c] = (c - 6 == r) ? 1.0 : 0.0;
  for (int r = 0; r < 3; ++r) {
    M[r][r] = eye;
    for (int c = 0; c < 3; ++c) {
      M[r][3 + c] = S[3 * r + c];         // sum f rcross(d)
      M[3 + r][3 + c] = -S[9 + 3 * r + c];  // - sum f rcross(d)^2
      M[3 + r][c] = -S[3 * r + c];        // the lower-left block is minus the upper-right
    }
  }
  if (a.phase) {
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) {
        M[r][c] -= a.c * S[18 + 3 * r + c];
        M[3 + r][c] -= a.c * S[27 + 3 * r + c];
        M[r][3 + c] -= a.c * S[27 + 3 * c + r];  // C12 = C21^T
        M[3 + r][3 + c] -= a.c * S[36 + 3 * r + c];
      }
  }
  // Gauss-Jordan with partial pivoting on [M | I]
  for (int k = 0; k < 6; ++k) {
    int p = k;
    for (int r = k + 1; r < 6; ++r)
      if (fabs(M[r][k]) > fabs(M[p][k])) p = r;
    if (!(fabs(M[p][k]) > 0.0)) {
      st->status = 2;
      return;
    }
    if (p != k)
      for (int c = 0; c < 12; ++c) {
        const double t = M[k][c];
        M[k][c] = M[p][c];
        M[p][c] = t;
      }
    const double inv = 1.0 / M[k][k];
    for (int c = 0; c < 12; ++c) M[k][c] *= inv;
    for (int r = 0; r < 6; ++r) {
      if (r == k) continue;
      const double f = M[r][k];
      if (f != 0.0)
        for (int c = 0; c < 12; ++c) M[r][c] -= f * M[k][c];
    }
  }
  for (int r = 0; r < 6; ++r)
    for (int c = 0; c < 6; ++c) m6inv[r + 6 * c] = M[r][6 + c];
}

// ---------------------------------------------------------------------------
// right-hand side (mobility_solver.cpp:282-437)
// ---------------------------------------------------------------------------
struct RhsArgs {
  const double *tab_p, *tab_a;
  int n_tab_p, n_tab_a;
  const double *phase, *omega0, *angle, *pdot, *vbody;
  double gff, tsf, fil_length;
};

__global__ void __launch_bounds__(kPT) pres_rhs_kernel(PA a, RhsArgs r, double *b) {
  const int w = pa_warp(), lane = threadIdx.x & 31;
  const bool prescribed_body = !a.free_body;
  double V[6] = {0, 0, 0, 0, 0, 0};
  if (prescribed_body && r.vbody != nullptr)
    for (int k = 0; k < 6; ++k) V[k] = r.vbody[k];
  if (w < a.fil_warps) {
    const int m = w;
    const double pdm = a.phase ? 0.0 : r.pdot[m];
    for (int k = lane; k < a.nseg; k += 32) {
      const int i = m * a.nseg + k;
      double o[3] = {0, 0, 0}, d[3], wd[3];
      if (!a.phase)
        for (int c = 0; c < 3; ++c) o[c] = pdm * a.kphi[3 * (size_t)i + c];
      if (prescribed_body) {
        seg_d(a, i, d);
        cross3(V + 3, d, wd);
        for (int c = 0; c < 3; ++c) o[c] += V[c] + wd[c];
      }
      for (int c = 0; c < 3; ++c) b[3 * (size_t)i + c] = o[c];
    }
    if (lane == 0) {
      if (a.angle) {
        double qa = pres_spline(r.phase[m], r.tab_a, r.n_tab_a) * 0.5 * r.omega0[m] / kPiP;
        const double kscale = r.omega0[m] * r.fil_length * r.fil_length * r.fil_length;
        qa -= r.tsf * kscale * r.angle[m];
        b[a.o_angle + m] = -qa;
      }
      if (a.phase) {
        double qp = pres_spline(r.phase[m], r.tab_p, r.n_tab_p) * 0.5 * r.omega0[m] / kPiP;
        qp *= r.gff;
        b[a.o_phase + m] = -qp;
      }
    }
  } else if (w < a.fil_warps + a.blob_warps) {
    const int j = 32 * (w - a.fil_warps) + lane;
    if (j < a.nb) {
      double o[3] = {0, 0, 0}, wd[3];
      if (prescribed_body) {
        cross3(V + 3, a.d_blobs + 3 * (size_t)j, wd);
        for (int c = 0; c < 3; ++c) o[c] = V[c] + wd[c];
      }
      for (int c = 0; c < 3; ++c) b[3 * ((size_t)a.ns + j) + c] = o[c];
    }
  }
  if (a.free_body && blockIdx.x == 0 && threadIdx.x < 6) b[a.o_body + threadIdx.x] = 0.0;
}

// ---------------------------------------------------------------------------
// operator (system_matrix_mult_new, mobility_solver.cpp:1806-2026)
// ---------------------------------------------------------------------------

// FP64 3-force records {x, y, z, f0, f1, f2} of every segment and blob with
// the forces of z; the 6-stride segment forces of the weakly coupled product.
__global__ void pres_pack_kernel(PA a, const double *z, const double *x_blobs, double *rec_s,
                                 double *rec_b, double *f6, const PresScalars *it) {
  if (it != nullptr && it->done) return;
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < a.ns) {
    double *r = rec_s + 6 * (size_t)p;
    for (int c = 0; c < 3; ++c) {
      r[c] = a.x_segs[3 * (size_t)p + c];
      r[3 + c] = z[3 * (size_t)p + c];
    }
    if (f6 != nullptr)
      for (int c = 0; c < 3; ++c) {
        f6[6 * (size_t)p + c] = z[3 * (size_t)p + c];
        f6[6 * (size_t)p + 3 + c] = 0.0;
      }
  } else if (p < a.ns + a.nb) {
    const int j = p - a.ns;
    double *r = rec_b + 6 * (size_t)j;
    for (int c = 0; c < 3; ++c) {
      r[c] = x_blobs[3 * (size_t)j + c];
      r[3 + c] = z[3 * ((size_t)a.ns + j) + c];
    }
  }
}

// FP32 3-force records {x - o, y - o, z - o, f0, f1, f2, 0, 0}: the
// positions relative to the solver's origin, as the FP32 work-queue kernel
// reads them.
__global__ void pres_pack32_kernel(PA a, const double *z, const double *x_blobs,
                                   const double *origin, float *rec_s, float *rec_b,
                                   const PresScalars *it) {
  if (it != nullptr && it->done) return;
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  const double *x;
  float *r;
  const double *f;
  if (p < a.ns) {
    x = a.x_segs + 3 * (size_t)p;
    f = z + 3 * (size_t)p;
    r = rec_s + 8 * (size_t)p;
  } else if (p < a.ns + a.nb) {
    const int j = p - a.ns;
    x = x_blobs + 3 * (size_t)j;
    f = z + 3 * ((size_t)a.ns + j);
    r = rec_b + 8 * (size_t)j;
  } else {
    return;
  }
  for (int c = 0; c < 3; ++c) {
    r[c] = float(x[c] - origin[c]);
    r[3 + c] = float(f[c]);
  }
  r[6] = 0.f;
  r[7] = 0.f;
}

// out = A z from the products: segments v_ss (or the 6-stride v6 of the
// weakly coupled product) + v_sb, blobs v_bb + v_bs, minus K [U; Omega;
// phase rates; angle rates]; phase and angle rows -K^T; body rows -K^T (the
// last CTA). resid != nullptr: out = resid - A z instead. it != nullptr (an
// Arnoldi step): out is column it->iter of out, and a finished solve skips.
__global__ void __launch_bounds__(kPT) pres_combine_kernel(PA a, const double *z, const double *v_ss,
                                                           const double *v6, const double *v_sb,
                                                           const double *v_bb, const double *v_bs,
                                                           const double *resid, double *out,
                                                           const PresScalars *it) {
  __shared__ double sh[8];
  if (it != nullptr) {
    if (it->done) return;
    out += (size_t)it->iter * a.n;
  }
  const int w = pa_warp(), lane = threadIdx.x & 31;
  double U[6] = {0, 0, 0, 0, 0, 0};
  if (a.free_body)
    for (int k = 0; k < 6; ++k) U[k] = z[a.o_body + k];
  double p6[6] = {0, 0, 0, 0, 0, 0};
  if (w < a.fil_warps) {
    const int m = w;
    const double pd = a.phase ? z[a.o_phase + m] : 0.0;
    const double ad = a.angle ? z[a.o_angle + m] : 0.0;
    double dp = 0.0, da = 0.0;
    for (int k = lane; k < a.nseg; k += 32) {
      const int i = m * a.nseg + k;
      double f[3], d[3], o[3], t[3];
      for (int c = 0; c < 3; ++c) {
        f[c] = z[3 * (size_t)i + c];
        const double vs = a.weak ? v6[6 * (size_t)i + c] : v_ss[3 * (size_t)i + c];
        o[c] = 0.0;
        if (a.free_body) o[c] -= U[c];
        if (a.phase) o[c] -= pd * a.kphi[3 * (size_t)i + c];
        if (a.angle) o[c] -= ad * a.kth[3 * (size_t)i + c];
        o[c] += vs + (v_sb != nullptr ? v_sb[3 * (size_t)i + c] : 0.0);
        if (a.phase) dp += a.kphi[3 * (size_t)i + c] * f[c];
        if (a.angle) da += a.kth[3 * (size_t)i + c] * f[c];
      }
      if (a.free_body) {
        seg_d(a, i, d);
        cross3(U + 3, d, t);
        for (int c = 0; c < 3; ++c) o[c] -= t[c];
        cross3(d, f, t);
        for (int c = 0; c < 3; ++c) {
          p6[c] += f[c];
          p6[3 + c] += t[c];
        }
      }
      for (int c = 0; c < 3; ++c) {
        const size_t row = 3 * (size_t)i + c;
        out[row] = resid != nullptr ? resid[row] - o[c] : o[c];
      }
    }
    dp = pw_sum(dp);
    da = pw_sum(da);
    if (lane == 0) {
      if (a.phase) out[a.o_phase + m] = resid != nullptr ? resid[a.o_phase + m] + dp : -dp;
      if (a.angle) out[a.o_angle + m] = resid != nullptr ? resid[a.o_angle + m] + da : -da;
    }
  } else if (w < a.fil_warps + a.blob_warps) {
    const int j = 32 * (w - a.fil_warps) + lane;
    if (j < a.nb) {
      const double *d = a.d_blobs + 3 * (size_t)j;
      double f[3], o[3], t[3];
      for (int c = 0; c < 3; ++c) {
        f[c] = z[3 * ((size_t)a.ns + j) + c];
        o[c] = a.free_body ? -U[c] : 0.0;
      }
      if (a.free_body) {
        cross3(U + 3, d, t);
        for (int c = 0; c < 3; ++c) o[c] -= t[c];
        cross3(d, f, t);
        for (int c = 0; c < 3; ++c) {
          p6[c] += f[c];
          p6[3 + c] += t[c];
        }
      }
      for (int c = 0; c < 3; ++c) {
        const size_t row = 3 * ((size_t)a.ns + j) + c;
        o[c] += v_bb[3 * (size_t)j + c] + (v_bs != nullptr ? v_bs[3 * (size_t)j + c] : 0.0);
        out[row] = resid != nullptr ? resid[row] - o[c] : o[c];
      }
    }
  }
  if (!a.free_body) return;
  const int W = a.fil_warps + a.blob_warps;
  for (int k = 0; k < 6; ++k) p6[k] = pw_sum(p6[k]);
  if (lane == 0 && w < W)
    for (int k = 0; k < 6; ++k) a.part6[6 * (size_t)w + k] = p6[k];
  if (!pres_last_cta(a.cnt)) return;
  sum_part6_warps(a, sh);
  if (threadIdx.x < 6) {
    const int row = a.o_body + threadIdx.x;
    out[row] = resid != nullptr ? resid[row] + sh[threadIdx.x] : -sh[threadIdx.x];
  }
  if (threadIdx.x == 0) *a.cnt = 0u;
}

// ---------------------------------------------------------------------------
// preconditioner (apply_preconditioner_new, mobility_solver.cpp:1040-1436)
// ---------------------------------------------------------------------------

// 2x2 inverse of [[c11, c12], [c12, c22]] of filament F: i11, i22, i12.
__device__ __forceinline__ void pres_cinv(const double *F, double &i11, double &i22, double &i12) {
  const double det = F[FC11] * F[FC22] - F[FC12] * F[FC12];
  i11 = F[FC22] / det;
  i22 = F[FC11] / det;
  i12 = -F[FC12] / det;
}

// Pass A. Segments s = c in, blobs cb in. Prescribed body: the per-filament
// phase/angle rows and their K corrections finish here. Free body: the
// phase/angle rows after their 2x2 solve are stored, the body block's
// right-hand side t = -in_body - sum (s; d x s) - sum (p v + a v'; p u + a u')
// is summed over the warps, and the last CTA writes B = M^-1 t.
__global__ void __launch_bounds__(kPT) pres_precond_a_kernel(PA a, const double *in, double *out,
                                                             const PresScalars *it) {
  __shared__ double sh[8];
  if (it != nullptr) {  // an Arnoldi step: in is column it->iter - 1 of in
    if (it->done) return;
    in += (size_t)(it->iter - 1) * a.n;
  }
  const int w = pa_warp(), lane = threadIdx.x & 31;
  double p6[6] = {0, 0, 0, 0, 0, 0};
  if (w < a.fil_warps) {
    const int m = w;
    const double *F = a.fil + (size_t)kFilC * m;
    double dp = 0.0, da = 0.0;
    for (int k = lane; k < a.nseg; k += 32) {
      const int i = m * a.nseg + k;
      double s[3], d[3], t[3];
      for (int c = 0; c < 3; ++c) {
        s[c] = a.c * in[3 * (size_t)i + c];
        dp += a.kphi[3 * (size_t)i + c] * s[c];
        if (a.angle) da += a.kth[3 * (size_t)i + c] * s[c];
      }
      if (a.free_body) {
        seg_d(a, i, d);
        cross3(d, s, t);
        for (int c = 0; c < 3; ++c) {
          p6[c] += s[c];
          p6[3 + c] += t[c];
        }
      }
      for (int c = 0; c < 3; ++c) out[3 * (size_t)i + c] = s[c];
    }
    dp = pw_sum(dp);
    da = pw_sum(da);
    double pm = 0.0, am = 0.0;  // the filament's phase and angle rows
    if (a.phase && a.angle) {
      double i11, i22, i12;
      pres_cinv(F, i11, i22, i12);
      const double p0 = -in[a.o_phase + m] - dp, a0 = -in[a.o_angle + m] - da;
      pm = p0 * i11 + a0 * i12;
      am = p0 * i12 + a0 * i22;
      if (!a.free_body) {
        pm /= a.c;
        am /= a.c;
      }
    } else if (a.phase) {  // prescribed body only (validated on the host)
      pm = (-in[a.o_phase + m] - dp) / (F[FC11] * a.c);
    } else if (a.angle) {
      am = (-in[a.o_angle + m] - da) / (F[FC22] * a.c);
    }
    if (!a.free_body && (a.phase || a.angle)) {
      for (int k = lane; k < a.nseg; k += 32) {
        const int i = m * a.nseg + k;
        for (int c = 0; c < 3; ++c) {
          double v = out[3 * (size_t)i + c];
          if (a.phase) v += a.c * pm * a.kphi[3 * (size_t)i + c];
          if (a.angle) v += a.c * am * a.kth[3 * (size_t)i + c];
          out[3 * (size_t)i + c] = v;
        }
      }
    }
    if (lane == 0) {
      if (a.phase) out[a.o_phase + m] = pm;
      if (a.angle) out[a.o_angle + m] = am;
    }
    if (a.free_body && a.phase) {
      for (int c = 0; c < 3; ++c) {
        p6[c] += lane == 0 ? pm * F[FVPHI + c] + am * F[FVTH + c] : 0.0;
        p6[3 + c] += lane == 0 ? pm * F[FUPHI + c] + am * F[FUTH + c] : 0.0;
      }
    }
  } else if (w < a.fil_warps + a.blob_warps) {
    const int j = 32 * (w - a.fil_warps) + lane;
    if (j < a.nb) {
      const double *d = a.d_blobs + 3 * (size_t)j;
      double s[3], t[3];
      for (int c = 0; c < 3; ++c) s[c] = a.cb * in[3 * ((size_t)a.ns + j) + c];
      if (a.free_body) {
        cross3(d, s, t);
        for (int c = 0; c < 3; ++c) {
          p6[c] += s[c];
          p6[3 + c] += t[c];
        }
      }
      for (int c = 0; c < 3; ++c) out[3 * ((size_t)a.ns + j) + c] = s[c];
    }
  }
  if (!a.free_body) return;
  const int W = a.fil_warps + a.blob_warps;
  for (int k = 0; k < 6; ++k) p6[k] = pw_sum(p6[k]);
  if (lane == 0 && w < W)
    for (int k = 0; k < 6; ++k) a.part6[6 * (size_t)w + k] = p6[k];
  if (!pres_last_cta(a.cnt)) return;
  sum_part6_warps(a, sh);
  if (threadIdx.x == 0) {
    double t[6], B[6];
    for (int k = 0; k < 6; ++k) t[k] = -in[a.o_body + k] - sh[k];
    for (int r = 0; r < 6; ++r) {
      double v = 0.0;
      for (int k = 0; k < 6; ++k) v += a.m6inv[r + 6 * k] * t[k];
      B[r] = v;
    }
    for (int k = 0; k < 6; ++k) out[a.o_body + k] = B[k];
    *a.cnt = 0u;
  }
}

// Pass B (free body): the phase/angle rows' correction by the body block B
// and s += c (B0 + B1 x d + p K_phi + a K_th), blobs += cb (B0 + B1 x d).
__global__ void __launch_bounds__(kPT) pres_precond_b_kernel(PA a, double *out,
                                                             const PresScalars *it) {
  if (it != nullptr && it->done) return;
  const int w = pa_warp(), lane = threadIdx.x & 31;
  double B[6];
  for (int k = 0; k < 6; ++k) B[k] = out[a.o_body + k];
  if (w < a.fil_warps) {
    const int m = w;
    const double *F = a.fil + (size_t)kFilC * m;
    double pm = 0.0, am = 0.0;
    if (a.phase) {
      double i11, i22, i12;
      pres_cinv(F, i11, i22, i12);
      const double vpB = F[FVPHI] * B[0] + F[FVPHI + 1] * B[1] + F[FVPHI + 2] * B[2];
      const double vtB = F[FVTH] * B[0] + F[FVTH + 1] * B[1] + F[FVTH + 2] * B[2];
      const double upB = F[FUPHI] * B[3] + F[FUPHI + 1] * B[4] + F[FUPHI + 2] * B[5];
      const double utB = F[FUTH] * B[3] + F[FUTH + 1] * B[4] + F[FUTH + 2] * B[5];
      pm = out[a.o_phase + m] / a.c - (i11 * vpB + i12 * vtB + i11 * upB + i12 * utB);
      am = out[a.o_angle + m] / a.c - (i12 * vpB + i22 * vtB + i12 * upB + i22 * utB);
    }
    __syncwarp();
    for (int k = lane; k < a.nseg; k += 32) {
      const int i = m * a.nseg + k;
      double d[3], t[3];
      seg_d(a, i, d);
      cross3(B + 3, d, t);
      for (int c = 0; c < 3; ++c) {
        double v = out[3 * (size_t)i + c] + a.c * (B[c] + t[c]);
        if (a.phase) {
          v += a.c * pm * a.kphi[3 * (size_t)i + c];
          v += a.c * am * a.kth[3 * (size_t)i + c];
        }
        out[3 * (size_t)i + c] = v;
      }
    }
    __syncwarp();
    if (lane == 0 && a.phase) {
      out[a.o_phase + m] = pm;
      out[a.o_angle + m] = am;
    }
  } else if (w < a.fil_warps + a.blob_warps) {
    const int j = 32 * (w - a.fil_warps) + lane;
    if (j < a.nb) {
      double t[3];
      cross3(B + 3, a.d_blobs + 3 * (size_t)j, t);
      for (int c = 0; c < 3; ++c) out[3 * ((size_t)a.ns + j) + c] += a.cb * (B[c] + t[c]);
    }
  }
}

// ---------------------------------------------------------------------------
// The four block hooks in the prescribed-cilia form of the reference's
// kernels (cuda_functions.cu:362-757 under PRESCRIBED_CILIA): forces only
// (the torque slots of f_segs are not read), rpy_interaction<3,3>, zero
// rotational segment velocities, Mbs_mult adding to Mbb_mult's result.
// ---------------------------------------------------------------------------
// Records of the solver's own force arrays: segments from f_segs (6 per
// segment, the first three), blobs from f_blobs.
__global__ void pres_hook_pack_kernel(PA a, const double *f_segs, const double *f_blobs,
                                      const double *x_blobs, double *rec_s, double *rec_b) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < a.ns) {
    double *r = rec_s + 6 * (size_t)p;
    for (int c = 0; c < 3; ++c) {
      r[c] = a.x_segs[3 * (size_t)p + c];
      r[3 + c] = f_segs[6 * (size_t)p + c];
    }
  } else if (p < a.ns + a.nb) {
    const int j = p - a.ns;
    double *r = rec_b + 6 * (size_t)j;
    for (int c = 0; c < 3; ++c) {
      r[c] = x_blobs[3 * (size_t)j + c];
      r[3 + c] = f_blobs[3 * (size_t)j + c];
    }
  }
}

// out (stride `stride`) = or += v (3 per target); stride 6 zeroes the
// rotational slots on assignment.
__global__ void pres_hook_out_kernel(const double *v, double *out, int n, int stride, int add) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int c = 0; c < 3; ++c) {
    const double t = v[3 * (size_t)i + c];
    double *o = out + (size_t)stride * i + c;
    *o = add ? *o + t : t;
  }
  if (stride == 6 && !add)
    for (int c = 3; c < 6; ++c) out[6 * (size_t)i + c] = 0.0;
}

// ---------------------------------------------------------------------------
// GMRES over flat vectors of n rows: G CTAs, `rows` consecutive rows each
// ---------------------------------------------------------------------------
struct GA {
  int n, G, rows, ld, pstride, max_iter;
  double *Q, *H, *beta, *cs, *sn, *y, *h1, *h2, *part;
  unsigned *cnt;
  PresScalars *st;
};

// ||v|| into *out (the last CTA), v of n rows.
__global__ void __launch_bounds__(kGT) pres_norm_kernel(GA g, const double *v, double *out) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int r0 = blockIdx.x * g.rows, r1 = min(g.n, r0 + g.rows);
  double t = 0.0;
  for (int r = r0 + threadIdx.x; r < r1; r += blockDim.x) t += v[r] * v[r];
  __shared__ double red[kGW];
  t = pw_sum(t);
  if (lane == 0) red[wid] = t;
  __syncthreads();
  if (threadIdx.x == 0) {
    double u = 0.0;
    for (int w = 0; w < kGW; ++w) u += red[w];
    g.part[(size_t)blockIdx.x * g.pstride] = u;
  }
  if (!pres_last_cta(g.cnt)) return;
  if (wid == 0) {
    const double s = pw_sum_strided(g.part, g.G, g.pstride);
    if (lane == 0) {
      *out = sqrt(s);
      *g.cnt = 0u;
    }
  }
}

// The warm-start tests of solve_linear_system (mobility_solver.cpp:2121-2320)
// on beta0 = ||rhs - A x0|| and ||rhs||: flag 3 zero right-hand side, 1 the
// warm start already solves the system, 2 discard it (beta0 > ||rhs||).
__global__ void pres_start_kernel(GA g, double tol) {
  PresScalars *st = g.st;
  const double nr = st->norm_rhs, b0 = st->beta0;
  st->tol = tol;
  st->iter = 1;
  int flag = 0;
  if (nr == 0.0) flag = 3;
  else if (fabs(b0) <= tol * nr) flag = 1;
  else if (fabs(b0) > nr) flag = 2;
  st->flag = flag;
  st->done = (flag == 1 || flag == 3) ? 1 : 0;
  st->iters = 0;
  st->status = (flag != 3 && !(b0 == b0 && fabs(b0) < INFINITY)) ? 1 : 0;
  st->rel = nr > 0.0 ? b0 / nr : 0.0;
  g.beta[0] = flag == 2 ? nr : b0;
}

// Q_0 = r0 / beta0 (flag 0) or rhs / ||rhs|| with x = 0 (flag 2); x = 0 for
// a zero right-hand side (flag 3).
__global__ void pres_q0_kernel(GA g, const double *rhs, double *x) {
  const PresScalars *st = g.st;
  const int flag = st->flag;
  const double beta0 = g.beta[0];
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < g.n; r += gridDim.x * blockDim.x) {
    if (flag == 3) {
      x[r] = 0.0;
    } else if (flag == 2) {
      x[r] = 0.0;
      g.Q[r] = rhs[r] / beta0;
    } else if (flag == 0) {
      g.Q[r] /= beta0;
    }
  }
}

// Dots <w, Q_i>, i < k, over this CTA's rows into part[cta][i]: columns in
// blocks of 8, every thread accumulating its rows' products for the 8 at once
// (coalesced row loads; two rows a thread at a time, sixteen loads in
// flight, each row's products added in row order), block sums per column;
// the last CTA sums the partials in a fixed order into h, four columns a warp
// at a time.
__device__ void pres_dots(const GA &g, const double *w, int k, double *h) {
  __shared__ double red[kGW][8];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int r0 = blockIdx.x * g.rows, r1 = min(g.n, r0 + g.rows);
  const int bd = blockDim.x;
  for (int i0 = 0; i0 < k; i0 += 8) {
    const int nc = min(8, k - i0);
    double acc[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[j] = 0.0;
    for (int r = r0 + threadIdx.x; r < r1; r += 2 * bd) {
      const bool two = r + bd < r1;
      const double wr = w[r], wr2 = two ? w[r + bd] : 0.0;
      const double *q = g.Q + (size_t)i0 * g.n + r;
      double a[8], b[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        a[j] = j < nc ? q[(size_t)j * g.n] : 0.0;
        b[j] = (j < nc && two) ? q[(size_t)j * g.n + bd] : 0.0;
      }
#pragma unroll
      for (int j = 0; j < 8; ++j)
        if (j < nc) acc[j] += a[j] * wr;
#pragma unroll
      for (int j = 0; j < 8; ++j)
        if (j < nc && two) acc[j] += b[j] * wr2;
    }
    const double sc = pw_sum8(acc);
    if ((lane & 3) == 0) red[wid][lane >> 2] = sc;
    __syncthreads();
    if ((int)threadIdx.x < nc) {
      double t = 0.0;
      for (int q = 0; q < kGW; ++q) t += red[q][threadIdx.x];
      g.part[(size_t)blockIdx.x * g.pstride + i0 + threadIdx.x] = t;
    }
    __syncthreads();
  }
  if (!pres_last_cta(g.cnt)) return;
  for (int i0 = 4 * wid; i0 < k; i0 += 4 * kGW) {
    const int m = min(4, k - i0);
    const double t = pw_sum_strided4(g.part + i0, g.G, g.pstride, m);
    if ((lane & 7) == 0 && (lane >> 3) < m) h[i0 + (lane >> 3)] = t;
  }
  __syncthreads();
  if (threadIdx.x == 0) *g.cnt = 0u;
}

// w -= sum_i h_i Q_i over this CTA's rows (h staged in shared memory; the
// columns of a row subtracted in order; two rows a thread at a time, sixteen
// loads in flight).
__device__ void pres_orth(const GA &g, double *w, int k, const double *h) {
  __shared__ double hs[kPresMaxIter];
  for (int i = threadIdx.x; i < k; i += blockDim.x) hs[i] = h[i];
  __syncthreads();
  const int r0 = blockIdx.x * g.rows, r1 = min(g.n, r0 + g.rows);
  const int bd = blockDim.x;
  const size_t n = g.n;
  for (int r = r0 + threadIdx.x; r < r1; r += 2 * bd) {
    const bool two = r + bd < r1;
    double t = w[r], u = two ? w[r + bd] : 0.0;
    const double *q = g.Q + r;
    int i = 0;
    for (; i + 8 <= k; i += 8) {
      double a[8], b[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        a[j] = q[(size_t)(i + j) * n];
        b[j] = two ? q[(size_t)(i + j) * n + bd] : 0.0;
      }
#pragma unroll
      for (int j = 0; j < 8; ++j) t -= hs[i + j] * a[j];
#pragma unroll
      for (int j = 0; j < 8; ++j) u -= hs[i + j] * b[j];
    }
    for (; i < k; ++i) {
      t -= hs[i] * q[(size_t)i * n];
      if (two) u -= hs[i] * q[(size_t)i * n + bd];
    }
    w[r] = t;
    if (two) w[r + bd] = u;
  }
  __syncthreads();
}

// Step k = st->iter, pass 1: h1 = Q^T w. (The step kernels read k from the
// device scalars and skip once the solve is finished, so a chunk of steps
// is the same launch sequence every time.)
__global__ void __launch_bounds__(kGT) pres_dots1_kernel(GA g) {
  if (g.st->done) return;
  const int k = g.st->iter;
  pres_dots(g, g.Q + (size_t)k * g.n, k, g.h1);
}

// Step k, pass 2: w -= Q h1, h2 = Q^T w.
__global__ void __launch_bounds__(kGT) pres_dots2_kernel(GA g) {
  if (g.st->done) return;
  const int k = g.st->iter;
  double *w = g.Q + (size_t)k * g.n;
  pres_orth(g, w, k, g.h1);
  pres_dots(g, w, k, g.h2);
}

// Step k: w -= Q h2, ||w||; the last CTA writes H(:, k-1), applies the
// earlier Givens rotations and the new one (mobility_solver.cpp:2370-2404),
// tests convergence (:2409-2413) and, when finishing, back-solves y (:2419-
// 2438) with warp-parallel inner sums. The column and the rotations are
// staged in shared memory for the serial rotation chain.
__global__ void __launch_bounds__(kGT) pres_norm_givens_kernel(GA g) {
  __shared__ double red[kGW];
  __shared__ double hc[kPresMaxIter + 1], css[kPresMaxIter], sns[kPresMaxIter];
  __shared__ int fin;
  if (g.st->done) return;
  const int k = g.st->iter;
  double *w = g.Q + (size_t)k * g.n;
  pres_orth(g, w, k, g.h2);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int r0 = blockIdx.x * g.rows, r1 = min(g.n, r0 + g.rows);
  double t = 0.0;
  for (int r = r0 + threadIdx.x; r < r1; r += blockDim.x) t += w[r] * w[r];
  t = pw_sum(t);
  if (lane == 0) red[wid] = t;
  __syncthreads();
  if (threadIdx.x == 0) {
    double u = 0.0;
    for (int q = 0; q < kGW; ++q) u += red[q];
    g.part[(size_t)blockIdx.x * g.pstride] = u;
  }
  if (!pres_last_cta(g.cnt)) return;
  const int ld = g.ld, c = k - 1;
  double *H = g.H;
  for (int i = threadIdx.x; i < k; i += blockDim.x) {
    hc[i] = g.h1[i] + g.h2[i];
    if (i < c) {
      css[i] = g.cs[i];
      sns[i] = g.sn[i];
    }
  }
  double ss = 0.0;
  if (wid == 0) ss = pw_sum_strided(g.part, g.G, g.pstride);
  __syncthreads();
  PresScalars *st = g.st;
  if (threadIdx.x == 0) {
    const double qn = sqrt(ss);
    st->qnorm = qn;
    hc[k] = qn;
    for (int i = 1; i < k; ++i) {
      const double a0 = hc[i - 1], a1 = hc[i];
      const double tt = css[i - 1] * a0 + sns[i - 1] * a1;
      hc[i] = css[i - 1] * a1 - sns[i - 1] * a0;
      hc[i - 1] = tt;
    }
    const double hk = hc[k], hd = hc[c];
    double cs, sn;
    if (hk == 0.0) {
      cs = 1.0;
      sn = 0.0;
    } else if (fabs(hk) > fabs(hd)) {
      const double tt = hd / hk;
      sn = (2.0 * (double)(hk > 0.0) - 1.0) / sqrt(1.0 + tt * tt);
      cs = tt * sn;
    } else {
      const double tt = hk / hd;
      cs = (2.0 * (double)(hd > 0.0) - 1.0) / sqrt(1.0 + tt * tt);
      sn = tt * cs;
    }
    g.cs[c] = cs;
    g.sn[c] = sn;
    hc[c] = cs * hd + sn * hk;
    hc[k] = 0.0;
    g.beta[k] = -sn * g.beta[c];
    g.beta[c] = cs * g.beta[c];
    const double rel = fabs(g.beta[k]) / st->norm_rhs;
    st->rel = rel;
    const int finished = (rel <= st->tol) || (k == g.max_iter) || !(rel == rel);
    if (!(rel == rel)) st->status = 1;
    st->iters = k;
    st->done = finished;
    if (!finished) st->iter = k + 1;
    fin = finished;
    *g.cnt = 0u;
  }
  __syncthreads();
  for (int i = threadIdx.x; i <= k; i += blockDim.x) H[i + (size_t)c * ld] = hc[i];
  __syncthreads();
  if (!fin || wid != 0) return;
  // y(k-1) = beta / H, then upward: y(i) = (beta(i) - sum_{j>i} H(i,j) y(j)) / H(i,i)
  for (int i = k - 1; i >= 0; --i) {
    double sacc = 0.0;
    for (int j = i + 1 + lane; j < k; j += 32) sacc += g.H[i + (size_t)j * ld] * g.y[j];
    sacc = pw_sum(sacc);
    if (lane == 0) g.y[i] = (g.beta[i] - sacc) / g.H[i + (size_t)i * ld];
    __syncwarp();
    __threadfence_block();
  }
}

// Q_k = w / ||w|| for the step just built (k = st->iter - 1; unless finished).
__global__ void pres_scale_kernel(GA g) {
  if (g.st->done) return;
  const int k = g.st->iter - 1;
  const double inv = 1.0 / g.st->qnorm;
  double *w = g.Q + (size_t)k * g.n;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < g.n; r += gridDim.x * blockDim.x)
    w[r] *= inv;
}

// tmp = sum_{i < k} y_i Q_i.
__global__ void pres_qy_kernel(GA g, int k, double *tmp) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < g.n; r += gridDim.x * blockDim.x) {
    double t = 0.0;
    for (int i = 0; i < k; ++i) t += g.y[i] * g.Q[(size_t)i * g.n + r];
    tmp[r] = t;
  }
}

__global__ void pres_axpy_kernel(double *x, const double *d, int n) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x)
    x[r] += d[r];
}

}  // namespace

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
void pres_free(tfs_solver *s) {
  PresState *p = s->pres;
  if (p == nullptr) return;
  double *dbufs[] = {p->kphi, p->kth, p->phase_v, p->omega0, p->angle_v, p->pdot, p->vbody,
                     p->tab_p, p->tab_a, p->fil, p->m6inv, p->b, p->x, p->z, p->tmp, p->Q, p->H,
                     p->beta, p->cs, p->sn, p->y, p->h1, p->h2, p->part, p->part6, p->rec_s,
                     p->rec_b, p->f6, p->v6, p->v_ss, p->v_sb, p->v_bb, p->v_bs, p->qpart};
  for (double *d : dbufs) cudaFree(d);
  cudaFree(p->cnt);
  cudaFree(p->st);
  cudaFree(p->qcnt);
  cudaFree(p->jobs_dev);
  cudaFree(p->rec_s32);
  cudaFree(p->rec_b32);
  cudaFree(p->x_all);
  cudaFree(p->v_all);
  cudaFree(p->rec_ff);
  cudaFree(p->body_dev);
  cudaFree(p->jobs_it_dev);
  cudaFree(p->jobs32_it_dev);
  for (cudaGraphExec_t g : p->graph)
    if (g) cudaGraphExecDestroy(g);
  cudaFree(p->jobs32_dev);
  if (p->st_host) cudaFreeHost(p->st_host);
  delete p;
  s->pres = nullptr;
}

namespace {

PA pres_pa(tfs_solver *s) {
  const PresState *p = s->pres;
  PA a{};
  a.ns = p->ns;
  a.nb = p->nb;
  a.nfil = p->nfil;
  a.nseg = p->nseg;
  a.n = p->n;
  a.o_body = p->o_body;
  a.o_phase = p->o_phase;
  a.o_angle = p->o_angle;
  a.free_body = p->free_body;
  a.phase = p->phase;
  a.angle = p->angle;
  a.weak = p->weak;
  a.c = 6.0 * kPiP * s->cfg.mu * s->cfg.a_seg;
  a.cb = 6.0 * kPiP * s->cfg.mu * s->cfg.a_blob;
  a.body = p->body_dev;
  a.x_segs = s->x_segs;
  a.d_blobs = s->diff;
  a.kphi = p->kphi;
  a.kth = p->kth;
  a.fil = p->fil;
  a.m6inv = p->m6inv;
  a.part6 = p->part6;
  a.cnt = p->cnt;
  a.fil_warps = p->nfil;
  a.blob_warps = (p->nb + 31) / 32;
  return a;
}

int pa_ctas(const PA &a) { return std::max(1, (a.fil_warps + a.blob_warps + kPW - 1) / kPW); }

GA pres_ga(tfs_solver *s) {
  PresState *p = s->pres;
  GA g{};
  g.n = p->n;
  g.G = p->G;
  g.rows = p->rows;
  g.ld = kPresMaxIter + 1;
  g.pstride = p->pstride;
  g.max_iter = p->max_iter;
  g.Q = p->Q;
  g.H = p->H;
  g.beta = p->beta;
  g.cs = p->cs;
  g.sn = p->sn;
  g.y = p->y;
  g.h1 = p->h1;
  g.h2 = p->h2;
  g.part = p->part;
  g.cnt = p->cnt;
  g.st = p->st;
  return g;
}

// One 3x3 work-queue job: targets (records tgt, n_tgt, radius at) against
// sources (records src, n_src, radius as) into out.
QueueJob pres_job(tfs_solver *s, const double *tgt, int n_tgt, double at, const double *src,
                  int n_src, double as, double *out, double *partial, unsigned *block_done) {
  QueueJob j{};
  j.tgt_rec = tgt;
  j.n_tgt = n_tgt;
  j.a_tgt = at;
  j.src_a = src;
  j.n_a = n_src;
  j.a_a = as;
  j.out = out;
  j.vd = 3;
  j.mode = OUT_ASSIGN;
  j.scale = 1.0 / (8.0 * kPiP * s->cfg.mu);
  const double q[5] = {at, as, (at + as) * (at + as), (at * at + as * as) / 3.0,
                       -(at * at + as * as)};
  for (int k = 0; k < 5; ++k) {
    j.pc64[0][k] = j.pc64[1][k] = q[k];
    j.pc32[0][k] = j.pc32[1][k] = (float)q[k];
  }
  queue_chunking(n_src, s->ns + s->nb, &j.chunk, &j.n_chunks);
  j.partial = partial;
  j.block_done = block_done;
  return j;
}

int pres_alloc(tfs_solver *s) {
  PresState *p = s->pres;
  const size_t n = p->n, ns = p->ns, nb = p->nb, nf = p->nfil;
  const int ld = kPresMaxIter + 1;
  // GMRES vector kernels: CTAs of at least 256 consecutive rows; up to one
  // per SM as the rows allow, beyond that a multiple of the SM count (at most
  // eight per SM). Each SM's FP64 pipe bounds these kernels on this part, so
  // every SM gets the same share of the rows.
  const size_t sms = (size_t)num_sms(), g0 = (n + 255) / 256;
  p->G = (int)std::max<size_t>(1, g0 <= sms ? g0 : std::min<size_t>(8 * sms, g0 / sms * sms));
  p->rows = (int)((n + p->G - 1) / p->G);
  p->pstride = kPresMaxIter + 2;
  const size_t warps = nf + (nb + 31) / 32;
  struct B {
    double **p;
    size_t n;
  } bufs[] = {{&p->kphi, 3 * ns}, {&p->kth, 3 * ns}, {&p->phase_v, nf}, {&p->omega0, nf},
              {&p->angle_v, nf}, {&p->pdot, nf}, {&p->vbody, 6}, {&p->fil, kFilC * nf},
              {&p->m6inv, 36}, {&p->b, n}, {&p->x, n}, {&p->z, n}, {&p->tmp, n},
              {&p->Q, n * ld}, {&p->H, (size_t)ld * ld}, {&p->beta, (size_t)ld},
              {&p->cs, (size_t)ld}, {&p->sn, (size_t)ld}, {&p->y, (size_t)ld},
              {&p->h1, (size_t)ld}, {&p->h2, (size_t)ld}, {&p->part, (size_t)p->G * p->pstride},
              {&p->part6, 6 * std::max<size_t>(1, warps)}, {&p->rec_s, 6 * ns}, {&p->rec_b, 6 * nb},
              {&p->v_ss, 3 * ns}, {&p->v_sb, 3 * ns}, {&p->v_bb, 3 * nb}, {&p->v_bs, 3 * nb}};
  int rc;
  for (auto &b : bufs)
    if ((rc = alloc_dev((void **)b.p, sizeof(double) * std::max<size_t>(1, b.n))) != TFS_OK) return rc;
  if (p->weak && ((rc = alloc_dev((void **)&p->f6, sizeof(double) * 6 * ns)) != TFS_OK ||
                  (rc = alloc_dev((void **)&p->v6, sizeof(double) * 6 * ns)) != TFS_OK))
    return rc;
  if ((rc = alloc_dev((void **)&p->cnt, sizeof(unsigned) * 4)) != TFS_OK ||
      (rc = alloc_dev((void **)&p->st, sizeof(PresScalars))) != TFS_OK)
    return rc;
  TFS_CUDA(cudaHostAlloc((void **)&p->st_host, sizeof(PresScalars), cudaHostAllocDefault),
           "cudaHostAlloc");
  // the work-queue jobs: seg <- seg (unless weakly coupled), seg <- blob,
  // blob <- blob, blob <- seg, each with its own partials and arrival counters
  const size_t part_s = (size_t)kMaxSplits * 3 * ns, part_b = (size_t)kMaxSplits * 3 * nb;
  const size_t blk_s = (ns + 31) / 32 + 1, blk_b = (nb + 31) / 32 + 1;
  if ((rc = alloc_dev((void **)&p->qpart, sizeof(double) * std::max<size_t>(1, 2 * part_s + 2 * part_b))) != TFS_OK ||
      (rc = alloc_dev((void **)&p->qcnt, sizeof(unsigned) * (2 + 2 * blk_s + 2 * blk_b))) != TFS_OK ||
      (rc = alloc_dev((void **)&p->jobs_dev, sizeof(QueueJob) * 4)) != TFS_OK)
    return rc;
  TFS_CUDA(cudaMemset(p->cnt, 0, sizeof(unsigned) * 4), "cudaMemset");
  TFS_CUDA(cudaMemset(p->qcnt, 0, sizeof(unsigned) * (2 + 2 * blk_s + 2 * blk_b)), "cudaMemset");
  TFS_CUDA(cudaMemset(p->x, 0, sizeof(double) * n), "cudaMemset");
  TFS_CUDA(cudaMemset(p->H, 0, sizeof(double) * ld * ld), "cudaMemset");
  TFS_CUDA(cudaMemset(p->vbody, 0, sizeof(double) * 6), "cudaMemset");
  unsigned *blk = p->qcnt + 2;
  double *part = p->qpart;
  const double as = s->cfg.a_seg, ab = s->cfg.a_blob;
  p->n_jobs = 0;
  if (ns > 0 && !p->weak)
    p->jobs[p->n_jobs++] = pres_job(s, p->rec_s, (int)ns, as, p->rec_s, (int)ns, as, p->v_ss, part, blk);
  if (ns > 0 && nb > 0)
    p->jobs[p->n_jobs++] = pres_job(s, p->rec_s, (int)ns, as, p->rec_b, (int)nb, ab, p->v_sb,
                                    part + part_s, blk + blk_s);
  if (nb > 0)
    p->jobs[p->n_jobs++] = pres_job(s, p->rec_b, (int)nb, ab, p->rec_b, (int)nb, ab, p->v_bb,
                                    part + 2 * part_s, blk + 2 * blk_s);
  if (nb > 0 && ns > 0)
    p->jobs[p->n_jobs++] = pres_job(s, p->rec_b, (int)nb, ab, p->rec_s, (int)ns, as, p->v_bs,
                                    part + 2 * part_s + part_b, blk + 2 * blk_s + blk_b);
  // costliest first
  std::stable_sort(p->jobs, p->jobs + p->n_jobs, [](const QueueJob &x, const QueueJob &y) {
    return (long long)x.n_tgt * (x.n_a + x.n_b) > (long long)y.n_tgt * (y.n_a + y.n_b);
  });
  TFS_CUDA(cudaMemcpy(p->jobs_dev, p->jobs, sizeof(QueueJob) * p->n_jobs, cudaMemcpyHostToDevice),
           "copy queue jobs");
  if (p->weak && ns > 0) {  // partials and counters of the absent seg <- seg job
    p->hook_ss = pres_job(s, p->rec_s, (int)ns, as, p->rec_s, (int)ns, as, p->v_ss, part, blk);
    TFS_CUDA(cudaMemcpy(p->jobs_dev + 3, &p->hook_ss, sizeof(QueueJob), cudaMemcpyHostToDevice),
             "copy queue jobs");
  }
  // the same jobs on FP32 records (FP32C inner solves): same partials and
  // arrival counters (launches never overlap), float2 partial sums
  if ((rc = alloc_dev((void **)&p->rec_s32, sizeof(float) * 8 * std::max<size_t>(1, ns))) != TFS_OK ||
      (rc = alloc_dev((void **)&p->rec_b32, sizeof(float) * 8 * std::max<size_t>(1, nb))) != TFS_OK ||
      (rc = alloc_dev((void **)&p->jobs32_dev, sizeof(QueueJob) * 4)) != TFS_OK)
    return rc;
  for (int j = 0; j < p->n_jobs; ++j) {
    QueueJob q = p->jobs[j];
    q.tgt_rec = q.tgt_rec == p->rec_s ? (const void *)p->rec_s32 : (const void *)p->rec_b32;
    q.src_a = q.src_a == p->rec_s ? (const void *)p->rec_s32 : (const void *)p->rec_b32;
    p->jobs32[j] = q;
  }
  TFS_CUDA(cudaMemcpy(p->jobs32_dev, p->jobs32, sizeof(QueueJob) * p->n_jobs,
                      cudaMemcpyHostToDevice),
           "copy queue jobs");
  // the step jobs: the same, skipping once the solve is finished
  if ((rc = alloc_dev((void **)&p->jobs_it_dev, sizeof(QueueJob) * 4)) != TFS_OK ||
      (rc = alloc_dev((void **)&p->jobs32_it_dev, sizeof(QueueJob) * 4)) != TFS_OK ||
      (rc = alloc_dev((void **)&p->body_dev, sizeof(double) * 3)) != TFS_OK)
    return rc;
  {
    QueueJob it64[4], it32[4];
    for (int j = 0; j < p->n_jobs; ++j) {
      it64[j] = p->jobs[j];
      it32[j] = p->jobs32[j];
      it64[j].skip = &p->st->done;
      it32[j].skip = &p->st->done;
    }
    TFS_CUDA(cudaMemcpy(p->jobs_it_dev, it64, sizeof(QueueJob) * p->n_jobs, cudaMemcpyHostToDevice),
             "copy queue jobs");
    TFS_CUDA(cudaMemcpy(p->jobs32_it_dev, it32, sizeof(QueueJob) * p->n_jobs,
                        cudaMemcpyHostToDevice),
             "copy queue jobs");
  }
  if (p->weak && ns > 0 && s->wc_z == nullptr &&  // the weakly coupled product's means, totals
      ((rc = alloc_dev((void **)&s->wc_z, sizeof(double) * 3 * p->nfil)) != TFS_OK ||
       (rc = alloc_dev((void **)&s->wc_f, sizeof(double) * 3 * p->nfil)) != TFS_OK))
    return rc;
  p->use_ff = !p->weak && s->cfg.a_seg == s->cfg.a_blob && ns + nb > 0;
  if (p->use_ff &&
      ((rc = alloc_dev((void **)&p->x_all, sizeof(double) * 3 * (ns + nb))) != TFS_OK ||
       (rc = alloc_dev((void **)&p->v_all, sizeof(double) * 3 * (ns + nb))) != TFS_OK ||
       (rc = alloc_dev(&p->rec_ff, ff_record_bytes() * (ns + nb))) != TFS_OK))
    return rc;
  // outputs of absent blocks stay zero
  for (double *v : {p->v_ss, p->v_sb})
    TFS_CUDA(cudaMemset(v, 0, sizeof(double) * std::max<size_t>(1, 3 * ns)), "cudaMemset");
  for (double *v : {p->v_bb, p->v_bs})
    TFS_CUDA(cudaMemset(v, 0, sizeof(double) * std::max<size_t>(1, 3 * nb)), "cudaMemset");
  return TFS_OK;
}

// out = A z (resid == nullptr) or resid - A z; fp32: the pair sums of the
// work-queue kernel in FP32 with compensated accumulation (the origin must be
// current: ensure_origin before). it != nullptr: an Arnoldi step (out is
// column it->iter of out; everything skips once the solve is finished).
int pres_operator(tfs_solver *s, int fp32, const double *z, const double *resid, double *out,
                  const PresScalars *it = nullptr) {
  PresState *p = s->pres;
  const PA a = pres_pa(s);
  const int np = p->ns + p->nb;
  if (np > 0) {
    if (fp32) {
      pres_pack32_kernel<<<(np + 255) / 256, 256, 0, s->stream>>>(a, z, s->x_blobs, s->origin,
                                                                  p->rec_s32, p->rec_b32, it);
      if (p->weak)  // the weakly coupled segment block stays FP64
        pres_pack_kernel<<<(np + 255) / 256, 256, 0, s->stream>>>(a, z, s->x_blobs, p->rec_s,
                                                                  p->rec_b, p->f6, it);
    } else {
      pres_pack_kernel<<<(np + 255) / 256, 256, 0, s->stream>>>(
          a, z, s->x_blobs, p->rec_s, p->rec_b, p->weak ? p->f6 : nullptr, it);
    }
    count_launch_n(fp32 && p->weak ? 2 : 1);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "prescribed pack kernel");
  if (p->weak && p->ns > 0) {  // (buffers allocated by the setup)
    e = launch_msf(s->x_segs, p->f6, p->nfil, p->nseg, s->cfg.a_seg, s->cfg.mu, s->wc_z, s->wc_f,
                   p->v6, s->stream);
    if (e != cudaSuccess) return cuda_fail(e, "weakly coupled segment product");
  }
  if (p->n_jobs > 0) {
    const QueueJob *d64 = it ? p->jobs_it_dev : p->jobs_dev;
    const QueueJob *d32 = it ? p->jobs32_it_dev : p->jobs32_dev;
    e = fp32 ? launch_queue(1, s->qtune[1][QK_MBB], Q_BLOB, d32, p->jobs32, p->n_jobs, p->qcnt,
                            s->stream)
             : launch_queue(0, s->qtune[0][QK_MBB], Q_BLOB, d64, p->jobs, p->n_jobs, p->qcnt,
                            s->stream);
    if (e != cudaSuccess) return cuda_fail(e, "RPY work-queue kernel (prescribed)");
  }
  pres_combine_kernel<<<pa_ctas(a), kPT, 0, s->stream>>>(a, z, p->v_ss, p->v6, p->v_sb, p->v_bb,
                                                         p->v_bs, resid, out, it);
  count_launch();
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "prescribed combine kernel");
  return TFS_OK;
}

// out = P^-1 in (in != out); it: as for pres_operator (in is column
// it->iter - 1 of in).
int pres_precond(tfs_solver *s, const double *in, double *out, const PresScalars *it = nullptr) {
  const PA a = pres_pa(s);
  pres_precond_a_kernel<<<pa_ctas(a), kPT, 0, s->stream>>>(a, in, out, it);
  count_launch();
  if (a.free_body) {
    pres_precond_b_kernel<<<pa_ctas(a), kPT, 0, s->stream>>>(a, out, it);
    count_launch();
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "prescribed preconditioner kernels");
  return TFS_OK;
}

int pres_rhs(tfs_solver *s) {
  PresState *p = s->pres;
  const PA a = pres_pa(s);
  RhsArgs r{};
  r.tab_p = p->tab_p;
  r.tab_a = p->tab_a;
  r.n_tab_p = p->n_tab_p;
  r.n_tab_a = p->n_tab_a;
  r.phase = p->phase_v;
  r.omega0 = p->omega0;
  r.angle = p->angle_v;
  r.pdot = p->pdot;
  r.vbody = p->vbody;
  r.gff = p->cfg.gen_force_magnitude_factor;
  r.tsf = p->cfg.torsional_spring_magnitude_factor;
  r.fil_length = p->cfg.fil_length;
  pres_rhs_kernel<<<pa_ctas(a), kPT, 0, s->stream>>>(a, r, p->b);
  count_launch();
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "prescribed right-hand side kernel");
  return TFS_OK;
}

int pres_check(tfs_solver *s) {
  TFS_CHECK_SOLVER(s);
  if (s->pres == nullptr) return fail(TFS_ESTATE, "call tfs_prescribed_setup first");
  return TFS_OK;
}

int upload(tfs_solver *s, double *dst, const double *src, size_t n, const char *what) {
  if (n == 0) return TFS_OK;
  TFS_CUDA(cudaMemcpyAsync(dst, src, sizeof(double) * n, cudaMemcpyHostToDevice, s->stream), what);
  return TFS_OK;
}

// Host read of the device scalars (synchronises the stream).
int pres_read_scalars(tfs_solver *s, const char *what) {
  PresState *p = s->pres;
  TFS_CUDA(cudaMemcpyAsync(p->st_host, p->st, sizeof(PresScalars), cudaMemcpyDeviceToHost,
                           s->stream),
           "read solve scalars");
  TFS_CUDA(cudaStreamSynchronize(s->stream), what);
  return TFS_OK;
}

// kPresChunk Arnoldi steps: preconditioner, operator, CGS2, norm and Givens,
// every kernel reading the step from the device scalars and skipping once the
// solve is finished (the same launch sequence every time).
int pres_chunk(tfs_solver *s, int fp32) {
  PresState *p = s->pres;
  const GA g = pres_ga(s);
  int rc;
  for (int c = 0; c < kPresChunk; ++c) {
    if ((rc = pres_precond(s, p->Q, p->z, p->st)) != TFS_OK) return rc;
    if ((rc = pres_operator(s, fp32, p->z, nullptr, p->Q, p->st)) != TFS_OK) return rc;
    pres_dots1_kernel<<<g.G, kGT, 0, s->stream>>>(g);
    pres_dots2_kernel<<<g.G, kGT, 0, s->stream>>>(g);
    pres_norm_givens_kernel<<<g.G, kGT, 0, s->stream>>>(g);
    pres_scale_kernel<<<g.G, kGT, 0, s->stream>>>(g);
    count_launch_n(4);
    TFS_CUDA(cudaGetLastError(), "prescribed Arnoldi step");
  }
  return TFS_OK;
}

// The chunk as a CUDA graph, captured once per precision (and work-queue
// variant); nullptr: launch it directly (capture unavailable, or kernel
// timing on).
cudaGraphExec_t pres_graph(tfs_solver *s, int fp32, long long *kernels) {
  PresState *p = s->pres;
  const int var = s->qtune[fp32][QK_MBB];
  if (!p->graphs_ok || s->timing) return nullptr;
  if (p->graph[fp32] != nullptr && p->graph_variant[fp32] == var) {
    *kernels = p->graph_kernels[fp32];
    return p->graph[fp32];
  }
  if (p->graph[fp32] != nullptr) {
    cudaGraphExecDestroy(p->graph[fp32]);
    p->graph[fp32] = nullptr;
  }
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  const long long before = launch_count();
  if (cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    cudaGetLastError();
    p->graphs_ok = false;
    return nullptr;
  }
  const int rc = pres_chunk(s, fp32);
  const cudaError_t e = cudaStreamEndCapture(s->stream, &graph);
  const long long recorded = launch_count() - before;
  count_launch_n(-recorded);  // recorded, not launched
  if (rc != TFS_OK || e != cudaSuccess || graph == nullptr ||
      cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) {
    cudaGetLastError();
    if (graph) cudaGraphDestroy(graph);
    p->graphs_ok = false;
    return nullptr;
  }
  cudaGraphDestroy(graph);
  p->graph[fp32] = exec;
  p->graph_kernels[fp32] = recorded;
  p->graph_variant[fp32] = var;
  *kernels = recorded;
  return exec;
}

// Arnoldi steps from the normalised Q_0 (beta[0], st->norm_rhs, st->tol and
// st->iter = 1 set) in chunks, one poll of the scalars per chunk, until
// |beta_k| <= tol norm_rhs or the cap; then x += P^-1 (Q y). fp32: FP32 pair
// sums in the operator. The first chunk of each precision runs eagerly (it
// initialises the launch paths), later ones replay the captured graph.
int pres_arnoldi(tfs_solver *s, int fp32, int *iters) {
  PresState *p = s->pres;
  const GA g = pres_ga(s);
  int rc;
  *iters = 0;
  const int max_chunks = p->max_iter / kPresChunk + 2;
  bool eager = p->graph[fp32] == nullptr;
  for (int c = 0; c < max_chunks; ++c) {
    long long kernels = 0;
    cudaGraphExec_t exec = eager ? nullptr : pres_graph(s, fp32, &kernels);
    if (exec != nullptr) {
      TFS_CUDA(cudaGraphLaunch(exec, s->stream), "prescribed Arnoldi chunk");
      count_launch_n(kernels);
    } else if ((rc = pres_chunk(s, fp32)) != TFS_OK) {
      return rc;
    }
    eager = false;
    if ((rc = pres_read_scalars(s, "prescribed Arnoldi chunk")) != TFS_OK) return rc;
    if (p->st_host->status != 0) return fail(TFS_ENAN, "non-finite GMRES residual");
    if (p->st_host->done) break;
  }
  if (!p->st_host->done) return fail(TFS_ENOTCONV, "GMRES did not finish within %d steps", p->max_iter);
  *iters = p->st_host->iters;
  pres_qy_kernel<<<g.G, kGT, 0, s->stream>>>(g, *iters, p->tmp);
  count_launch();
  if ((rc = pres_precond(s, p->tmp, p->z)) != TFS_OK) return rc;
  pres_axpy_kernel<<<g.G, kGT, 0, s->stream>>>(p->x, p->z, p->n);
  count_launch();
  TFS_CUDA(cudaGetLastError(), "prescribed GMRES finish");
  return TFS_OK;
}

// out = resid - A z with the pair sums in float-float arithmetic (use_ff):
// v = M z over the concatenated particles, then the couplings.
int pres_operator_ff(tfs_solver *s, const double *z, const double *resid, double *out) {
  PresState *p = s->pres;
  int rc;
  if ((rc = ensure_origin(s)) != TFS_OK) return rc;
  const int np = p->ns + p->nb;
  TFS_CUDA(cudaMemcpyAsync(p->x_all, s->x_segs, sizeof(double) * 3 * p->ns,
                           cudaMemcpyDeviceToDevice, s->stream),
           "gather positions");
  TFS_CUDA(cudaMemcpyAsync(p->x_all + 3 * (size_t)p->ns, s->x_blobs, sizeof(double) * 3 * p->nb,
                           cudaMemcpyDeviceToDevice, s->stream),
           "gather positions");
  const size_t scratch = (size_t)kMaxSplits * 3 * (2 * (size_t)p->ns + 2 * (size_t)p->nb);
  cudaError_t e = launch_bb_ff(p->x_all, z, np, s->origin, s->cfg.a_seg,
                               1.0 / (8.0 * kPiP * s->cfg.mu), p->rec_ff, p->v_all, p->qpart,
                               scratch, s->stream);
  if (e != cudaSuccess) return cuda_fail(e, "float-float product (prescribed)");
  const PA a = pres_pa(s);
  pres_combine_kernel<<<pa_ctas(a), kPT, 0, s->stream>>>(a, z, p->v_all, nullptr, nullptr,
                                                         p->v_all + 3 * (size_t)p->ns, nullptr,
                                                         resid, out, nullptr);
  count_launch();
  TFS_CUDA(cudaGetLastError(), "prescribed combine kernel");
  return TFS_OK;
}

// Q_0 = b - A x (FP64, or float-float pair sums under FP32C when every
// particle has the same radius) and its norm into st->beta0 (returned).
int pres_residual(tfs_solver *s, double *norm) {
  PresState *p = s->pres;
  const GA g = pres_ga(s);
  int rc;
  const bool ff = p->use_ff && s->cfg.precision == TFS_FP32C;
  if ((rc = ff ? pres_operator_ff(s, p->x, p->b, p->Q) : pres_operator(s, 0, p->x, p->b, p->Q)) !=
      TFS_OK)
    return rc;
  pres_norm_kernel<<<g.G, kGT, 0, s->stream>>>(g, p->Q, &p->st->beta0);
  count_launch();
  TFS_CUDA(cudaGetLastError(), "prescribed residual");
  if ((rc = pres_read_scalars(s, "prescribed residual")) != TFS_OK) return rc;
  *norm = p->st_host->beta0;
  return TFS_OK;
}

// Start an inner solve on Q_0 = r (unnormalised, ||r|| = nr; pres_q0_kernel
// then divides it by beta[0] = nr): the stopping test |beta_k| <= tol nr,
// from step 1.
__global__ void pres_inner_start_kernel(GA g, double nr, double tol) {
  PresScalars *st = g.st;
  st->norm_rhs = nr;
  st->tol = tol;
  st->iter = 1;
  st->flag = 0;
  st->done = 0;
  st->status = 0;
  g.beta[0] = nr;
}

int pres_solve(tfs_solver *s, int *iters_out) {
  PresState *p = s->pres;
  if (!p->have_kin) return fail(TFS_ESTATE, "set the kinematics first");
  const bool fp32 = s->cfg.precision == TFS_FP32C;
  const GA g = pres_ga(s);
  int rc;
  if (fp32 && (rc = ensure_origin(s)) != TFS_OK) return rc;  // the FP32 records' origin
  if ((rc = pres_rhs(s)) != TFS_OK) return rc;
  // ||rhs||; r0 = rhs - A x0 into Q_0 (FP64); beta0 = ||r0||; the warm-start
  // tests (mobility_solver.cpp:2121-2320)
  pres_norm_kernel<<<g.G, kGT, 0, s->stream>>>(g, p->b, &p->st->norm_rhs);
  count_launch();
  rc = fp32 && p->use_ff ? pres_operator_ff(s, p->x, p->b, p->Q)
                         : pres_operator(s, 0, p->x, p->b, p->Q);
  if (rc != TFS_OK) return rc;
  pres_norm_kernel<<<g.G, kGT, 0, s->stream>>>(g, p->Q, &p->st->beta0);
  pres_start_kernel<<<1, 1, 0, s->stream>>>(g, s->tol);
  pres_q0_kernel<<<g.G, kGT, 0, s->stream>>>(g, p->b, p->x);
  count_launch_n(3);
  TFS_CUDA(cudaGetLastError(), "prescribed GMRES start");
  if ((rc = pres_read_scalars(s, "prescribed GMRES start")) != TFS_OK) return rc;
  if (p->st_host->status == 1) return fail(TFS_ENAN, "non-finite residual at the start");
  const double nb = p->st_host->norm_rhs;
  int iters = 0, cycles = 0;
  double rel = nb > 0.0 ? p->st_host->beta0 / nb : 0.0;
  if (!p->st_host->done) {
    if (!fp32) {
      if ((rc = pres_arnoldi(s, 0, &iters)) != TFS_OK) return rc;
      rel = p->st_host->rel;
      cycles = 1;
    } else {
      // iterative refinement: inner GMRES with FP32 pair sums on the FP64
      // residual r, each to max(1e-7, tol ||b|| / (2 ||r||)), until
      // ||b - A x|| <= tol ||b|| in FP64 (a warm start within ~20x of the
      // tolerance needs one cycle); a cycle that does not reduce the residual
      // hands over to FP64 GMRES from the current x
      double cur = p->st_host->flag == 2 ? nb : p->st_host->beta0;
      bool fp64_finish = false;
      auto inner_tol = [&]() {
        return fp64_finish ? s->tol * nb / cur : std::max(kPresInnerFloor, 0.5 * s->tol * nb / cur);
      };
      pres_inner_start_kernel<<<1, 1, 0, s->stream>>>(g, cur, inner_tol());  // Q_0 normalised
      count_launch();
      for (;;) {
        int it = 0;
        if ((rc = pres_arnoldi(s, fp64_finish ? 0 : 1, &it)) != TFS_OK) return rc;
        iters += it;
        ++cycles;
        double nr;
        if ((rc = pres_residual(s, &nr)) != TFS_OK) return rc;
        if (!(nr == nr)) return fail(TFS_ENAN, "non-finite residual in the refinement");
        rel = nr / nb;
        if (rel <= s->tol || fp64_finish || cycles >= s->max_outer + 1) break;
        if (nr >= cur) {  // stalled: finish in FP64
          fp64_finish = true;
          ++p->fallbacks;
        }
        cur = nr;
        pres_inner_start_kernel<<<1, 1, 0, s->stream>>>(g, cur, inner_tol());
        pres_q0_kernel<<<g.G, kGT, 0, s->stream>>>(g, p->b, p->x);
        count_launch_n(2);
        TFS_CUDA(cudaGetLastError(), "prescribed refinement restart");
      }
    }
  }
  TFS_CUDA(cudaStreamSynchronize(s->stream), "prescribed solve");
  s->last_iters = iters;
  s->last_outer = cycles;
  s->last_rel = rel;
  if (iters_out) *iters_out = iters;
  if (fp32 && rel > s->tol) return fail(TFS_ENOTCONV, "refinement stopped at %.3e", rel);
  return TFS_OK;
}

}  // namespace

// One block hook in the prescribed-cilia form: tgt_segs / src_segs pick the
// block (seg <- seg assigns, seg <- blob adds, blob <- blob assigns, blob <-
// seg adds).
int pres_hook(tfs_solver *s, bool tgt_segs, bool src_segs) {
  PresState *p = s->pres;
  const int n_tgt = tgt_segs ? p->ns : p->nb;
  const bool add = tgt_segs != src_segs;
  if (n_tgt == 0) return TFS_OK;
  double *out = tgt_segs ? s->v_segs : s->v_blobs;
  const int stride = tgt_segs ? 6 : 3;
  if ((src_segs ? p->ns : p->nb) == 0) {  // no sources: assign zero, or leave the sum alone
    if (!add)
      TFS_CUDA(cudaMemsetAsync(out, 0, sizeof(double) * stride * n_tgt, s->stream), "cudaMemsetAsync");
    return TFS_OK;
  }
  const PA a = pres_pa(s);
  const int np = p->ns + p->nb;
  pres_hook_pack_kernel<<<(np + 255) / 256, 256, 0, s->stream>>>(a, s->f_segs, s->f_blobs,
                                                                  s->x_blobs, p->rec_s, p->rec_b);
  count_launch();
  const void *tgt = tgt_segs ? (const void *)p->rec_s : (const void *)p->rec_b;
  const void *src = src_segs ? (const void *)p->rec_s : (const void *)p->rec_b;
  int j = -1;
  for (int q = 0; q < p->n_jobs; ++q)
    if (p->jobs[q].tgt_rec == tgt && p->jobs[q].src_a == src) j = q;
  double *v = nullptr;
  if (j >= 0) {
    cudaError_t e = launch_queue(0, s->qtune[0][QK_MBB], Q_BLOB, p->jobs_dev + j, &p->jobs[j], 1,
                                 p->qcnt, s->stream);
    if (e != cudaSuccess) return cuda_fail(e, "RPY work-queue kernel (prescribed hook)");
    v = p->jobs[j].out;
  } else {  // weakly coupled: the solve has no seg <- seg job; the hook's own
    cudaError_t e = launch_queue(0, s->qtune[0][QK_MBB], Q_BLOB, p->jobs_dev + 3, &p->hook_ss, 1,
                                 p->qcnt, s->stream);
    if (e != cudaSuccess) return cuda_fail(e, "RPY work-queue kernel (prescribed hook)");
    v = p->v_ss;
  }
  pres_hook_out_kernel<<<(n_tgt + 255) / 256, 256, 0, s->stream>>>(v, out, n_tgt, stride, add);
  count_launch();
  TFS_CUDA(cudaGetLastError(), "prescribed hook");
  return TFS_OK;
}

}  // namespace tfs

using namespace tfs;

extern "C" {

int tfs_prescribed_config_default(tfs_prescribed_config *pc, int flags, int nseg, double dl) {
  if (pc == nullptr) return fail(TFS_EINVAL, "null config");
  std::memset(pc, 0, sizeof *pc);
  pc->flags = flags;
  pc->gen_force_magnitude_factor = 1.0;
  pc->torsional_spring_magnitude_factor = 2.0;
  pc->fil_length = dl * (double)(nseg - 1);
  return TFS_OK;
}

int tfs_prescribed_setup(tfs_solver *s, const tfs_prescribed_config *pc,
                         const double *phase_force_refs, int n_phase_refs,
                         const double *angle_force_refs, int n_angle_refs) {
  TFS_CHECK_SOLVER(s);
  if (pc == nullptr) return fail(TFS_EINVAL, "null config");
  const int flags = pc->flags;
  if (flags & ~(TFS_PRESCRIBED_BODY | TFS_DYNAMIC_PHASE | TFS_DYNAMIC_ANGLE | TFS_WEAKLY_COUPLED))
    return fail(TFS_EINVAL, "unknown prescribed-cilia flags 0x%x", flags);
  const bool free_body = !(flags & TFS_PRESCRIBED_BODY);
  const bool phase = flags & TFS_DYNAMIC_PHASE, angle = flags & TFS_DYNAMIC_ANGLE;
  if (free_body && phase != angle)
    return fail(TFS_EINVAL,
                "free body: dynamic phase and dynamic shape rotation go together (the reference's "
                "free-body preconditioner, mobility_solver.cpp:1227-1393, indexes both)");
  if (s->cfg.nswim != 1) return fail(TFS_EINVAL, "the prescribed-cilia solve takes one swimmer");
  const int nseg = s->cfg.nseg;
  if (s->ns > 0 && (nseg < 1 || s->ns % nseg != 0))
    return fail(TFS_EINVAL, "the segments must form whole filaments of nseg = %d", nseg);
  if (s->nb > 0 && !s->have_refs) return fail(TFS_ESTATE, "set the blob references first");
  if (phase && (phase_force_refs == nullptr || n_phase_refs < 2))
    return fail(TFS_EINVAL, "dynamic phase needs the phase generalised-force table (>= 2 values)");
  if (angle && (angle_force_refs == nullptr || n_angle_refs < 2))
    return fail(TFS_EINVAL, "dynamic shape rotation needs the angle generalised-force table");
  pres_free(s);
  PresState *p = new (std::nothrow) PresState;
  if (p == nullptr) return fail(TFS_ENOMEM, "host allocation failed");
  s->pres = p;
  p->cfg = *pc;
  p->free_body = free_body;
  p->phase = phase;
  p->angle = angle;
  p->weak = flags & TFS_WEAKLY_COUPLED;
  p->nseg = nseg;
  p->nfil = s->ns > 0 ? s->ns / nseg : 0;
  p->ns = s->ns;
  p->nb = s->nb;
  p->o_body = 3 * (p->ns + p->nb);
  p->o_phase = p->o_body + (free_body ? 6 : 0);
  p->o_angle = p->o_phase + (phase ? p->nfil : 0);
  p->n = p->o_angle + (angle ? p->nfil : 0);
  p->max_iter = std::min(kPresMaxIter, p->n);
  int rc = pres_alloc(s);
  if (rc == TFS_OK && phase) {
    if ((rc = alloc_dev((void **)&p->tab_p, sizeof(double) * n_phase_refs)) == TFS_OK)
      rc = upload(s, p->tab_p, phase_force_refs, n_phase_refs, "copy phase force table");
    p->n_tab_p = n_phase_refs;
  }
  if (rc == TFS_OK && angle) {
    if ((rc = alloc_dev((void **)&p->tab_a, sizeof(double) * n_angle_refs)) == TFS_OK)
      rc = upload(s, p->tab_a, angle_force_refs, n_angle_refs, "copy angle force table");
    p->n_tab_a = n_angle_refs;
  }
  if (rc == TFS_OK) {
    cudaError_t e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) rc = cuda_fail(e, "prescribed setup");
  }
  if (rc != TFS_OK) pres_free(s);
  return rc;
}

int tfs_prescribed_size(tfs_solver *s, int *n) {
  int rc;
  if ((rc = pres_check(s)) != TFS_OK) return rc;
  if (n == nullptr) return fail(TFS_EINVAL, "null output");
  *n = s->pres->n;
  return TFS_OK;
}

int tfs_prescribed_set_kinematics(tfs_solver *s, const tfs_prescribed_kinematics *k) {
  int rc;
  if ((rc = pres_check(s)) != TFS_OK) return rc;
  if (k == nullptr) return fail(TFS_EINVAL, "null kinematics");
  PresState *p = s->pres;
  const size_t ns = p->ns, nf = p->nfil;
  if (ns > 0 && k->vel_dir_phase == nullptr) return fail(TFS_EINVAL, "null vel_dir_phase");
  if (p->angle && ns > 0 && (k->vel_dir_angle == nullptr || k->shape_rotation_angle == nullptr))
    return fail(TFS_EINVAL, "dynamic shape rotation needs vel_dir_angle and shape_rotation_angle");
  if ((p->phase || p->angle) && nf > 0 && (k->phase == nullptr || k->omega0 == nullptr))
    return fail(TFS_EINVAL, "the generalised forces need phase and omega0");
  if (!p->phase && nf > 0 && k->phase_dot == nullptr)
    return fail(TFS_EINVAL, "prescribed phase rates (phase_dot) needed without dynamic phase");
  if ((rc = upload(s, p->kphi, k->vel_dir_phase, 3 * ns, "copy kinematics")) != TFS_OK) return rc;
  if (p->angle) {
    if ((rc = upload(s, p->kth, k->vel_dir_angle, 3 * ns, "copy kinematics")) != TFS_OK ||
        (rc = upload(s, p->angle_v, k->shape_rotation_angle, nf, "copy kinematics")) != TFS_OK)
      return rc;
  }
  if (p->phase || p->angle) {
    if ((rc = upload(s, p->phase_v, k->phase, nf, "copy kinematics")) != TFS_OK ||
        (rc = upload(s, p->omega0, k->omega0, nf, "copy kinematics")) != TFS_OK)
      return rc;
  }
  if (!p->phase && (rc = upload(s, p->pdot, k->phase_dot, nf, "copy kinematics")) != TFS_OK)
    return rc;
  if (k->v_body != nullptr) {
    if ((rc = upload(s, p->vbody, k->v_body, 6, "copy body velocities")) != TFS_OK) return rc;
  } else {
    TFS_CUDA(cudaMemsetAsync(p->vbody, 0, sizeof(double) * 6, s->stream), "cudaMemsetAsync");
  }
  // per-filament constants and (free body) the body block's inverse, on the
  // current segment positions and body pose (swimmer::make_precon_mat runs
  // after the filaments' kinematics, swimmer.cpp:433-466); the body position
  // the solve's kernels read
  if ((rc = upload(s, p->body_dev, s->pose.x, 3, "copy body position")) != TFS_OK) return rc;
  const PA a = pres_pa(s);
  if (p->nfil > 0) {
    pres_fil_kernel<<<(p->nfil + kPW - 1) / kPW, kPT, 0, s->stream>>>(a, p->fil);
    count_launch();
  }
  TFS_CUDA(cudaMemsetAsync(p->st, 0, sizeof(PresScalars), s->stream), "cudaMemsetAsync");
  if (p->free_body) {
    pres_m6_kernel<<<1, 256, 0, s->stream>>>(a, p->m6inv, p->st);
    count_launch();
  }
  TFS_CUDA(cudaGetLastError(), "prescribed kinematics kernels");
  TFS_CUDA(cudaMemcpyAsync(p->st_host, p->st, sizeof(PresScalars), cudaMemcpyDeviceToHost, s->stream),
           "read solve scalars");
  TFS_CUDA(cudaStreamSynchronize(s->stream), "prescribed kinematics");
  if (p->st_host->status == 2) return fail(TFS_ENAN, "singular body block of the preconditioner");
  p->have_kin = true;
  return TFS_OK;
}

int tfs_prescribed_solve(tfs_solver *s, int *gmres_iters) {
  int rc;
  if ((rc = pres_check(s)) != TFS_OK) return rc;
  return pres_solve(s, gmres_iters);
}

int tfs_prescribed_compute_velocities(tfs_solver *s, const tfs_prescribed_kinematics *k,
                                      int *gmres_iters) {
  int rc;
  if ((rc = tfs_prescribed_set_kinematics(s, k)) != TFS_OK) return rc;
  return pres_solve(s, gmres_iters);
}

int tfs_prescribed_apply(tfs_solver *s, int which, const double *in, double *out) {
  int rc;
  if ((rc = pres_check(s)) != TFS_OK) return rc;
  PresState *p = s->pres;
  if (!p->have_kin) return fail(TFS_ESTATE, "set the kinematics first");
  if (out == nullptr || (which != 2 && in == nullptr)) return fail(TFS_EINVAL, "null vector");
  if (which == 0 || which == 1) {
    if ((rc = upload(s, p->tmp, in, p->n, "copy vector")) != TFS_OK) return rc;
    rc = which == 0 ? pres_operator(s, s->cfg.precision == TFS_FP32C, p->tmp, nullptr, p->z)
                    : pres_precond(s, p->tmp, p->z);
    if (rc != TFS_OK) return rc;
    TFS_CUDA(cudaMemcpyAsync(out, p->z, sizeof(double) * p->n, cudaMemcpyDeviceToHost, s->stream),
             "copy result");
  } else if (which == 2) {
    if ((rc = pres_rhs(s)) != TFS_OK) return rc;
    TFS_CUDA(cudaMemcpyAsync(out, p->b, sizeof(double) * p->n, cudaMemcpyDeviceToHost, s->stream),
             "copy result");
  } else {
    return fail(TFS_EINVAL, "which: 0 operator, 1 preconditioner, 2 right-hand side");
  }
  TFS_CUDA(cudaStreamSynchronize(s->stream), "prescribed apply");
  return TFS_OK;
}

int tfs_prescribed_precon_matrix(tfs_solver *s, double *m36) {
  int rc;
  if ((rc = pres_check(s)) != TFS_OK) return rc;
  if (m36 == nullptr) return fail(TFS_EINVAL, "null output");
  TFS_CUDA(cudaMemcpyAsync(m36, s->pres->m6inv, sizeof(double) * 36, cudaMemcpyDeviceToHost,
                           s->stream),
           "copy matrix");
  TFS_CUDA(cudaStreamSynchronize(s->stream), "copy matrix");
  return TFS_OK;
}

// The solution of the last solve (and the warm start of the next): segment
// forces (3 per segment), blob forces, body velocities, phase and angle
// rates; NULL skips a part, and parts the configuration lacks read as zero.
int tfs_prescribed_solution(tfs_solver *s, double *f_segs, double *f_blobs, double *v_body,
                            double *phase_dot, double *angle_dot) {
  int rc;
  if ((rc = pres_check(s)) != TFS_OK) return rc;
  PresState *p = s->pres;
  struct Part {
    double *dst;
    int off, n;
    bool present;
  } parts[] = {{f_segs, 0, 3 * p->ns, true},
               {f_blobs, 3 * p->ns, 3 * p->nb, true},
               {v_body, p->o_body, 6, p->free_body},
               {phase_dot, p->o_phase, p->nfil, p->phase},
               {angle_dot, p->o_angle, p->nfil, p->angle}};
  for (const Part &q : parts) {
    if (q.dst == nullptr || q.n == 0) continue;
    if (q.present)
      TFS_CUDA(cudaMemcpyAsync(q.dst, p->x + q.off, sizeof(double) * q.n, cudaMemcpyDeviceToHost,
                               s->stream),
               "copy solution");
    else
      std::memset(q.dst, 0, sizeof(double) * q.n);
  }
  TFS_CUDA(cudaStreamSynchronize(s->stream), "copy solution");
  return TFS_OK;
}

int tfs_prescribed_set_solution(tfs_solver *s, const double *f_segs, const double *f_blobs,
                                const double *v_body, const double *phase_dot,
                                const double *angle_dot) {
  int rc;
  if ((rc = pres_check(s)) != TFS_OK) return rc;
  PresState *p = s->pres;
  struct Part {
    const double *src;
    int off, n;
    bool present;
  } parts[] = {{f_segs, 0, 3 * p->ns, true},
               {f_blobs, 3 * p->ns, 3 * p->nb, true},
               {v_body, p->o_body, 6, p->free_body},
               {phase_dot, p->o_phase, p->nfil, p->phase},
               {angle_dot, p->o_angle, p->nfil, p->angle}};
  for (const Part &q : parts)
    if (q.src != nullptr && q.present && (rc = upload(s, p->x + q.off, q.src, q.n, "copy warm start")) != TFS_OK)
      return rc;
  TFS_CUDA(cudaStreamSynchronize(s->stream), "copy warm start");
  return TFS_OK;
}

}  // extern "C"
