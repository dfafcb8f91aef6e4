// gmres_persistent.cu -- the inner GMRES of the FP32C iterative refinement
// as one cooperative (persistent) kernel.
//
// Same system, preconditioner, Givens convention, warm-start tests and
// stopping rule as the multi-kernel GMRES of gmres.cu (the reference's
// solve_linear_system, mobility_solver.cpp:2092-2570, free-body branches),
// in mixed precision: the blob-blob product M_bb in FP32 (compensated per
// tile) and the Arnoldi vectors in FP32 -- the Krylov basis, the
// Gram-Schmidt dots and updates, norms, body sums and the preconditioner --
// with the Hessenberg matrix, Givens rotations, convergence test and
// triangular solve in FP64. The inner solve of the refinement asks for a
// 1e-4 reduction, and two Gram-Schmidt passes in FP32 keep the basis
// orthogonal to ~1e-7, so the FP32 vectors cost no accuracy the outer
// (float-float residual) loop needs; they take the FP64 pipe, at ~1/19 of
// the SM's issue rate on GB300, off every phase. At the medium swimmer
// (2 562 blobs) an Arnoldi step is ~10 us of arithmetic; issued as seven
// kernels per step it took ~150-190 us of launch gaps and serialised
// reductions. Here one launch runs the whole solve:
//
//   start | M_bb | residual | scale + preconditioner | { M_bb + Givens |
//   w, CGS pass-1 dots | h1, w -= Q h1, pass-2 dots, partials of w' |
//   h2, ||w''||, Q_k, z_k = P^-1 Q_k } x k | Q y | update
//
// with a grid barrier between phases (four per Arnoldi step), one CTA per
// SM; with a zero warm start (PgArgs::zero_start) the first M_bb and the
// residual are skipped (r0 = rhs). Every CTA owns a contiguous slice of
// blobs (its rows of every vector).
// Reductions are deterministic (per-CTA partials added in CTA order, fixed
// shuffle trees): the Gram-Schmidt coefficients, 6-vectors and squared norms,
// which every CTA needs at once, are summed by every CTA itself from the
// staged partials (identical bits everywhere); when k x G exceeds the staging
// buffers the coefficients are summed one per warp across the grid and read
// back after an extra barrier. The new vector's norm and body sums follow
// from the Pythagorean identity (||w''||^2 = ||w'||^2 - ||h2||^2, and the
// stored sums of earlier vectors), so no barrier separates them from the
// second pass. Givens rotations, the convergence test and the final
// triangular solve run in CTA 0 while the others start the next M_bb; CTA 0
// publishes its decision for the others to read after the next barrier.
// The M_bb product is cut into (target block x source split) units spread
// over all CTAs (a target whose only pair inside contact in a tile is its own
// blob adds the r = 0 term directly); partial sums go to global memory and
// each row's owner adds the splits in order. One launch may carry several
// independent solves (PgArgs array + CTA map), each on its own CTAs.
//
// Grid barrier: one monotonic arrival counter per solve in global memory
// (the e-th barrier passes at e x P arrivals). Every wait is bounded (2 s of
// globaltimer, plus an iteration cap); a CTA that gives up raises an abort
// word that ends every other wait at once, and the solve reports
// TFS_ETIMEOUT. The launch is cooperative, so all CTAs are resident together
// (or the launch fails and the multi-kernel path runs). Data other CTAs wrote
// is read with ld.global.cg (L2), never through L1.
#include <cuda_runtime.h>

#include <algorithm>

#include "gmres.h"
#include "rpy_tile.cuh"
#include "tfs_kernels.h"

namespace tfs {

namespace {

constexpr int kPB = 512;       // threads per CTA (one CTA per SM)
constexpr int kPW = kPB / 32;  // warps per CTA
constexpr int kPTS = 128;      // sources per shared-memory tile of M_bb
constexpr int kPK = 352;       // Krylov columns + 1 (max_iter <= 350)
constexpr int kMaxRows = 3 * kMaxPgBlobsPerCta;
constexpr int kHB = 4096;      // doubles of the staging buffer (H columns, M_bb partials)

// bytes of dynamic shared memory before the resident Krylov rows (vectors of V)
template <typename V>
constexpr size_t pg_dyn_fixed() {
  return 8 * (size_t)kHB + sizeof(V) * (8 * (size_t)kMaxPgCtas + 12 * kPK);
}

// control words CTA 0 publishes each Arnoldi step
enum { C_FINISH = 0, C_REL, C_STATUS, kCtl };

// p6 slots: per-CTA partial 6-vectors sum_m (l_m ; d_m x l_m)
enum { K_SOLN = 0, K_R0, K_RHS, K_Z, K_W, K_T, kP6Slots };
// ps slots: per-CTA partial sums of squares
enum { S_RHS = 0, S_R0, S_NORM, kPsSlots };

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ double ldcg(const double *p) { return __ldcg(p); }

// 1 / sqrt(x) of a Krylov vector's squared norm: the refined FP32 estimate
// (a few ulp) for FP64 vectors, the hardware approximation for FP32 ones.
__device__ __forceinline__ double vrsqrt(double x) { return rsqrt_far(x); }
__device__ __forceinline__ float vrsqrt(float x) { return rsqrtf(x); }

// Phase trace of the Arnoldi steps (builds with -DTFS_PG_TRACE only):
// globaltimer stamps of thread 0 of CTAs 0 and 1 at eight points of every
// step k, [cta][k][phase]: 0 step start (M_bb begins; CTA 0 meanwhile runs
// the Givens step), 1 after the barrier that ends M_bb, 2 w = A z formed,
// 3 after the barrier of the first-pass dots, 4 h1 summed, 5 after the
// barrier of the second-pass dots and partials, 6 h2 summed, 7 Q_k, z_k and
// the records done (the step's last barrier follows). The last solve of a
// launch leaves its trace; tfs_pg_trace reads it.
#ifdef TFS_PG_TRACE
constexpr int kTraceSteps = 352, kTracePhases = 8;
__device__ unsigned long long g_pg_trace[2][kTraceSteps][kTracePhases];
#define PG_STAMP(kk, ph)                                                   \
  do {                                                                     \
    if (p.rank < 2 && threadIdx.x == 0 && (kk) < kTraceSteps)              \
      g_pg_trace[p.rank][(kk)][(ph)] = global_ns();                        \
  } while (0)
#else
#define PG_STAMP(kk, ph) \
  do {                   \
  } while (0)
#endif

// Release-add to and acquire-load of a barrier word at GPU scope.
__device__ __forceinline__ void red_release(unsigned *w, unsigned v) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(w), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned ld_acquire(const unsigned *w) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(w) : "memory");
  return v;
}

// Bounded grid barrier; false in every thread of the CTA if it was abandoned.
// bar[0] counts arrivals over the whole launch (zeroed before it): the e-th
// barrier of a solve is passed once it reaches e * P, so no CTA has to reset
// it (each CTA keeps its own count e in *epoch, shared memory). bar[2] is
// the abort word. After the CTA barrier, thread 0 arrives with a release
// reduction (cumulative: it orders every write the CTA made before the CTA
// barrier) and polls with acquire loads, so the CTA's later reads see what
// every CTA wrote before arriving; those reads bypass L1 (ld.global.cg)
// wherever they read other CTAs' data.
__device__ bool pg_barrier(const PgArgs &p, unsigned *epoch) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned *vb = p.bar;
    int good = 1;
    const unsigned target = (*epoch + 1u) * ((unsigned)p.P + p.bar_extra);
    *epoch += 1u;
    red_release(p.bar, 1u);
    const unsigned long long t0 = global_ns();
    unsigned spins = 0;
    while (ld_acquire(p.bar) < target) {
      ++spins;
      if ((spins & 15u) == 0u && vb[2] != 0u) {  // another CTA gave up
        good = 0;
        break;
      }
      if (spins > (1u << 25) || ((spins & 63u) == 0 && global_ns() - t0 > kPgTimeoutNs)) {
        atomicExch(p.bar + 2, 1u);
        good = 0;
        break;
      }
    }
    if (!good) {
      atomicExch(&p.g.st->status, 2);
      atomicExch(&p.g.st->done, 1);
    }
    ok = good;
  }
  __syncthreads();
  return ok != 0;
}

template <typename V>
struct PSlice {
  int m0, m1;       // blobs [m0, m1)
  int rows;         // 3 (m1 - m0)
  bool owner;       // this CTA owns a slice (rank < G)
  bool body;        // this CTA writes the six body rows of global vectors
  const V *d;       // the slice's d_m = R ref_m, d[3 (m - m0) + j] (shared memory)
};

template <typename V>
__device__ __forceinline__ PSlice<V> pg_slice(const PgArgs &p, const V *dsl) {
  PSlice<V> s;
  s.d = dsl;
  const int c = p.rank;
  s.owner = c < p.g.G;
  s.m0 = s.owner ? min(p.g.nb, c * p.g.blobs_per_cta) : p.g.nb;
  s.m1 = s.owner ? min(p.g.nb, s.m0 + p.g.blobs_per_cta) : p.g.nb;
  s.rows = 3 * (s.m1 - s.m0);
  s.body = c == p.g.G - 1;
  return s;
}

// Warp sum with a fixed shuffle pattern (the same bits in every lane).
template <typename V>
__device__ __forceinline__ V warp_sum(V v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Stage elems floats of buf (global) into dst (shared), eight loads in
// flight per thread; no barrier.
template <typename V>
__device__ __forceinline__ void stage(const V *buf, int elems, V *dst) {
  for (int q0 = 0; q0 < elems; q0 += 8 * kPB) {
    V v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int q = q0 + u * kPB + (int)threadIdx.x;
      v[u] = q < elems ? __ldcg(buf + q) : V(0);
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int q = q0 + u * kPB + (int)threadIdx.x;
      if (q < elems) dst[q] = v[u];
    }
  }
}

// Stage the slice's rows of the S split products (mpart, (hi, lo) FP32
// pairs) into dst[sp * rows + r], eight loads in flight per thread; no barrier.
template <typename V>
__device__ __forceinline__ void stage_splits(const PgArgs &p, const PSlice<V> &sl, float2 *dst) {
  const int rows = sl.rows, tot = p.S * rows, nb = p.g.nb;
  for (int q0 = 0; q0 < tot; q0 += 8 * kPB) {
    float2 v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int q = q0 + u * kPB + (int)threadIdx.x;
      const int sp = q / max(rows, 1), r = q - sp * rows;
      v[u] = q < tot ? __ldcg(p.mpart + ((size_t)sp * nb + sl.m0) * 3 + r) : make_float2(0.f, 0.f);
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int q = q0 + u * kPB + (int)threadIdx.x;
      if (q < tot) dst[q] = v[u];
    }
  }
}

// out[j] = sum over c < G of cst[j * G + c], j < count <= kPW: warp j adds
// lane-strided subsets then a fixed shuffle tree. No barrier.
template <typename V>
__device__ __forceinline__ void sum_staged(const V *cst, int G, int count, V *out) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (wid < count) {
    V s = V(0);
    for (int c = lane; c < G; c += 32) s += cst[wid * G + c];
    s = warp_sum(s);
    if (lane == 0) out[wid] = s;
  }
}

// Stage and sum count vectors of per-CTA partials (buf[j * G + c]) into
// out[0..count); ends with a barrier.
template <typename V>
__device__ void cta_sums(const V *buf, int G, int count, V *out, V *cst) {
  stage(buf, count * G, cst);
  __syncthreads();
  sum_staged(cst, G, count, out);
  __syncthreads();
}

// This CTA's partials of the slice rows ls: warp j < 6 sums component j of
// sum_m (l_m ; d_m x l_m) into p6 slot kt_slot and, with sq_slot >= 0, warp
// 6 the sum of squares into ps slot sq_slot (lanes stride over blobs or
// rows, then a fixed shuffle tree). No barrier; ls must be complete.
template <typename V>
__device__ void slice_partials(const PgArgs &p, const PSlice<V> &sl, const V *ls, int kt_slot,
                               int sq_slot) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (!sl.owner || wid >= (sq_slot >= 0 ? 7 : 6)) return;
  V s = V(0);
  if (wid < 3) {
    for (int m = sl.m0 + lane; m < sl.m1; m += 32) s += ls[3 * (m - sl.m0) + wid];
  } else if (wid < 6) {  // (d x l)_j = d_a l_b - d_b l_a, (a, b) = (j + 1, j + 2) mod 3
    const int a = (wid - 2) % 3, b = (wid - 1) % 3;
    for (int m = sl.m0 + lane; m < sl.m1; m += 32) {
      const V *d = sl.d + 3 * (m - sl.m0);
      const V *v = ls + 3 * (m - sl.m0);
      s += d[a] * v[b] - d[b] * v[a];
    }
  } else {
    for (int r = lane; r < sl.rows; r += 32) s += ls[r] * ls[r];
  }
  s = warp_sum(s);
  if (lane == 0) {
    const int G = p.g.G, c = p.rank;
    if (wid < 6) reinterpret_cast<V *>(p.p6)[(size_t)(kt_slot * 6 + wid) * G + c] = s;
    else reinterpret_cast<V *>(p.ps)[(size_t)sq_slot * G + c] = s;
  }
}

// z = P^-1 (q rows of the slice in shared memory, q_vel), given
// bsum = sum_m (q_m ; d_m x q_m) / bscale: b = -bsum * bscale, the body part
// (U', Omega') = KTKinv b - N q_vel (mobility_solver.cpp:1437-1509), then
// z_m = 6 pi mu a (q_m + U' + Omega' x d_m). Writes zv (6, shared) and the
// slice's z rows into zs (shared); ends with a barrier.
template <typename V>
__device__ void precond(const PgArgs &p, const PSlice<V> &sl, const V *qs, const V *qvel,
                        const V *bsum, V bscale, V *zs, V *zv, const V *mats) {
  if (threadIdx.x < 6) {
    const int i = threadIdx.x;
    const V *N = mats, *Kinv = mats + 36;
    V t1 = V(0), t2 = V(0);
    V u1 = V(0), u2 = V(0);
    for (int k = 0; k < 6; k += 2) {
      t1 += Kinv[i + 6 * k] * (-bsum[k] * bscale);
      u1 += Kinv[i + 6 * (k + 1)] * (-bsum[k + 1] * bscale);
      t2 += N[i + 6 * k] * qvel[k];
      u2 += N[i + 6 * (k + 1)] * qvel[k + 1];
    }
    zv[i] = (t1 + u1) - (t2 + u2);
  }
  __syncthreads();
  const V u0 = zv[0], u1 = zv[1], u2 = zv[2], w0 = zv[3], w1 = zv[4], w2 = zv[5];
  const V minv = V(p.minv);
  for (int m = sl.m0 + threadIdx.x; m < sl.m1; m += kPB) {
    const V *d = sl.d + 3 * (m - sl.m0);
    const V *l = qs + 3 * (m - sl.m0);
    V b0 = l[0] + u0, b1 = l[1] + u1, b2 = l[2] + u2;
    b0 += w1 * d[2] - w2 * d[1];
    b1 += w2 * d[0] - w0 * d[2];
    b2 += w0 * d[1] - w1 * d[0];
    V *o = zs + 3 * (m - sl.m0);
    o[0] = minv * b0;
    o[1] = minv * b1;
    o[2] = minv * b2;
  }
  __syncthreads();
}

// FP32 source records {x - origin, f, 0, 0} of the slice's blobs for M_bb.
template <typename V>
__device__ void pack_records(const PgArgs &p, const PSlice<V> &sl, const V *fs) {
  for (int m = sl.m0 + threadIdx.x; m < sl.m1; m += kPB) {
    const V *f = fs + 3 * (m - sl.m0);
    float4 a, b;
    a.x = p.x32[3 * (size_t)m];
    a.y = p.x32[3 * (size_t)m + 1];
    a.z = p.x32[3 * (size_t)m + 2];
    a.w = float(f[0]);
    b.x = float(f[1]);
    b.y = float(f[2]);
    b.z = 0.f;
    b.w = 0.f;
    float4 *r = reinterpret_cast<float4 *>(p.rec + 8 * (size_t)m);
    r[0] = a;
    r[1] = b;
  }
}

// One staged tile of M_bb for the NT targets of this thread (NT = 1 in a
// warp where no lane has a second target), FP32 pairs; the tile's sum is
// added compensated into (hi, lo).
template <int NT>
__device__ __forceinline__ void mbb_tile(const float (&xt)[2], const float (&yt)[2],
                                         const float (&zt)[2], const int (&i)[2], int base,
                                         int cnt, const float *src, const PairConst<float> &pc,
                                         float (&hi)[2][3], float (&lo)[2][3]) {
  float x[NT], y[NT], z[NT], v[NT][3];
  unsigned nf[NT];  // pairs inside the contact distance
#pragma unroll
  for (int t = 0; t < NT; ++t) {
    x[t] = xt[t];
    y[t] = yt[t];
    z[t] = zt[t];
    nf[t] = 0u;
#pragma unroll
    for (int k = 0; k < 3; ++k) v[t][k] = 0.f;
  }
#pragma unroll 2
  for (int j = 0; j < cnt; ++j) {
    float sx, sy, sz, f[3];
    RecLoad<float, 3>::get(src + 8 * j, sx, sy, sz, f);
#pragma unroll
    for (int t = 0; t < NT; ++t) {
      const float dx = x[t] - sx, dy = y[t] - sy, dz = z[t] - sz;
      const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
      const bool far = r2 > pc.asum2;
      nf[t] += far ? 0u : 1u;
      const float rs = rsqrt_far(r2);
      far_pair<float, 3, 3>(v[t], dx, dy, dz, far ? rs : 0.f, f, pc);
    }
  }
  // a target whose only pair inside the contact distance in this tile is
  // its own blob (r = 0) takes the self term 4/(3a) F here (the nested
  // branch of the pair function at r = 0); targets with any other such
  // pair rescan the tile with the full formula, self pair included
#pragma unroll
  for (int t = 0; t < NT; ++t) {
    const int js = i[t] - base;
    const unsigned self_in = (js >= 0 && js < cnt) ? 1u : 0u;
    if (nf[t] == self_in) {
      if (self_in) {
        float sx, sy, sz, f[3];
        RecLoad<float, 3>::get(src + 8 * js, sx, sy, sz, f);
        const float A = 4.f / (3.f * pc.ai);
#pragma unroll
        for (int k = 0; k < 3; ++k) v[t][k] += A * f[k];
      }
      nf[t] = 0u;
    }
  }
  unsigned any = 0u;
#pragma unroll
  for (int t = 0; t < NT; ++t) any |= nf[t];
  if (__any_sync(0xffffffffu, any != 0u)) near_pass<float, 3, 3, NT>(v, x, y, z, nf, src, cnt, pc);
#pragma unroll
  for (int t = 0; t < NT; ++t)
#pragma unroll
    for (int k = 0; k < 3; ++k) two_sum(hi[t][k], lo[t][k], v[t][k]);
}

// M_bb of the packed records: (target block x source split) units over the
// CTAs other than CTA 0 (which meanwhile runs the Givens step), up to two
// targets per thread (warps whose lanes all have one take the one-target
// pass), FP32 pairs, per-tile compensated sums; each split's sum is written
// as its (hi, lo) FP32 pair mpart[(split * nb + target) * 3 + k] (the
// consumer adds the splits compensated and scales by 1 / (8 pi mu)).
__device__ void mbb_units(const PgArgs &p, float *src) {
  const int nb = p.g.nb;
  const int units = p.TB * p.S;
  const int first = p.P > 1 ? 1 : 0, workers = p.P - first;
  if (p.rank < first) return;
  PairConst<float> pc;
  pc.ai = p.a;
  pc.aj = p.a;
  pc.asum2 = p.pc_asum2;
  pc.s = p.pc_s;
  pc.s3 = p.pc_s3;
  for (int u = p.rank - first; u < units; u += workers) {
    const int tb = u / p.S, sp = u - tb * p.S;
    const int t0 = tb * p.tbs, t1 = min(nb, t0 + p.tbs);
    const int s0 = sp * p.chunk, s1 = min(nb, s0 + p.chunk);
    if (t0 >= t1 || s0 >= s1) continue;  // CTA-uniform
    int i[2];
    bool act[2];
    float xt[2], yt[2], zt[2], hi[2][3], lo[2][3];
#pragma unroll
    for (int t = 0; t < 2; ++t) {
      i[t] = t0 + (int)threadIdx.x + t * kPB;
      act[t] = i[t] < t1;
      if (!act[t]) i[t] = t1 - 1;
      xt[t] = __ldcg(p.x32 + 3 * (size_t)i[t]);
      yt[t] = __ldcg(p.x32 + 3 * (size_t)i[t] + 1);
      zt[t] = __ldcg(p.x32 + 3 * (size_t)i[t] + 2);
#pragma unroll
      for (int k = 0; k < 3; ++k) hi[t][k] = lo[t][k] = 0.f;
    }
    const bool warp_active = __any_sync(0xffffffffu, act[0] || act[1]);
    const bool two = __any_sync(0xffffffffu, act[1]);
    for (int base = s0; base < s1; base += kPTS) {
      const int cnt = min(kPTS, s1 - base);
      __syncthreads();
      const float4 *g = reinterpret_cast<const float4 *>(p.rec + 8 * (size_t)base);
      float4 *d = reinterpret_cast<float4 *>(src);
      for (int q = threadIdx.x; q < 2 * cnt; q += kPB) d[q] = __ldcg(g + q);
      __syncthreads();
      if (!warp_active) continue;
      if (two) mbb_tile<2>(xt, yt, zt, i, base, cnt, src, pc, hi, lo);
      else mbb_tile<1>(xt, yt, zt, i, base, cnt, src, pc, hi, lo);
    }
#pragma unroll
    for (int t = 0; t < 2; ++t) {
      if (!act[t]) continue;
      float2 *o = p.mpart + ((size_t)sp * nb + i[t]) * 3;
#pragma unroll
      for (int k = 0; k < 3; ++k) o[k] = make_float2(hi[t][k], lo[t][k]);
    }
  }
}

// ws (slice rows) = M_bb z - (U + Omega x d_m) with v = sum over splits of
// the partial products (in split order, (hi, lo) row sums in acc), (U, Omega)
// = zv. The slice's partials are staged through stage (kHB doubles) with
// parallel loads.
template <typename V>
__device__ void apply_rows(const PgArgs &p, const PSlice<V> &sl, const V *zv, V *ws,
                           double *stage, float2 *acc) {
  const int nb = p.g.nb, rows = sl.rows;
  const int per = rows > 0 ? max(1, kHB / rows) : 1;  // splits per staging round
  float2 *st2 = reinterpret_cast<float2 *>(stage);
  for (int r = threadIdx.x; r < rows; r += kPB) acc[r] = make_float2(0.f, 0.f);
  for (int s0 = 0; s0 < p.S; s0 += per) {
    const int s1 = min(p.S, s0 + per);
    __syncthreads();
    for (int q = threadIdx.x; q < (s1 - s0) * rows; q += kPB) {
      const int s = s0 + q / rows, r = q - (q / rows) * rows;
      st2[q] = __ldcg(p.mpart + ((size_t)s * nb + sl.m0) * 3 + r);
    }
    __syncthreads();
    for (int r = threadIdx.x; r < rows; r += kPB) {
      float h = acc[r].x, l = acc[r].y;
      for (int s = 0; s < s1 - s0; ++s) {
        two_sum(h, l, st2[s * rows + r].x);
        l += st2[s * rows + r].y;
      }
      acc[r] = make_float2(h, l);
    }
  }
  __syncthreads();
  const V scale = V(p.scale);
  for (int r = threadIdx.x; r < rows; r += kPB) {
    const int m = sl.m0 + r / 3, j = r - 3 * (r / 3);
    const V *d = sl.d + 3 * (m - sl.m0);
    V body;
    if (j == 0) body = zv[0] - d[1] * zv[5] + d[2] * zv[4];
    else if (j == 1) body = zv[1] - d[2] * zv[3] + d[0] * zv[5];
    else body = zv[2] - d[0] * zv[4] + d[1] * zv[3];
    ws[r] = -body + scale * (V(acc[r].x) + V(acc[r].y));
  }
  __syncthreads();
}

// The Krylov basis in global memory, FP32: row r of vector i at
// [i n + r] of the (FP64-sized) basis buffer.
template <typename V>
__device__ __forceinline__ V *qglobal(const PgArgs &p) {
  return reinterpret_cast<V *>(p.g.Q);
}

// Row r of the slice's Krylov vector i: from the CTA's resident copy
// (columns i < Kr, shared memory) or from global memory.
template <typename V>
__device__ __forceinline__ V qrow(const PgArgs &p, const PSlice<V> &sl, const V *qres, int i,
                                      int r) {
  return i < p.Kr ? qres[(size_t)i * sl.rows + r]
                  : __ldcg(qglobal<V>(p) + (size_t)i * p.g.n + 3 * (size_t)sl.m0 + r);
}

// Store the slice rows ws as Krylov vector i (resident copy, or global
// memory beyond the resident columns).
template <typename V>
__device__ void store_q(const PgArgs &p, const PSlice<V> &sl, V *qres, int i, const V *ws) {
  for (int r = threadIdx.x; r < sl.rows; r += kPB) {
    if (i < p.Kr) qres[(size_t)i * sl.rows + r] = ws[r];
    else qglobal<V>(p)[(size_t)i * p.g.n + 3 * (size_t)sl.m0 + r] = ws[r];
  }
}

// dots of the slice rows ws with Q_i, i < k, into pd[i * G + c]: tpi
// adjacent threads per i (16, 8 or 4 as k allows one pass; four per pass
// beyond), rows r = part (mod tpi), then a fixed shuffle tree.
template <typename V>
__device__ void slice_dots(const PgArgs &p, const PSlice<V> &sl, const V *ws, int k, V *pd,
                           const V *qres) {
  if (!sl.owner) return;
  const int tpi = k <= kPB / 16 ? 16 : k <= kPB / 8 ? 8 : 4;
  const int part = threadIdx.x & (tpi - 1);
  for (int i0 = 0; i0 < k; i0 += kPB / tpi) {
    const int i = i0 + (int)threadIdx.x / tpi;
    V s = V(0), u = V(0);
    if (i < k) {
      int r = part;
      if (i < p.Kr) {
        const V *q = qres + (size_t)i * sl.rows;
        for (; r + tpi < sl.rows; r += 2 * tpi) {
          s += ws[r] * q[r];
          u += ws[r + tpi] * q[r + tpi];
        }
        if (r < sl.rows) s += ws[r] * q[r];
      } else {
        for (; r < sl.rows; r += tpi) s += ws[r] * qrow(p, sl, qres, i, r);
      }
    }
    s += u;
    for (int o = 1; o < tpi; o <<= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (i < k && part == 0) pd[(size_t)i * p.g.G + p.rank] = s;
  }
}

// ws (slice rows) += sign * sum_{i<k} h_i Q_i: four adjacent threads per row
// (when the rows allow), each over i = sub (mod 4) with two running sums,
// then a fixed shuffle tree; one thread per row with four sums otherwise.
template <typename V>
__device__ void slice_axpy(const PgArgs &p, const PSlice<V> &sl, const V *h, int k, V *ws,
                           V sign, const V *qres) {
  if (4 * sl.rows <= kPB) {
    const int r = threadIdx.x >> 2, sub = threadIdx.x & 3;
    V t = V(0), u = V(0);
    if (r < sl.rows) {
      int i = sub;
      for (; i + 4 < k; i += 8) {
        t += h[i] * qrow(p, sl, qres, i, r);
        u += h[i + 4] * qrow(p, sl, qres, i + 4, r);
      }
      if (i < k) t += h[i] * qrow(p, sl, qres, i, r);
    }
    t += u;
    t += __shfl_xor_sync(0xffffffffu, t, 1);
    t += __shfl_xor_sync(0xffffffffu, t, 2);
    if (r < sl.rows && sub == 0) ws[r] += sign * t;
  } else {
    for (int r = threadIdx.x; r < sl.rows; r += kPB) {
      V t[4] = {V(0), V(0), V(0), V(0)};
      int i = 0;
      for (; i + 3 < k; i += 4)
#pragma unroll
        for (int u = 0; u < 4; ++u) t[u] += h[i + u] * qrow(p, sl, qres, i + u, r);
      for (; i < k; ++i) t[0] += h[i] * qrow(p, sl, qres, i, r);
      ws[r] += sign * ((t[0] + t[1]) + (t[2] + t[3]));
    }
  }
  __syncthreads();
}

// v[l] += sign * sum_{i<k} h_i Q_i,vel(l): warp l < 6, lanes over i, fixed
// tree; the body rows of every Krylov vector are resident in qvres[6 i + l].
template <typename V>
__device__ void vel_axpy(const V *qvres, const V *h, int k, V *v, V sign) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (wid < 6) {
    V s = V(0);
    for (int i = lane; i < k; i += 32) s += h[i] * qvres[6 * i + wid];
    s = warp_sum(s);
    if (lane == 0) v[wid] += sign * s;
  }
  __syncthreads();
}

// Gram-Schmidt coefficients, spread over the grid: warp w of CTA c sums
// h_j = sum_c' pd[j * G + c'] + w_vel . Q_j,vel for j = c + P (w + kPW t),
// into hg[j] (global); lanes l < 6 start from the body term w_vel,l Q_j,vel(l),
// lanes stride over c', then a fixed shuffle tree.
template <typename V>
__device__ void reduce_dots(const PgArgs &p, const V *pd, int k, const V *wv,
                            const V *qvres, V *hg) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int G = p.g.G;
  for (int j = p.rank + p.P * wid; j < k; j += p.P * kPW) {
    V s = lane < 6 ? wv[lane] * qvres[6 * j + lane] : V(0);
    for (int c = lane; c < G; c += 32) s += __ldcg(pd + (size_t)j * G + c);
    s = warp_sum(s);
    if (lane == 0) hg[j] = s;
  }
}

// The same sums as reduce_dots, h[j] for j < k into shared memory, in every
// CTA (identical bits: the same order), when the k x G partials fit the
// staging buffers stg (hb and the partial-sum staging after it): false, with
// nothing done, otherwise. The partials are staged with eight
// loads in flight per thread. Ends with a barrier.
template <typename V>
__device__ bool local_dots(const PgArgs &p, const V *pd, int k, const V *wv,
                           const V *qvres, V *h, V *stg) {
  const int G = p.g.G, tot = k * G;
  if (tot > kHB * (int)(sizeof(double) / sizeof(V)) + 8 * kMaxPgCtas) return false;
  for (int q0 = 0; q0 < tot; q0 += 8 * kPB) {
    V v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int q = q0 + u * kPB + (int)threadIdx.x;
      v[u] = q < tot ? __ldcg(pd + q) : V(0);
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int q = q0 + u * kPB + (int)threadIdx.x;
      if (q < tot) stg[q] = v[u];
    }
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int j = wid; j < k; j += kPW) {
    V s = lane < 6 ? wv[lane] * qvres[6 * j + lane] : V(0);
    for (int c = lane; c < G; c += 32) s += stg[(size_t)j * G + c];
    s = warp_sum(s);
    if (lane == 0) h[j] = s;
  }
  __syncthreads();
  return true;
}

// Givens rotations of the new Hessenberg column (mobility_solver.cpp:
// 2370-2413): hcol[0..k] in, rotated in place; updates cs, sn, beta;
// returns |beta_k| / norm_rhs. One thread.
__device__ double givens_step(int k, double *hcol, double *cs, double *sn, double *beta,
                              double norm_rhs) {
  for (int i = 1; i < k; ++i) {
    const double tt = cs[i - 1] * hcol[i - 1] + sn[i - 1] * hcol[i];
    hcol[i] = cs[i - 1] * hcol[i] - sn[i - 1] * hcol[i - 1];
    hcol[i - 1] = tt;
  }
  const double hd = hcol[k - 1], hs = hcol[k];
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
  hcol[k - 1] = cs[k - 1] * hd + sn[k - 1] * hs;
  hcol[k] = 0.0;
  beta[k] = -sn[k - 1] * beta[k - 1];
  beta[k - 1] = cs[k - 1] * beta[k - 1];
  return fabs(beta[k]) / norm_rhs;
}

// y = H^-1 beta (:2419-2438) in yv (shared), by the whole CTA: columns
// j < k - 1 of H staged from global memory into hb (kHB doubles) in chunks,
// column k - 1 from hcol; warp 0 substitutes column by column.
__device__ void back_substitute(const PgArgs &p, int k, const double *hcol, const double *beta,
                                double *yv, double *hb) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int ld = p.g.max_iter + 1;
  for (int i = threadIdx.x; i < k; i += kPB) yv[i] = beta[i];
  int jhi = k - 1;
  while (jhi >= 0) {
    // columns jhi, jhi-1, ..., jlo (rows 0..j each) fit in hb
    int jlo = jhi, used = jhi + 1;
    while (jlo > 0 && used + jlo <= kHB) {
      used += jlo;
      --jlo;
    }
    __syncthreads();
    int off = 0;
    for (int j = jhi; j >= jlo; --j) {
      for (int i = threadIdx.x; i <= j; i += kPB)
        hb[off + i] = (j == k - 1) ? hcol[i] : ldcg(p.g.H + i + (size_t)j * ld);
      off += j + 1;
    }
    __syncthreads();
    if (wid == 0) {
      off = 0;
      for (int j = jhi; j >= jlo; --j) {
        const double yj = yv[j] / hb[off + j];
        __syncwarp();
        for (int i = lane; i < j; i += 32) yv[i] -= hb[off + i] * yj;
        __syncwarp();
        if (lane == 0) yv[j] = yj;
        __syncwarp();
        off += j + 1;
      }
    }
    jhi = jlo - 1;
  }
  __syncthreads();
}

}  // namespace

template <typename V>
__global__ void __launch_bounds__(kPB, 1) gmres_persistent_kernel(const PgArgs *__restrict__ gp,
                                                                  const int2 *__restrict__ cmap) {
  // this CTA's solve (several independent solves may share one launch, each
  // on its own CTAs with its own barrier words)
  __shared__ PgArgs pshared;
  if (threadIdx.x == 0) {
    const int2 m = cmap[blockIdx.x];
    pshared = gp[m.x];
    pshared.rank = m.y;
  }
  __syncthreads();
  const PgArgs &p = pshared;
  __shared__ unsigned epoch;  // grid barriers passed (thread 0)
  if (threadIdx.x == 0) epoch = 0u;
  __shared__ __align__(16) float src[8 * kPTS];
  __shared__ V ws[kMaxRows];        // w (then Q_k, tmp) rows of the slice
  __shared__ V zs[kMaxRows];        // z = P^-1 q rows of the slice
  __shared__ float2 acc[kMaxRows];  // (hi, lo) row sums of the M_bb splits
  __shared__ V h1[kPK], h2[kPK], yf[kPK];
  __shared__ double cs[kPK], sn[kPK], beta[kPK], hcol[kPK], yv[kPK];
  __shared__ double tmp8[8];
  __shared__ V tf[8];
  __shared__ V wvel[6], qvel[6], zv[6], wsum6[6];
  __shared__ V dsl[kMaxRows], mats[72], qn_s[2];
  // dynamic: staging buffer (kHB doubles), then of the vector type: staged
  // per-CTA partials (8 x kMaxPgCtas), body rows of every Krylov vector
  // (6 x kPK), sum_m (Q_i,m ; d_m x Q_i,m) of every Krylov vector (6 x kPK),
  // resident Krylov rows (Kr x rows)
  extern __shared__ double dyn[];
  double *hb = dyn;
  V *cst = reinterpret_cast<V *>(hb + kHB), *qvres = cst + 8 * kMaxPgCtas,
    *qsres = qvres + 6 * kPK, *qres = qsres + 6 * kPK;
  // per-CTA partials in the vector type
  V *p6 = reinterpret_cast<V *>(p.p6), *ps = reinterpret_cast<V *>(p.ps);
  V *pd1 = reinterpret_cast<V *>(p.pd1), *pd2 = reinterpret_cast<V *>(p.pd2);

  const GmresArgs &g = p.g;
  GmresScalars *st = g.st;
  const PSlice sl = pg_slice(p, dsl);
  const int nb = g.nb, vel = 3 * nb, G = g.G;
  const V scale = V(p.scale);

  // ---- start: the slice's d_m and the body matrices into shared memory,
  //      warm start into soln, FP32 targets, records, ||rhs|| partials
  for (int r = threadIdx.x; r < sl.rows; r += kPB) dsl[r] = V(g.diff[3 * (size_t)sl.m0 + r]);
  for (int q = threadIdx.x; q < 72; q += kPB) mats[q] = V(g.mats[q]);
  for (int r = threadIdx.x; r < sl.rows; r += kPB) {
    const int t = 3 * sl.m0 + r;
    const double x0 = g.f_blobs[t];
    g.soln[t] = x0;
    ws[r] = V(x0);
    zs[r] = V(g.rhs[t]);
  }
  for (int m = sl.m0 + threadIdx.x; m < sl.m1; m += kPB)
    for (int k = 0; k < 3; ++k)
      p.x32[3 * (size_t)m + k] = float(g.x_blobs[3 * (size_t)m + k] - g.origin[k]);
  if (sl.body && threadIdx.x < 6) g.soln[vel + threadIdx.x] = g.v_bodies[threadIdx.x];
  __syncthreads();
  if (!p.zero_start) pack_records(p, sl, ws);
  slice_partials(p, sl, zs, K_RHS, S_RHS);
  slice_partials(p, sl, ws, K_SOLN, -1);
  if (!pg_barrier(p, &epoch)) return;

  // the residual's slots: r0 = rhs with a zero warm start (A 0 = 0: its
  // M_bb, the residual pass and two barriers are skipped)
  const int k_r0 = p.zero_start ? K_RHS : K_R0, s_r0 = p.zero_start ? S_RHS : S_R0;
  if (p.zero_start) {
    for (int r = threadIdx.x; r < sl.rows; r += kPB) ws[r] = zs[r];
    __syncthreads();
  } else {
    // ---- M_bb of the warm start
    mbb_units(p, src);
    if (!pg_barrier(p, &epoch)) return;

    // ---- residual r0 = rhs - A soln (slice rows), partials
    if (threadIdx.x < 6) zv[threadIdx.x] = V(g.v_bodies[threadIdx.x]);
    __syncthreads();
    apply_rows(p, sl, zv, ws, hb, acc);  // ws = A soln (blob rows)
    for (int r = threadIdx.x; r < sl.rows; r += kPB) ws[r] = zs[r] - ws[r];  // zs = rhs rows
    __syncthreads();
    slice_partials(p, sl, ws, K_R0, S_R0);
    if (!pg_barrier(p, &epoch)) return;
  }

  // ---- beta_0, warm-start tests (mobility_solver.cpp:2279-2320), Q_0,
  //      preconditioner of Q_0, records (every CTA decides the same)
  double norm_rhs;
  {
    cta_sums(ps + (size_t)S_RHS * G, G, 1, tf, cst);
    double rhs_vel[6], t = tf[0];
    for (int j = 0; j < 6; ++j) {
      rhs_vel[j] = g.rhs[vel + j];
      t += rhs_vel[j] * rhs_vel[j];
    }
    norm_rhs = sqrt(t);
    cta_sums(p6 + (size_t)K_SOLN * 6 * G, G, 6, tf, cst);
    double r0v[6];
    for (int j = 0; j < 6; ++j) r0v[j] = rhs_vel[j] - (-(double)tf[j]);
    __syncthreads();
    cta_sums(ps + (size_t)s_r0 * G, G, 1, tf, cst);
    double bb = tf[0];
    for (int j = 0; j < 6; ++j) bb += r0v[j] * r0v[j];
    double beta0 = sqrt(bb);
    int flag = 0;
    if (norm_rhs == 0.0) flag = 3;
    else if (fabs(beta0) <= g.tol * norm_rhs) flag = 1;
    else if (fabs(beta0) > norm_rhs) {
      flag = 2;
      beta0 = norm_rhs;
    }
    __syncthreads();
    if (flag == 1 || flag == 3) {
      if (flag == 3) {
        for (int r = threadIdx.x; r < sl.rows; r += kPB) g.f_blobs[3 * sl.m0 + r] = 0.0;
        if (sl.body && threadIdx.x < 6) g.v_bodies[threadIdx.x] = 0.0;
      }
      if (p.rank == 0 && threadIdx.x == 0) {
        st->norm_rhs = norm_rhs;
        st->flag = flag;
        st->iters = 0;
        st->rel = 0.0;
        st->status = 0;
        st->done = 1;
      }
      return;
    }
    // Q_0: r0 / beta0, or rhs / ||rhs|| with a zero start (flag 2)
    int kslot;
    double inv;
    if (flag == 2) {
      for (int r = threadIdx.x; r < sl.rows; r += kPB) {
        ws[r] = zs[r];
        g.soln[3 * sl.m0 + r] = 0.0;
      }
      if (sl.body && threadIdx.x < 6) g.soln[vel + threadIdx.x] = 0.0;
      if (threadIdx.x < 6) qvel[threadIdx.x] = V(rhs_vel[threadIdx.x] / norm_rhs);
      kslot = K_RHS;
      inv = norm_rhs;
    } else {
      if (threadIdx.x < 6) qvel[threadIdx.x] = V(r0v[threadIdx.x] / beta0);
      kslot = k_r0;
      inv = beta0;
    }
    const V rinv = V(1.0 / inv);
    __syncthreads();
    for (int r = threadIdx.x; r < sl.rows; r += kPB) ws[r] = ws[r] * rinv;
    __syncthreads();
    store_q(p, sl, qres, 0, ws);
    if (threadIdx.x < 6) qvres[threadIdx.x] = qvel[threadIdx.x];
    if (threadIdx.x == 0) beta[0] = beta0;
    // z = P^-1 Q_0: sum_m (Q_0 ; d x Q_0) = (partials of the unscaled vector) / inv
    cta_sums(p6 + (size_t)kslot * 6 * G, G, 6, tf, cst);
    if (threadIdx.x < 6) qsres[threadIdx.x] = tf[threadIdx.x] * rinv;
    precond(p, sl, ws, qvel, tf, rinv, zs, zv, mats);
    pack_records(p, sl, zs);
    slice_partials(p, sl, zs, K_Z, -1);
  }
  if (!pg_barrier(p, &epoch)) return;

  // ---- Arnoldi steps. Step k: M_bb z_{k-1} (CTA 0 meanwhile finishes step
  //      k-1's Givens rotation and convergence test), w = A z_{k-1}, two
  //      classical Gram-Schmidt passes, ||w||, Q_k = w / ||w||, z_k = P^-1 Q_k.
  V *h1g = reinterpret_cast<V *>(p.aux + kCtl), *h2g = h1g + kPK, *yg = h2g + kPK;
  int k = 1;
  double qn = 0.0;
  for (;;) {
    PG_STAMP(k, 0);
    mbb_units(p, src);
    if (p.rank == 0 && k > 1) {
      // Givens rotation (mobility_solver.cpp:2370-2413) of step kk = k - 1
      const int kk = k - 1;
      if (threadIdx.x == 0) {
        for (int i = 0; i < kk; ++i) hcol[i] = (double)h1[i] + (double)h2[i];
        hcol[kk] = qn;
        const double rel = givens_step(kk, hcol, cs, sn, beta, norm_rhs);
        int fin = rel <= g.tol || kk == g.max_iter;
        int stt = 0;
        if (!(rel == rel)) {
          fin = 1;
          stt = 1;
        }
        tmp8[0] = fin;
        tmp8[1] = rel;
        tmp8[2] = stt;
      }
      __syncthreads();
      const int ld = g.max_iter + 1;
      for (int i = threadIdx.x; i <= kk; i += kPB) g.H[i + (size_t)(kk - 1) * ld] = hcol[i];
      if (tmp8[0] != 0.0) {
        back_substitute(p, kk, hcol, beta, yv, hb);
        for (int i = threadIdx.x; i < kk; i += kPB) yg[i] = V(yv[i]);
      }
      if (threadIdx.x == 0) {
        p.aux[C_FINISH] = tmp8[0];
        p.aux[C_REL] = tmp8[1];
        p.aux[C_STATUS] = tmp8[2];
      }
    }
    if (!pg_barrier(p, &epoch)) return;
    if (k > 1 && ldcg(p.aux + C_FINISH) != 0.0) {
      k -= 1;
      break;
    }
    PG_STAMP(k, 1);

    // w = A z (slice rows; body rows w_vel = -sum (z ; d x z) in every CTA),
    // CGS pass 1 partial dots
    stage(p6 + (size_t)K_Z * 6 * G, 6 * G, cst);
    if (p.S * sl.rows <= kHB) {
      float2 *st2 = reinterpret_cast<float2 *>(hb);
      stage_splits(p, sl, st2);
      __syncthreads();
      sum_staged(cst, G, 6, tf);
      // tpr adjacent threads per row add the splits sp = sub (mod tpr),
      // compensated, then combine their (hi, lo) pairs by a fixed shuffle tree
      const int tpr = 8 * sl.rows <= kPB ? 8 : 4 * sl.rows <= kPB ? 4 : 2 * sl.rows <= kPB ? 2 : 1;
      for (int r0 = 0; r0 < sl.rows; r0 += kPB / tpr) {
        const int r = r0 + (int)threadIdx.x / tpr, sub = threadIdx.x & (tpr - 1);
        float h = 0.f, l = 0.f;
        if (r < sl.rows)
          for (int sp = sub; sp < p.S; sp += tpr) {
            two_sum(h, l, st2[sp * sl.rows + r].x);
            l += st2[sp * sl.rows + r].y;
          }
        for (int o = 1; o < tpr; o <<= 1) {
          const float ho = __shfl_xor_sync(0xffffffffu, h, o);
          const float lo = __shfl_xor_sync(0xffffffffu, l, o);
          two_sum(h, l, ho);
          l += lo;
        }
        if (r < sl.rows && sub == 0) {
          const int m = sl.m0 + r / 3, j = r - 3 * (r / 3);
          const V *d = sl.d + 3 * (m - sl.m0);
          V body;
          if (j == 0) body = zv[0] - d[1] * zv[5] + d[2] * zv[4];
          else if (j == 1) body = zv[1] - d[2] * zv[3] + d[0] * zv[5];
          else body = zv[2] - d[0] * zv[4] + d[1] * zv[3];
          ws[r] = -body + scale * (V(h) + V(l));
        }
      }
      __syncthreads();
    } else {
      __syncthreads();
      sum_staged(cst, G, 6, tf);
      apply_rows(p, sl, zv, ws, hb, acc);
    }
    if (threadIdx.x < 6) wvel[threadIdx.x] = -tf[threadIdx.x];
    PG_STAMP(k, 2);
    slice_dots(p, sl, ws, k, pd1, qres);
    if (!pg_barrier(p, &epoch)) return;
    PG_STAMP(k, 3);
    // h1 (summed by every CTA while the partials fit the staging buffers,
    // else spread over the grid and published)
    V *stg = reinterpret_cast<V *>(hb);
    if (!local_dots(p, pd1, k, wvel, qvres, h1, stg)) {
      reduce_dots(p, pd1, k, wvel, qvres, h1g);
      if (!pg_barrier(p, &epoch)) return;
      for (int i = threadIdx.x; i < k; i += kPB) h1[i] = __ldcg(h1g + i);
      __syncthreads();
    }
    PG_STAMP(k, 4);

    // w' = w - Q h1; CGS pass 2 partial dots, and ||w'||^2 and
    // sum (w' ; d x w') partials
    slice_axpy(p, sl, h1, k, ws, V(-1), qres);
    vel_axpy(qvres, h1, k, wvel, V(-1));
    slice_dots(p, sl, ws, k, pd2, qres);
    slice_partials(p, sl, ws, K_W, S_NORM);
    if (!pg_barrier(p, &epoch)) return;
    PG_STAMP(k, 5);
    if (!local_dots(p, pd2, k, wvel, qvres, h2, stg)) {
      reduce_dots(p, pd2, k, wvel, qvres, h2g);
      if (!pg_barrier(p, &epoch)) return;
      for (int i = threadIdx.x; i < k; i += kPB) h2[i] = __ldcg(h2g + i);
      __syncthreads();
    }
    PG_STAMP(k, 6);

    // w'' = w' - Q h2; with Q orthonormal, ||w''||^2 = ||w'||^2 - ||h2||^2
    // and sum (w'' ; d x w'') = sum (w' ; d x w') - sum_i h2_i S_i, S_i the
    // sums of Q_i (kept in qsres); Q_k = w'' / ||w''||, z_k = P^-1 Q_k.
    // After the first pass h2 is small against w' (the lost orthogonality),
    // so the difference carries no cancellation.
    stage(ps + (size_t)S_NORM * G, G, cst);
    stage(p6 + (size_t)K_W * 6 * G, 6 * G, cst + G);
    __syncthreads();
    sum_staged(cst, G, 7, tf);
    __syncthreads();
    {
      // warp j < 6: the body sum j of w''; warp 6: ||w''||^2 (lanes over i)
      const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
      if (wid < 7) {
        V t = V(0);
        if (wid < 6) {
          for (int i = lane; i < k; i += 32) t += h2[i] * qsres[6 * i + wid];
        } else {
          for (int i = lane; i < k; i += 32) t -= h2[i] * h2[i];
          if (lane < 6) t += wvel[lane] * wvel[lane];
        }
        t = warp_sum(t);
        if (lane == 0) {
          if (wid < 6) {
            wsum6[wid] = tf[1 + wid] - t;
          } else {
            const V w2 = tf[0] + t;
            const V y = vrsqrt(w2);
            qn_s[0] = w2 * y;
            qn_s[1] = y;
          }
        }
      }
    }
    __syncthreads();
    slice_axpy(p, sl, h2, k, ws, V(-1), qres);
    vel_axpy(qvres, h2, k, wvel, V(-1));
    qn = qn_s[0];
    const V rqn = qn_s[1];
    for (int r = threadIdx.x; r < sl.rows; r += kPB) ws[r] = ws[r] * rqn;
    __syncthreads();
    store_q(p, sl, qres, k, ws);
    if (threadIdx.x < 6) {
      qvel[threadIdx.x] = wvel[threadIdx.x] * rqn;
      qvres[6 * k + threadIdx.x] = qvel[threadIdx.x];
      qsres[6 * k + threadIdx.x] = wsum6[threadIdx.x] * rqn;
    }
    __syncthreads();
    precond(p, sl, ws, qvel, wsum6, rqn, zs, zv, mats);
    pack_records(p, sl, zs);
    slice_partials(p, sl, zs, K_Z, -1);
    PG_STAMP(k, 7);
    if (!pg_barrier(p, &epoch)) return;
    ++k;
  }

  // ---- tmp = Q y (slice rows in ws, body rows in qvel), z = P^-1 tmp,
  //      soln += z -> (f_blobs, v_bodies) (:2440-2563)
  for (int i = threadIdx.x; i < k; i += kPB) yf[i] = __ldcg(yg + i);
  for (int r = threadIdx.x; r < sl.rows; r += kPB) ws[r] = V(0);
  if (threadIdx.x < 6) qvel[threadIdx.x] = V(0);
  __syncthreads();
  slice_axpy(p, sl, yf, k, ws, V(1), qres);
  vel_axpy(qvres, yf, k, qvel, V(1));
  slice_partials(p, sl, ws, K_T, -1);
  if (!pg_barrier(p, &epoch)) return;
  cta_sums(p6 + (size_t)K_T * 6 * G, G, 6, tf, cst);
  precond(p, sl, ws, qvel, tf, V(1), zs, zv, mats);
  for (int r = threadIdx.x; r < sl.rows; r += kPB) {
    const int t = 3 * sl.m0 + r;
    const double x = g.soln[t] + (double)zs[r];
    g.soln[t] = x;
    g.f_blobs[t] = x;
  }
  if (sl.body && threadIdx.x < 6) {
    const double x = g.soln[vel + threadIdx.x] + (double)zv[threadIdx.x];
    g.soln[vel + threadIdx.x] = x;
    g.v_bodies[threadIdx.x] = x;
  }
  if (p.rank == 0 && threadIdx.x == 0) {
    st->norm_rhs = norm_rhs;
    st->rel = ldcg(p.aux + C_REL);
    st->iters = k;
    st->flag = 0;
    st->status = (int)ldcg(p.aux + C_STATUS);
    st->done = 1;
  }
}

// Resident Krylov columns and dynamic shared memory of the kernel with
// vectors of V for slices of `rows` rows; false when not even one column fits.
template <typename V>
bool pg_smem(long avail, int rows, int max_iter, int *Kr, size_t *dyn) {
  const long cols = (avail - (long)pg_dyn_fixed<V>()) / (long)(sizeof(V) * rows);
  if (cols < 1) return false;
  *Kr = (int)std::min<long>(max_iter + 1, cols);
  *dyn = pg_dyn_fixed<V>() + sizeof(V) * (size_t)*Kr * rows;
  return true;
}

// The largest dynamic shared memory a CTA of the instantiation may use (set
// once per instantiation, so that one setting serves every shape: solves of
// several shapes share launches); false when no CTA of it fits an SM.
template <typename V>
bool pg_ready(int optin, size_t dyn) {
  cudaFuncAttributes fa{};
  int occ = 0;
  if (cudaFuncGetAttributes(&fa, gmres_persistent_kernel<V>) != cudaSuccess ||
      cudaFuncSetAttribute(gmres_persistent_kernel<V>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)(optin - (long)fa.sharedSizeBytes)) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, gmres_persistent_kernel<V>, kPB, dyn) !=
          cudaSuccess ||
      occ < 1) {
    cudaGetLastError();
    return false;
  }
  return true;
}

int pg_grid(int nb, int sms, int max_iter, PgShape *shape) {
  int dev = 0, optin = 0;
  cudaFuncAttributes f32{}, f64{};
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) !=
          cudaSuccess ||
      cudaFuncGetAttributes(&f32, gmres_persistent_kernel<float>) != cudaSuccess ||
      cudaFuncGetAttributes(&f64, gmres_persistent_kernel<double>) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  const int P = sms;  // one CTA per SM
  if (P > kMaxPgCtas) return 0;
  int G = std::max(1, std::min(P, (nb + 3) / 4));
  int per = std::max(1, (nb + G - 1) / G);
  G = std::max(1, (nb + per - 1) / per);
  if (per > kMaxPgBlobsPerCta) return 0;
  const int rows = 3 * per;
  // dynamic shared memory: the staging buffers, then as many resident Krylov
  // columns of the slice as fit (all max_iter + 1 when possible)
  if (!pg_smem<float>((long)optin - (long)f32.sharedSizeBytes - 1024, rows, max_iter, &shape->Kr,
                      &shape->dyn_smem) ||
      !pg_smem<double>((long)optin - (long)f64.sharedSizeBytes - 1024, rows, max_iter,
                       &shape->Kr64, &shape->dyn_smem64) ||
      !pg_ready<float>(optin, shape->dyn_smem) || !pg_ready<double>(optin, shape->dyn_smem64))
    return 0;
  const int workers = P > 1 ? P - 1 : 1;  // CTA 0 runs the Givens step meanwhile
  const int TB = std::max(1, (nb + 2 * kPB - 1) / (2 * kPB));
  const int tbs = (nb + TB - 1) / TB;
  int S = std::max(1, std::min(workers / TB, nb / 32));
  const int chunk = (nb + S - 1) / S;
  S = (nb + chunk - 1) / chunk;
  shape->P = P;
  shape->G = G;
  shape->blobs_per_cta = per;
  shape->TB = TB;
  shape->tbs = tbs;
  shape->S = S;
  shape->chunk = chunk;
  return 1;
}

int pg_trace_read(unsigned long long *out, int capacity, int *steps) {
#ifdef TFS_PG_TRACE
  const int n = 2 * kTraceSteps * kTracePhases;
  if (steps) *steps = kTraceSteps;
  if (out == nullptr || capacity < n) return -1;
  return cudaMemcpyFromSymbol(out, g_pg_trace, sizeof(unsigned long long) * n) == cudaSuccess ? 0 : -2;
#else
  (void)out;
  (void)capacity;
  if (steps) *steps = 0;
  return -3;
#endif
}

cudaError_t launch_gmres_persistent(const PgArgs *gp, const int2 *cmap, int ctas, size_t dyn_smem,
                                    int vec64, cudaStream_t st) {
  void *args[] = {const_cast<PgArgs **>(&gp), const_cast<int2 **>(&cmap)};
  const void *fn = vec64 ? (const void *)gmres_persistent_kernel<double>
                         : (const void *)gmres_persistent_kernel<float>;
  cudaError_t e = cudaLaunchCooperativeKernel(fn, dim3(ctas), dim3(kPB), args, dyn_smem, st);
  count_launch();
  return e;
}

}  // namespace tfs
