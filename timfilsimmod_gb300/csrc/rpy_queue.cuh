// rpy_queue.cuh -- the persistent work-queue form of the all-pairs RPY
// products: one launch evaluates any number of products ("jobs": a target
// set against one or two packed source sets, of one or many swimmers) and
// their source-split reductions.
//
// Work unit = (job, target block, source chunk). A target block is the
// BLOCK*TPT targets one CTA holds in registers; a chunk is `chunk`
// consecutive sources of the job's concatenated source sets (A, then B).
// The grid is persistent (resident CTAs per SM x SMs, or fewer when there
// are fewer units); every CTA takes units from one device counter until
// they run out, so SMs stay busy to the end whatever the mix of job sizes
// (the wave tail of a grid of equal CTAs disappears). Jobs are ordered by
// the host with the costliest pairs first.
//
// Determinism. A unit writes its targets' chunk sums to the job's partial
// buffer [chunk][target][vd]; the last unit of a target block to finish
// (an arrival counter per block) adds the block's partials in chunk order
// and writes (or adds to) the output. Which CTA computes which unit does not
// change a bit of the result: each target's sum is fixed by the job's chunk
// size alone, which depends only on its own source count (queue_chunking),
// never on the launch shape, the launch variant or the other jobs. So a
// swimmer's product is the same, bit for bit, alone and in a batch.
//
// Counters. counters[0] hands out units, counters[1] counts CTAs that have
// finished; the last CTA to finish resets both, and the last unit of each
// target block resets that block's arrival counter, so the buffers are zero
// again for the next launch without a memset. No CTA ever waits for another.
#pragma once

#include <atomic>

#include <cuda_runtime.h>

#include "rpy_tile.cuh"
#include "tfs_kernels.h"

namespace tfs {

// Target positions come from the job's packed records of the target kind
// (the FP32 records hold the origin-relative positions already rounded to
// FP32, so a unit does no FP64 work before its pairs).
template <typename T, int VD>
__device__ __forceinline__ void load_target_rec(const QueueJob &job, int i, T &x, T &y, T &z) {
  constexpr int L = Rec<T, VD == 6 ? 6 : 3>::len;
  const T *r = reinterpret_cast<const T *>(job.tgt_rec) + (size_t)i * L;
  x = r[0];
  y = r[1];
  z = r[2];
}

// Pair constants of (target kind, source set `set`), precomputed by the host.
template <typename T>
__device__ __forceinline__ PairConst<T> job_pair_const(const QueueJob &job, int set) {
  PairConst<T> pc;
  if constexpr (sizeof(T) == 4) {
    const float *q = job.pc32[set];
    pc.ai = q[0]; pc.aj = q[1]; pc.asum2 = q[2]; pc.s = q[3]; pc.s3 = q[4];
  } else {
    const double *q = job.pc64[set];
    pc.ai = q[0]; pc.aj = q[1]; pc.asum2 = q[2]; pc.s = q[3]; pc.s3 = q[4];
  }
  return pc;
}

// One unit: the BLOCK*TPT targets of block `blk` against chunk `c`.
// FP32: the chunk sum of each target component is kept as an unevaluated
// (hi, lo) pair of floats (per-tile FP32 sums folded by TwoSum) and stored
// as such; the block's last unit adds the pairs of all chunks in chunk
// order with TwoSum and converts once to FP64, times 1/(8 pi mu). FP64: plain
// FP64 sums, added in chunk order.
template <typename T, int VD, int FDA, int FDB, int BLOCK, int TPT, int TS>
__device__ __forceinline__ void queue_unit(const QueueJob &job, int blk, int c, T *smem,
                                           float *hl, int *s_last) {
  constexpr bool kComp = sizeof(T) == 4;
  const int n_tgt = job.n_tgt;
  const int tile0 = blk * BLOCK * TPT;

  T xt[TPT], yt[TPT], zt[TPT];
  T v[TPT][VD];
#pragma unroll
  for (int t = 0; t < TPT; ++t) {
    int i = tile0 + t * BLOCK + threadIdx.x;
    i = i < n_tgt ? i : n_tgt - 1;  // duplicate the last target; not written
    load_target_rec<T, VD>(job, i, xt[t], yt[t], zt[t]);
#pragma unroll
    for (int k = 0; k < VD; ++k) v[t][k] = T(0);
  }
  if (kComp) {
    for (int q = threadIdx.x; q < 2 * TPT * VD * BLOCK; q += BLOCK) hl[q] = 0.f;
  }
  // a warp whose targets all lie past the end (the last, partial block)
  // skips the pairs and only helps stage the tiles
  const int warp0 = tile0 + (threadIdx.x & ~31);
  const bool compute = warp0 < n_tgt;
  const int n_src = job.n_a + job.n_b;
  const int s0 = c * job.chunk;
  const int s1 = min(s0 + job.chunk, n_src);
  {
    const PairConst<T> pc = job_pair_const<T>(job, 0);
    const int lo = min(s0, job.n_a), hi = min(s1, job.n_a);
    if (lo < hi)
      sum_source_range<T, VD, FDA, BLOCK, TPT, TS>(
          v, xt, yt, zt, reinterpret_cast<const T *>(job.src_a), lo, hi, pc, smem, hl, compute);
  }
  if constexpr (FDB > 0) {
    const PairConst<T> pc = job_pair_const<T>(job, 1);
    const int lo = max(s0 - job.n_a, 0), hi = max(s1 - job.n_a, 0);
    if (lo < hi)
      sum_source_range<T, VD, (FDB > 0 ? FDB : 3), BLOCK, TPT, TS>(
          v, xt, yt, zt, reinterpret_cast<const T *>(job.src_b), lo, hi, pc, smem, hl, compute);
  }

  const double sc = job.scale;
  const bool direct = job.n_chunks == 1;
#pragma unroll
  for (int t = 0; t < TPT; ++t) {
    const int i = tile0 + t * BLOCK + threadIdx.x;
    if (i >= n_tgt) continue;
    if (direct) {
      double *o = job.out + (size_t)i * VD;
#pragma unroll
      for (int k = 0; k < VD; ++k) {
        const double r = sc * Comp<T, VD, BLOCK, TPT>::get(v, hl, t, k);
        o[k] = job.mode == OUT_ACCUMULATE ? o[k] + r : r;
      }
    } else if constexpr (kComp) {
      float2 *o = reinterpret_cast<float2 *>(job.partial) + ((size_t)c * n_tgt + i) * VD;
#pragma unroll
      for (int k = 0; k < VD; ++k) {
        const float *h = hl + ((t * VD + k) * 2) * BLOCK + threadIdx.x;
        o[k] = make_float2(h[0], h[BLOCK]);
      }
    } else {
      double *o = reinterpret_cast<double *>(job.partial) + ((size_t)c * n_tgt + i) * VD;
#pragma unroll
      for (int k = 0; k < VD; ++k) o[k] = (double)v[t][k];
    }
  }
  if (direct) return;

  // Arrival of this chunk for the block (the CTA's partial writes, ordered
  // by the barrier, then one GPU-scope fence and the counter); the last
  // arrival reduces the block's partials in chunk order.
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    *s_last = atomicAdd(job.block_done + blk, 1u) == (unsigned)(job.n_chunks - 1) ? 1 : 0;
    __threadfence();
  }
  __syncthreads();
  if (*s_last == 0) return;
  const int nc = job.n_chunks;
  const size_t stride = (size_t)n_tgt * VD;
#pragma unroll
  for (int t = 0; t < TPT; ++t) {
    const int i = tile0 + t * BLOCK + threadIdx.x;
    if (i >= n_tgt) continue;
    double r[VD];
    if constexpr (kComp) {
      const float2 *p = reinterpret_cast<const float2 *>(job.partial) + (size_t)i * VD;
      float H[VD], L[VD];
#pragma unroll
      for (int k = 0; k < VD; ++k) H[k] = L[k] = 0.f;
      int cc = 0;
      for (; cc + 4 <= nc; cc += 4) {  // four chunks' loads in flight, added in order
        float2 a[4][VD];
#pragma unroll
        for (int w = 0; w < 4; ++w)
#pragma unroll
          for (int k = 0; k < VD; ++k) a[w][k] = __ldcg(p + (size_t)(cc + w) * stride + k);
#pragma unroll
        for (int w = 0; w < 4; ++w)
#pragma unroll
          for (int k = 0; k < VD; ++k) {
            two_sum(H[k], L[k], a[w][k].x);
            L[k] += a[w][k].y;
          }
      }
      for (; cc < nc; ++cc) {
#pragma unroll
        for (int k = 0; k < VD; ++k) {
          const float2 a = __ldcg(p + (size_t)cc * stride + k);
          two_sum(H[k], L[k], a.x);
          L[k] += a.y;
        }
      }
#pragma unroll
      for (int k = 0; k < VD; ++k) r[k] = sc * ((double)H[k] + (double)L[k]);
    } else {
      const double *p = reinterpret_cast<const double *>(job.partial) + (size_t)i * VD;
#pragma unroll
      for (int k = 0; k < VD; ++k) r[k] = 0.0;
      int cc = 0;
      for (; cc + 4 <= nc; cc += 4) {  // four chunks' loads in flight, added in order
        double a[4][VD];
#pragma unroll
        for (int w = 0; w < 4; ++w)
#pragma unroll
          for (int k = 0; k < VD; ++k) a[w][k] = __ldcg(p + (size_t)(cc + w) * stride + k);
#pragma unroll
        for (int w = 0; w < 4; ++w)
#pragma unroll
          for (int k = 0; k < VD; ++k) r[k] += a[w][k];
      }
      for (; cc < nc; ++cc) {
#pragma unroll
        for (int k = 0; k < VD; ++k) r[k] += __ldcg(p + (size_t)cc * stride + k);
      }
#pragma unroll
      for (int k = 0; k < VD; ++k) r[k] *= sc;
    }
    double *o = job.out + (size_t)i * VD;
    if (job.mode == OUT_ACCUMULATE) {
#pragma unroll
      for (int k = 0; k < VD; ++k) o[k] += r[k];
    } else {
#pragma unroll
      for (int k = 0; k < VD; ++k) o[k] = r[k];
    }
  }
  if (threadIdx.x == 0) job.block_done[blk] = 0u;
}

template <typename T, int FDA, int FDB, int BLOCK, int TPT, int TS, int MINB>
__global__ void __launch_bounds__(BLOCK, MINB) rpy_queue_kernel(const QueueArgs q) {
  constexpr int LA = Rec<T, FDA>::len;
  constexpr int LB = FDB > 0 ? Rec<T, (FDB > 0 ? FDB : 3)>::len : 0;
  constexpr int LMAX = LA > LB ? LA : LB;
  extern __shared__ __align__(16) unsigned char queue_smem[];
  T *smem = reinterpret_cast<T *>(queue_smem);
  float *hl = reinterpret_cast<float *>(queue_smem + sizeof(T) * TS * LMAX);
  __shared__ int s_end[kQueueMaxJobs];  // exclusive end unit of job j
  __shared__ int s_unit, s_last;

  // per-job unit ranges for this launch's target blocks (BLOCK*TPT targets)
  if (threadIdx.x == 0) {
    int acc = 0;
    for (int j = 0; j < q.n_jobs; ++j) {
      const QueueJob &jb = q.jobs[j];
      const bool skip = jb.skip != nullptr && *jb.skip != 0;
      const int nblk = skip ? 0 : (jb.n_tgt + BLOCK * TPT - 1) / (BLOCK * TPT);
      acc += nblk * jb.n_chunks;
      s_end[j] = acc;
    }
  }
  __syncthreads();
  const int n_units = q.n_jobs > 0 ? s_end[q.n_jobs - 1] : 0;

  // A CTA takes its next unit only when it is free for it: a unit reserved
  // ahead would keep an SM busy after the others have run out of work. (The
  // counter's round trip stalls one CTA; the other resident CTAs keep the SM
  // issuing.)
  for (;;) {
    if (threadIdx.x == 0) s_unit = (int)atomicAdd(q.counters, 1u);
    __syncthreads();
    const int u = s_unit;
    if (u >= n_units) break;
    int lo = 0, hi = q.n_jobs - 1;  // first job whose end exceeds u
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (s_end[mid] > u) hi = mid; else lo = mid + 1;
    }
    const QueueJob &job = q.jobs[lo];
    const int local = u - (lo > 0 ? s_end[lo - 1] : 0);
    const int blk = local / job.n_chunks, c = local - blk * job.n_chunks;
    if (job.vd == 6)
      queue_unit<T, 6, FDA, FDB, BLOCK, TPT, TS>(job, blk, c, smem, hl, &s_last);
    else
      queue_unit<T, 3, FDA, FDB, BLOCK, TPT, TS>(job, blk, c, smem, hl, &s_last);
    __syncthreads();  // s_unit and the shared tiles are reused by the next unit
  }
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(q.counters + 1, 1u) == gridDim.x - 1) {
      q.counters[0] = 0u;
      q.counters[1] = 0u;
    }
  }
}

// Dynamic shared memory: the source tile plus, for FP32, the compensated
// running sums of the larger (6-component) target kind.
template <typename T, int FDA, int FDB, int BLOCK, int TPT, int TS>
constexpr size_t queue_smem_bytes() {
  constexpr int LA = Rec<T, FDA>::len;
  constexpr int LB = FDB > 0 ? Rec<T, (FDB > 0 ? FDB : 3)>::len : 0;
  constexpr int LMAX = LA > LB ? LA : LB;
  return sizeof(T) * TS * LMAX + (sizeof(T) == 4 ? sizeof(float) * 2 * TPT * 6 * BLOCK : 0);
}

// Launch one instantiation with `ctas` CTAs; with ctas == 0 only report the
// resident CTAs per SM (cached per device).
template <typename T, int FDA, int FDB, int BLOCK, int TPT, int TS, int MINB>
cudaError_t queue_launch_fn(const QueueArgs &a, int ctas, cudaStream_t st, int *resident) {
  constexpr size_t smem = queue_smem_bytes<T, FDA, FDB, BLOCK, TPT, TS>();
  static std::atomic<int> occupancy[kMaxDevices];
  auto kern = rpy_queue_kernel<T, FDA, FDB, BLOCK, TPT, TS, MINB>;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  if (occupancy[dev].load() == 0) {
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int occ = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, BLOCK, smem);
    if (e != cudaSuccess) return e;
    occupancy[dev].store(occ < 1 ? 1 : occ);
  }
  if (resident) *resident = occupancy[dev].load();
  if (ctas <= 0) return cudaSuccess;
  kern<<<ctas, BLOCK, smem, st>>>(a);
  return cudaGetLastError();
}

// One row of a queue dispatch table: the three source specifications in
// the order of QueueSources.
#define TFS_QUEUE_ROW(T, B, P, S, M)                                                     \
  {                                                                                      \
    queue_launch_fn<T, 6, 0, B, P, S, M>, queue_launch_fn<T, 3, 0, B, P, S, M>,          \
        queue_launch_fn<T, 6, 3, B, P, S, M>                                             \
  }

}  // namespace tfs
