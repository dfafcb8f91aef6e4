// rpy_kernels.cu -- all-pairs RPY mobility, barrier-force and support
// kernels for sm_103a.
//
// Layout. User arrays stay in the reference's AoS float64 layouts. Before a
// product, the sources are packed once into fixed-size records
// (pack_sources): FP64 segments {x,y,z,fx,fy,fz,tx,ty,tz,0} (80 B), FP64 blobs
// {x,y,z,fx,fy,fz} (48 B), FP32 segments {x,y,z,fx,fy,fz,tx,ty,tz,0,0,0}
// (48 B), FP32 blobs {x,y,z,fx,fy,fz,0,0} (32 B). Records are multiples of
// 16 B so a tile of consecutive sources is one contiguous, 16-B aligned block
// that the CTA stages into shared memory with 16-B vector loads; every thread
// then reads each record by broadcast.
// FP32 positions are stored relative to an origin (the mean particle
// position, computed on the device), which keeps FP32 rounding of
// differences relative to the swimmer's size rather than to absolute
// coordinates.
//
// Work decomposition. A CTA owns BLOCK*TPT targets (TPT per thread, strided
// by BLOCK) and one contiguous chunk of the sources; grid.y is the number of
// source splits. With one split the CTA writes (or adds) the final velocities
// (assign/accumulate semantics of cuda_functions.cu:463-468 and :625-630);
// with several, each CTA writes its partial sums to a scratch buffer and
// reduce_partials adds them in split order. Either way every target sums its
// sources in a fixed order, so results are deterministic.
#include <cuda_runtime.h>

#include <atomic>

#include <algorithm>

#include "rpy_tile.cuh"
#include "tfs_device.cuh"
#include "tfs_kernels.h"

namespace tfs {

// ---------------------------------------------------------------------------
// Origin/extent of a particle set: origin = mean position, extent = max over
// particles of max |x_k - origin_k|. One CTA; used for FP32 centring and for
// the FP32 candidate test of the barrier kernel.
// ---------------------------------------------------------------------------
constexpr int kOriginCTAs = 64;

// One pass over all particles, kOriginCTAs CTAs: the FP32 bounds of the
// positions (min and max are exact in any order); the last CTA to finish
// combines the CTAs' bounds and writes the origin, the centre of the bounds
// (out[0..2]), and out[3], an upper bound of every |x_k - o_k|: the largest
// half-width plus the FP32 rounding of the coordinates (2^-23 of the largest
// magnitude). The FP32 products and the barrier's candidate test measure
// positions from this origin. Per-CTA bounds live in out[4..] (as floats).
__global__ void __launch_bounds__(256) origin_kernel(const double *__restrict__ xa, int na,
                                                     const double *__restrict__ xb, int nb,
                                                     double *__restrict__ out /* [4 + 4 kOriginCTAs] */,
                                                     unsigned *__restrict__ counter) {
  __shared__ float red[8][6];
  __shared__ bool last;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, n = na + nb;
  float *part = reinterpret_cast<float *>(out + 4);
  float v[6] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
  for (int i = blockIdx.x * blockDim.x + tid; i < n; i += gridDim.x * blockDim.x) {
    const double *x = i < na ? xa + 3 * (size_t)i : xb + 3 * (size_t)(i - na);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const float c = float(x[k]);
      v[k] = fminf(v[k], c);
      v[k + 3] = fmaxf(v[k + 3], c);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      const float w = __shfl_xor_sync(0xffffffffu, v[k], o);
      v[k] = k < 3 ? fminf(v[k], w) : fmaxf(v[k], w);
    }
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < 6; ++k) red[wid][k] = v[k];
  __syncthreads();
  if (tid < 6) {
    float b = red[0][tid];
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w)
      b = tid < 3 ? fminf(b, red[w][tid]) : fmaxf(b, red[w][tid]);
    part[6 * blockIdx.x + tid] = b;
  }
  __syncthreads();
  if (tid == 0) {
    __threadfence();
    last = atomicAdd(counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last || wid != 0) return;
  __threadfence();
  float u[6] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
  for (int c = lane; c < (int)gridDim.x; c += 32)
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      const float w = __ldcg(part + 6 * c + k);
      u[k] = k < 3 ? fminf(u[k], w) : fmaxf(u[k], w);
    }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      const float w = __shfl_xor_sync(0xffffffffu, u[k], o);
      u[k] = k < 3 ? fminf(u[k], w) : fmaxf(u[k], w);
    }
  if (lane == 0) {
    double ext = 0.0, mag = 0.0;
    for (int k = 0; k < 3; ++k) {
      const double lo = n > 0 ? (double)u[k] : 0.0, hi = n > 0 ? (double)u[k + 3] : 0.0;
      out[k] = 0.5 * (lo + hi);
      ext = fmax(ext, 0.5 * (hi - lo));
      mag = fmax(mag, fmax(fabs(lo), fabs(hi)));
    }
    out[3] = ext + mag * 1.1920928955078125e-07;
    counter[0] = 0;
  }
}

// ---------------------------------------------------------------------------
// Source packing: AoS float64 positions/forces -> records.
// ---------------------------------------------------------------------------
template <typename T, int FD>
__global__ void pack_sources_kernel(T *__restrict__ rec, const double *__restrict__ x,
                                    const double *__restrict__ f, int n,
                                    const double *__restrict__ origin) {
  constexpr int L = Rec<T, FD>::len;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double o0 = 0.0, o1 = 0.0, o2 = 0.0;
  if (origin != nullptr) {
    o0 = origin[0];
    o1 = origin[1];
    o2 = origin[2];
  }
  T *r = rec + (size_t)i * L;
  r[0] = T(x[3 * (size_t)i] - o0);
  r[1] = T(x[3 * (size_t)i + 1] - o1);
  r[2] = T(x[3 * (size_t)i + 2] - o2);
#pragma unroll
  for (int k = 0; k < FD; ++k) r[3 + k] = T(f[(size_t)FD * i + k]);
#pragma unroll
  for (int k = 3 + FD; k < L; ++k) r[k] = T(0);
}

// out[i] (= or +=) sum over splits of partial[s][i], s in order.
__global__ void reduce_partials_kernel(double *__restrict__ out,
                                       const double *__restrict__ partial, int n_elems,
                                       int splits, int accumulate, const int *skip) {
  if (skip != nullptr && *skip) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_elems) return;
  double s = 0.0;
  for (int p = 0; p < splits; ++p) s += partial[(size_t)p * n_elems + i];
  out[i] = accumulate ? out[i] + s : s;
}

// ---------------------------------------------------------------------------
// Barrier (steric) forces, cuda_functions.cu:1240-1436 without a plane wall.
// Targets are segments (skip self and the nearest neighbours on the same
// filament; adds into f_segs) or blobs (skip self; assigns
// f_blobs_repulsion). A pair can act only inside 1.1 (a_i + a_j), so the
// sources are binned on a hashed grid of cells at least that wide (FP32
// positions relative to the origin, with a margin that bounds their
// rounding): bar_bin_kernel puts every source into its cell's bucket, and
// bar_pair_kernel tests each target against the 27 cells around it, keeps
// the sources that pass the FP32 candidate test, sorts them by index and runs
// the reference's FP64 test and force on them in that order -- the
// reference's sequential sum over all sources, since pairs out of reach add
// nothing. A bucket or candidate list that overflows marks the call, and
// bar_apply_kernel then recomputes every target by the plain sequential loop
// over all sources; otherwise it applies the binned sums.
// ---------------------------------------------------------------------------
constexpr int kBarSlots = 8;   // sources per bucket
constexpr int kBarCand = 48;   // candidates per target

// Hash of a cell (its integer coordinates) into buckets of T (a power of two).
__device__ __forceinline__ unsigned bar_hash(int cx, int cy, int cz, unsigned T) {
  return (((unsigned)cx * 73856093u) ^ ((unsigned)cy * 19349663u) ^ ((unsigned)cz * 83492791u)) &
         (T - 1u);
}

// The pair constants of one target kind (the thresholds of the reference's
// test and of the FP32 candidate test).
struct BarPairConst {
  double asum_seg, asum_blob, emag;
  float thr2_seg, thr2_blob;
};

__device__ __forceinline__ BarPairConst bar_pair_const(const BarrierArgs &a, bool target_blob) {
  BarPairConst c;
  // |d_fp32 - d| <= 2 sqrt(3) extent 2^-24 =: delta (each coordinate is
  // rounded once to FP32, relative 2^-24), plus FP32 arithmetic in d^2.
  const float delta = float(4.0 * a.origin[3] * 5.9604644775390625e-08 + 1e-30);
  c.asum_seg = target_blob ? a.a_blob + a.a_seg : 2.0 * a.a_seg;
  c.asum_blob = target_blob ? 2.0 * a.a_blob : a.a_seg + a.a_blob;
  const float thr_seg = float(1.1 * c.asum_seg) + 2.f * delta;
  const float thr_blob = float(1.1 * c.asum_blob) + 2.f * delta;
  c.thr2_seg = thr_seg * thr_seg * 1.0001f;
  c.thr2_blob = thr_blob * thr_blob * 1.0001f;
  c.emag = a.repulsive_force_factor * (double)a.end_force_magnitude;
  return c;
}

__device__ __forceinline__ const double *bar_pos(const BarrierArgs &a, int j) {
  return j < a.num_segs ? a.x_segs + 3 * (size_t)j : a.x_blobs + 3 * (size_t)(j - a.num_segs);
}

// The reference's pair (exclusions, FP64 test and force) of target i
// (position xi, filament fil_i) with source jj, added into f.
__device__ __forceinline__ void bar_pair(const BarrierArgs &a, const BarPairConst &c,
                                         bool target_blob, int i, int fil_i, const double *xi,
                                         int jj, double *f) {
  const bool src_is_seg = jj < a.num_segs;
  // exclusions, :1319 and :1410
  if (target_blob) {
    if (i + a.num_segs == jj) return;
  } else if (src_is_seg) {
    const int fil_j = jj / a.nseg;
    if (fil_i == fil_j && (i - jj <= 1 && jj - i <= 1)) return;
  }
  const double asum = src_is_seg ? c.asum_seg : c.asum_blob;
  const double *xj = bar_pos(a, jj);
  const double dx = xi[0] - xj[0], dy = xi[1] - xj[1], dz = xi[2] - xj[2];
  const double dist = sqrt(dx * dx + dy * dy + dz * dz);
  if (dist < 1.1 * asum) {
    const double chi = 10.0 / asum;
    double fac = fmin(1.0, 1.0 - chi * (dist - asum));
    fac *= c.emag * fac * fac * fac;
    const double dm1 = 1.0 / dist;
    f[0] += fac * dx * dm1;
    f[1] += fac * dy * dm1;
    f[2] += fac * dz * dm1;
  }
}

// Cell width: the larger candidate reach of either target kind, 1% wider so
// that a pair within reach lies in neighbouring cells despite rounding.
__device__ __forceinline__ float bar_cell(const BarrierArgs &a) {
  const BarPairConst s = bar_pair_const(a, false), b = bar_pair_const(a, true);
  const float r2 = 1.001f * fmaxf(fmaxf(s.thr2_seg, s.thr2_blob), fmaxf(b.thr2_seg, b.thr2_blob));
  return 1.01f * sqrtf(r2);
}

// Bins every source: bucket of its cell, slot from the bucket's counter;
// entry {x, y, z, index} with the FP32 origin-relative position.
__global__ void bar_bin_kernel(const BarrierArgs a, BarGrid g) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= a.num_segs + a.num_blobs) return;
  const double *x = bar_pos(a, j);
  const float px = float(x[0] - a.origin[0]), py = float(x[1] - a.origin[1]),
              pz = float(x[2] - a.origin[2]);
  const float h = bar_cell(a);
  const unsigned b = bar_hash((int)floorf(px / h), (int)floorf(py / h), (int)floorf(pz / h), g.T);
  const unsigned slot = atomicAdd(g.count + b, 1u);
  if (slot < (unsigned)kBarSlots) g.entry[(size_t)b * kBarSlots + slot] = make_float4(px, py, pz, __int_as_float(j));
  else atomicExch(g.overflow, 1u);
}

// One thread per target (segments, then blobs): its binned sum into g.sum.
__global__ void bar_pair_kernel(const BarrierArgs a, BarGrid g) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int n_tgt = a.num_segs + (a.free_body ? a.num_blobs : 0);
  if (t >= n_tgt) return;
  const bool tb = t >= a.num_segs;
  const int i = tb ? t - a.num_segs : t;
  const double *xp = tb ? a.x_blobs + 3 * (size_t)i : a.x_segs + 3 * (size_t)i;
  const double xi[3] = {xp[0], xp[1], xp[2]};
  const float px = float(xi[0] - a.origin[0]), py = float(xi[1] - a.origin[1]),
              pz = float(xi[2] - a.origin[2]);
  const BarPairConst c = bar_pair_const(a, tb);
  const float h = bar_cell(a);
  const int cx = (int)floorf(px / h), cy = (int)floorf(py / h), cz = (int)floorf(pz / h);
  // the 27 cells' buckets and counts, all loads in flight at once
  unsigned bk[27];
  int cnt[27];
#pragma unroll
  for (int k = 0; k < 27; ++k) {
    bk[k] = bar_hash(cx + k % 3 - 1, cy + (k / 3) % 3 - 1, cz + k / 9 - 1, g.T);
    cnt[k] = (int)min(__ldg(g.count + bk[k]), (unsigned)kBarSlots);
  }
  int cand[kBarCand];
  int n = 0;
  bool over = false;
#pragma unroll
  for (int k = 0; k < 27; ++k) {
    const int ex = cx + k % 3 - 1, ey = cy + (k / 3) % 3 - 1, ez = cz + k / 9 - 1;
    for (int s = 0; s < cnt[k]; ++s) {
      const float4 e = __ldg(g.entry + (size_t)bk[k] * kBarSlots + s);
      // another cell sharing the bucket
      if ((int)floorf(e.x / h) != ex || (int)floorf(e.y / h) != ey || (int)floorf(e.z / h) != ez)
        continue;
      const int j = __float_as_int(e.w);
      const float ddx = px - e.x, ddy = py - e.y, ddz = pz - e.z;
      const float d2f = ddx * ddx + ddy * ddy + ddz * ddz;
      if (d2f >= (j < a.num_segs ? c.thr2_seg : c.thr2_blob)) continue;
      if (n < kBarCand) cand[n++] = j;
      else over = true;
    }
  }
  if (over) atomicExch(g.overflow, 1u);
  // the reference's order: increasing source index (insertion sort)
  for (int p = 1; p < n; ++p) {
    const int v = cand[p];
    int q = p - 1;
    while (q >= 0 && cand[q] > v) {
      cand[q + 1] = cand[q];
      --q;
    }
    cand[q + 1] = v;
  }
  double f[3] = {0.0, 0.0, 0.0};
  const int fil_i = tb ? -1 : i / a.nseg;
  for (int p = 0; p < n; ++p) bar_pair(a, c, tb, i, fil_i, xi, cand[p], f);
  g.sum[3 * (size_t)t] = f[0];
  g.sum[3 * (size_t)t + 1] = f[1];
  g.sum[3 * (size_t)t + 2] = f[2];
}

// Applies the binned sums, or -- after an overflow -- recomputes each
// target by the sequential loop over every source (the FP32 candidate test,
// then the reference's pair), which gives the same sums.
__global__ void bar_apply_kernel(const BarrierArgs a, BarGrid g) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int n_tgt = a.num_segs + (a.free_body ? a.num_blobs : 0);
  if (t >= n_tgt) return;
  const bool tb = t >= a.num_segs;
  const int i = tb ? t - a.num_segs : t;
  double f[3];
  if (*(volatile const unsigned *)g.overflow == 0u) {
    f[0] = g.sum[3 * (size_t)t];
    f[1] = g.sum[3 * (size_t)t + 1];
    f[2] = g.sum[3 * (size_t)t + 2];
  } else {
    const double *xp = tb ? a.x_blobs + 3 * (size_t)i : a.x_segs + 3 * (size_t)i;
    const double xi[3] = {xp[0], xp[1], xp[2]};
    const float px = float(xi[0] - a.origin[0]), py = float(xi[1] - a.origin[1]),
                pz = float(xi[2] - a.origin[2]);
    const BarPairConst c = bar_pair_const(a, tb);
    const int fil_i = tb ? -1 : i / a.nseg;
    f[0] = f[1] = f[2] = 0.0;
    for (int j = 0; j < a.num_segs + a.num_blobs; ++j) {
      const double *xj = bar_pos(a, j);
      const float ddx = px - float(xj[0] - a.origin[0]), ddy = py - float(xj[1] - a.origin[1]),
                  ddz = pz - float(xj[2] - a.origin[2]);
      if (ddx * ddx + ddy * ddy + ddz * ddz >= (j < a.num_segs ? c.thr2_seg : c.thr2_blob))
        continue;
      bar_pair(a, c, tb, i, fil_i, xi, j, f);
    }
  }
  if (tb) {
    a.f_blobs_repulsion[3 * (size_t)i] = f[0];
    a.f_blobs_repulsion[3 * (size_t)i + 1] = f[1];
    a.f_blobs_repulsion[3 * (size_t)i + 2] = f[2];
  } else {
    a.f_segs[6 * (size_t)i] += f[0];
    a.f_segs[6 * (size_t)i + 1] += f[1];
    a.f_segs[6 * (size_t)i + 2] += f[2];
  }
}

// ---------------------------------------------------------------------------
// Host-side launchers
// ---------------------------------------------------------------------------
// SM count of each device, set once per device; host threads may race to set it.
static std::atomic<int> g_num_sms[kMaxDevices];

int num_sms() {
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= kMaxDevices) dev = 0;
  if (g_num_sms[dev].load() == 0) {
    int n = 0;
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    g_num_sms[dev].store(n > 0 ? n : 1);
  }
  return g_num_sms[dev].load();
}

cudaError_t launch_reduce_partials(double *out, const double *partial, int n_elems, int splits,
                                   int accumulate, cudaStream_t st) {
  if (n_elems <= 0) return cudaSuccess;
  reduce_partials_kernel<<<(n_elems + 255) / 256, 256, 0, st>>>(out, partial, n_elems, splits,
                                                                accumulate, nullptr);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_origin(const double *xa, int na, const double *xb, int nb, double *out,
                          unsigned *counter, cudaStream_t st) {
  const int ctas = std::max(1, std::min(kOriginCTAs, (na + nb + 255) / 256));
  origin_kernel<<<ctas, 256, 0, st>>>(xa, na, xb, nb, out, counter);
  count_launch();
  return cudaGetLastError();
}

size_t origin_elems() { return 4 + 4 * (size_t)kOriginCTAs; }

template <typename T, int FD>
static cudaError_t pack_t(void *rec, const double *x, const double *f, int n,
                          const double *origin, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  pack_sources_kernel<T, FD><<<(n + 255) / 256, 256, 0, st>>>(reinterpret_cast<T *>(rec), x, f,
                                                               n, origin);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_pack(int fp32, int fd, void *rec, const double *x, const double *f, int n,
                        const double *origin, cudaStream_t st) {
  if (fp32) return fd == 6 ? pack_t<float, 6>(rec, x, f, n, origin, st)
                           : pack_t<float, 3>(rec, x, f, n, origin, st);
  return fd == 6 ? pack_t<double, 6>(rec, x, f, n, nullptr, st)
                 : pack_t<double, 3>(rec, x, f, n, nullptr, st);
}

// FP32x2 records: {-x,-x,-y,-y,-z,-z,f0,f0,...} (see rpy_tile_x2.cuh).
template <int FD>
__global__ void pack_sources_x2_kernel(float *__restrict__ rec, const double *__restrict__ x,
                                       const double *__restrict__ f, int n,
                                       const double *__restrict__ origin) {
  constexpr int L = FD == 6 ? 20 : 12;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float *r = rec + (size_t)i * L;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float m = float(origin[k] - x[3 * (size_t)i + k]);
    r[2 * k] = m;
    r[2 * k + 1] = m;
  }
#pragma unroll
  for (int k = 0; k < FD; ++k) {
    const float q = float(f[(size_t)FD * i + k]);
    r[6 + 2 * k] = q;
    r[6 + 2 * k + 1] = q;
  }
#pragma unroll
  for (int k = 6 + 2 * FD; k < L; ++k) r[k] = 0.f;
}

cudaError_t launch_pack_x2(int fd, void *rec, const double *x, const double *f, int n,
                           const double *origin, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  if (fd == 6)
    pack_sources_x2_kernel<6><<<(n + 255) / 256, 256, 0, st>>>(reinterpret_cast<float *>(rec), x,
                                                                f, n, origin);
  else
    pack_sources_x2_kernel<3><<<(n + 255) / 256, 256, 0, st>>>(reinterpret_cast<float *>(rec), x,
                                                                f, n, origin);
  count_launch();
  return cudaGetLastError();
}

size_t record_bytes(int fp32, int fd) {
  if (fp32) return fd == 6 ? 48 : 32;
  return fd == 6 ? 80 : 48;
}

int combo_of(int vd, int fda, int fdb) {
  if (vd == 6 && fda == 6 && fdb == 0) return C_SS;
  if (vd == 6 && fda == 3 && fdb == 0) return C_SB;
  if (vd == 3 && fda == 3 && fdb == 0) return C_BB;
  if (vd == 3 && fda == 6 && fdb == 0) return C_BS;
  if (vd == 6 && fda == 6 && fdb == 3) return C_SX;
  if (vd == 3 && fda == 6 && fdb == 3) return C_BX;
  return -1;
}

// Sources per split are a multiple of this (also the smallest split).
constexpr int kMinChunk = 64;

// Source splits for a launch of `ctas` target CTAs over n_src sources: the
// largest split count whose grid fits `waves` full waves (resident CTAs per
// SM x SMs), so no wave runs part-empty; at least two tiles per split.
static int choose_splits(int ctas, int n_src, int resident, int waves, int ts) {
  (void)ts;
  const long slots = (long)resident * num_sms() * std::max(1, waves);
  int s = (int)std::max(1L, slots / std::max(1, ctas));
  s = std::min(s, kMaxSplits);
  s = std::min(s, std::max(1, n_src / kMinChunk));
  return std::max(1, s);
}

cudaError_t launch_tile(const TileArgs &a_in, int vd, int fda, int fdb, TileTuning tune,
                        double *scratch, size_t scratch_elems, int mode, cudaStream_t st,
                        cudaEvent_t *ev) {
  TileArgs a = a_in;
  const int combo = combo_of(vd, fda, fdb);
  if (combo < 0) return cudaErrorInvalidValue;
  const int nvar = a.fp32 ? kNumVariantsF32 : kNumVariantsF64;
  if (tune.variant < 0 || tune.variant >= nvar) tune.variant = 0;
  if (tune.waves <= 0) tune.waves = 1;
  const TileVariant var = a.fp32 ? g_variants_f32[tune.variant] : g_variants_f64[tune.variant];
  const TileFn fn = !a.fp32 ? g_tile_f64[tune.variant][combo]
                    : var.x2 ? g_tile_f32x2[tune.variant - kNumVariantsF32Scalar][combo]
                             : g_tile_f32[tune.variant][combo];
  if (var.x2 && (a.src_a2 == nullptr || (a.n_b > 0 && a.src_b2 == nullptr)))
    return cudaErrorInvalidValue;
  if (a.n_tgt <= 0) return cudaSuccess;
  const int per_cta = var.block * var.tpt;
  const int ctas = (a.n_tgt + per_cta - 1) / per_cta;
  const int n_src = a.n_a + a.n_b;
  int resident = 1;
  cudaError_t qe = fn(a, dim3(0), st, &resident);
  if (qe != cudaSuccess) return qe;
  int splits = a.splits > 0 ? std::min(a.splits, kMaxSplits)
                            : choose_splits(ctas, n_src, resident, tune.waves, var.ts);
  if ((size_t)splits * a.n_tgt * vd > scratch_elems) splits = 1;
  if (n_src == 0) splits = 1;
  int chunk = (n_src + splits - 1) / splits;
  chunk = ((chunk + kMinChunk - 1) / kMinChunk) * kMinChunk;
  if (chunk == 0) chunk = kMinChunk;
  splits = std::max(1, (n_src + chunk - 1) / chunk);
  a.chunk = chunk;
  const dim3 grid(ctas, splits);
  cudaError_t e;
  if (ev) cudaEventRecord(ev[0], st);
  if (splits == 1) {
    a.mode = mode;
    e = fn(a, grid, st, nullptr);
    count_launch();
    if (ev) cudaEventRecord(ev[1], st);
    return e;
  }
  double *final_out = a.out;
  a.mode = OUT_PARTIAL;
  a.out = scratch;
  e = fn(a, grid, st, nullptr);
  count_launch();
  if (ev) cudaEventRecord(ev[1], st);
  if (e != cudaSuccess) return e;
  const int n_elems = a.n_tgt * vd;
  reduce_partials_kernel<<<(n_elems + 255) / 256, 256, 0, st>>>(
      final_out, scratch, n_elems, splits, mode == OUT_ACCUMULATE ? 1 : 0, a.skip);
  count_launch();
  return cudaGetLastError();
}

// The hashed grid of barrier_grid_bytes(): bucket counters (a power of two
// at least twice the sources), the overflow word, the buckets, the sums.
static BarGrid bar_grid(void *base, int n_src) {
  unsigned T = 64;
  while (T < 2u * (unsigned)n_src) T <<= 1;
  BarGrid g;
  char *p = static_cast<char *>(base);
  g.T = T;
  g.count = reinterpret_cast<unsigned *>(p);
  g.overflow = g.count + T;
  const size_t off_e = ((4 * (size_t)T + 4) + 15) / 16 * 16;
  g.entry = reinterpret_cast<float4 *>(p + off_e);
  g.sum = reinterpret_cast<double *>(p + off_e + 16 * (size_t)T * kBarSlots);
  return g;
}

size_t barrier_grid_bytes(int num_segs, int num_blobs) {
  const int n_src = num_segs + num_blobs;
  unsigned T = 64;
  while (T < 2u * (unsigned)n_src) T <<= 1;
  const size_t off_e = ((4 * (size_t)T + 4) + 15) / 16 * 16;
  return off_e + 16 * (size_t)T * kBarSlots + 24 * (size_t)std::max(n_src, 1);
}

cudaError_t launch_barrier(const BarrierArgs &a, cudaStream_t st) {
  const int n_src = a.num_segs + a.num_blobs;
  const int n_tgt = a.num_segs + (a.free_body ? a.num_blobs : 0);
  if (n_src <= 0 || n_tgt <= 0) return cudaSuccess;
  if (a.grid == nullptr) return cudaErrorInvalidValue;
  const BarGrid g = bar_grid(a.grid, n_src);
  cudaError_t e = cudaMemsetAsync(g.count, 0, 4 * ((size_t)g.T + 1), st);
  if (e != cudaSuccess) return e;
  bar_bin_kernel<<<(n_src + 255) / 256, 256, 0, st>>>(a, g);
  count_launch();
  bar_pair_kernel<<<(n_tgt + 127) / 128, 128, 0, st>>>(a, g);
  count_launch();
  bar_apply_kernel<<<(n_tgt + 255) / 256, 256, 0, st>>>(a, g);
  count_launch();
  return cudaGetLastError();
}

}  // namespace tfs
