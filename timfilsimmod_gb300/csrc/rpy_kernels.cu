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

// Two passes over all particles, kOriginCTAs CTAs each: pass 0 sums the
// positions (the mean goes to out[0..2]), pass 1 takes the largest
// |x_k - o_k| (out[3]). Per-CTA partials live in out[4..], the last CTA to
// finish combines them in CTA order (deterministic).
__global__ void __launch_bounds__(256) origin_kernel(const double *__restrict__ xa, int na,
                                                     const double *__restrict__ xb, int nb,
                                                     double *__restrict__ out /* [4 + 4 kOriginCTAs] */,
                                                     unsigned *__restrict__ counter, int pass) {
  __shared__ double red[256][3];
  __shared__ bool last;
  const int tid = threadIdx.x, n = na + nb;
  double *part = out + 4;
  double s[3] = {0, 0, 0};
  double o[3] = {0, 0, 0};
  if (pass == 1)
    for (int k = 0; k < 3; ++k) o[k] = out[k];
  for (int i = blockIdx.x * blockDim.x + tid; i < n; i += gridDim.x * blockDim.x) {
    const double *x = i < na ? xa + 3 * (size_t)i : xb + 3 * (size_t)(i - na);
    if (pass == 0) {
      for (int k = 0; k < 3; ++k) s[k] += x[k];
    } else {
      for (int k = 0; k < 3; ++k) s[0] = fmax(s[0], fabs(x[k] - o[k]));
    }
  }
  for (int k = 0; k < 3; ++k) red[tid][k] = s[k];
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (tid < w) {
      if (pass == 0)
        for (int k = 0; k < 3; ++k) red[tid][k] += red[tid + w][k];
      else
        red[tid][0] = fmax(red[tid][0], red[tid + w][0]);
    }
    __syncthreads();
  }
  if (tid == 0) {
    if (pass == 0)
      for (int k = 0; k < 3; ++k) part[3 * blockIdx.x + k] = red[0][k];
    else
      part[3 * kOriginCTAs + blockIdx.x] = red[0][0];
    __threadfence();
    last = atomicAdd(counter + pass, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last || tid != 0) return;
  __threadfence();
  if (pass == 0) {
    double t[3] = {0, 0, 0};
    for (int c = 0; c < (int)gridDim.x; ++c)
      for (int k = 0; k < 3; ++k) t[k] += __ldcg(part + 3 * c + k);
    for (int k = 0; k < 3; ++k) out[k] = n > 0 ? t[k] / n : 0.0;
  } else {
    double m = 0.0;
    for (int c = 0; c < (int)gridDim.x; ++c) m = fmax(m, __ldcg(part + 3 * kOriginCTAs + c));
    out[3] = m;
  }
  counter[pass] = 0;
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
// A candidate test on FP32 positions (relative to the origin, with a margin
// that bounds their rounding) discards the vast majority of pairs on the FP32
// pipe; candidates are then tested and evaluated in FP64 exactly as the
// reference does. Targets are segments (kind 0: skip self and the nearest
// neighbours on the same filament; adds into f_segs) or blobs (kind 1: skip
// self; assigns f_blobs_repulsion).
// ---------------------------------------------------------------------------
// Bounds of the FP32 origin-relative positions of each tile of BLOCK
// consecutive sources (segments then blobs): boxes[6 t ..] = min xyz, max xyz.
template <int BLOCK>
__global__ void __launch_bounds__(BLOCK) tile_box_kernel(const BarrierArgs a, int n_src) {
  __shared__ float red[BLOCK / 32][6];
  const int j = blockIdx.x * BLOCK + threadIdx.x;
  float v[6] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
  if (j < n_src) {
    const double *xs = j < a.num_segs ? a.x_segs + 3 * (size_t)j
                                      : a.x_blobs + 3 * (size_t)(j - a.num_segs);
    for (int k = 0; k < 3; ++k) v[k] = v[k + 3] = float(xs[k] - a.origin[k]);
  }
  for (int o = 16; o > 0; o >>= 1)
    for (int k = 0; k < 6; ++k) {
      const float w = __shfl_xor_sync(0xffffffffu, v[k], o);
      v[k] = k < 3 ? fminf(v[k], w) : fmaxf(v[k], w);
    }
  if ((threadIdx.x & 31) == 0)
    for (int k = 0; k < 6; ++k) red[threadIdx.x >> 5][k] = v[k];
  __syncthreads();
  if (threadIdx.x < 6) {
    const int k = threadIdx.x;
    float b = red[0][k];
    for (int w = 1; w < BLOCK / 32; ++w) b = k < 3 ? fminf(b, red[w][k]) : fmaxf(b, red[w][k]);
    a.boxes[6 * (size_t)blockIdx.x + k] = b;
  }
}

template <int BLOCK>
__global__ void __launch_bounds__(BLOCK) barrier_kernel(const BarrierArgs a) {
  static_assert(BLOCK == 128, "source tiles are the 128-source tiles of tile_box_kernel");
  __shared__ double sxd[BLOCK][3];
  __shared__ float sxf[BLOCK][3];
  __shared__ float cbox_w[BLOCK / 32][6], cbox[6];
  const int i = blockIdx.x * BLOCK + threadIdx.x;
  const int n_tgt = a.target_blobs ? a.num_blobs : a.num_segs;
  const bool active = i < n_tgt;
  const double *xt = a.target_blobs ? a.x_blobs : a.x_segs;
  const int ii = active ? i : 0;
  const double o0 = a.origin[0], o1 = a.origin[1], o2 = a.origin[2];
  const double extent = a.origin[3];
  const double xi = n_tgt > 0 ? xt[3 * (size_t)ii] : 0.0;
  const double yi = n_tgt > 0 ? xt[3 * (size_t)ii + 1] : 0.0;
  const double zi = n_tgt > 0 ? xt[3 * (size_t)ii + 2] : 0.0;
  const float xif = float(xi - o0), yif = float(yi - o1), zif = float(zi - o2);
  // |d_fp32 - d| <= 2 sqrt(3) extent 2^-24 =: delta (each coordinate is
  // rounded once to FP32, relative 2^-24), plus FP32 arithmetic in d^2.
  const float delta = float(4.0 * extent * 5.9604644775390625e-08 + 1e-30);
  const int fil_i = active && !a.target_blobs ? i / a.nseg : -1;
  const double emag = a.repulsive_force_factor * (double)a.end_force_magnitude;
  // contact distances of the two source kinds and their FP32 candidate
  // thresholds (squared, with the rounding margin), hoisted out of the loop
  const double asum_seg = a.target_blobs ? a.a_blob + a.a_seg : 2.0 * a.a_seg;
  const double asum_blob = a.target_blobs ? 2.0 * a.a_blob : a.a_seg + a.a_blob;
  const float thr_seg = float(1.1 * asum_seg) + 2.f * delta;
  const float thr_blob = float(1.1 * asum_blob) + 2.f * delta;
  const float thr2_seg = thr_seg * thr_seg * 1.0001f, thr2_blob = thr_blob * thr_blob * 1.0001f;
  const int n_src = a.num_segs + a.num_blobs;
  // this CTA's share of the sources (grid.y splits them)
  const int s0 = blockIdx.y * a.chunk;
  const int s1 = min(s0 + a.chunk, n_src);
  // bounds of this CTA's targets; a source tile whose bounds lie farther than
  // the larger candidate threshold (with a 0.1% margin over the FP32
  // rounding of both tests) has no pair the filter below would pass, and is
  // skipped by the whole CTA
  const float cull2 = 1.001f * fmaxf(thr2_seg, thr2_blob);
  if (a.boxes != nullptr) {
    float v[6] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
    if (active) {
      v[0] = v[3] = xif;
      v[1] = v[4] = yif;
      v[2] = v[5] = zif;
    }
    for (int o = 16; o > 0; o >>= 1)
      for (int k = 0; k < 6; ++k) {
        const float w = __shfl_xor_sync(0xffffffffu, v[k], o);
        v[k] = k < 3 ? fminf(v[k], w) : fmaxf(v[k], w);
      }
    if ((threadIdx.x & 31) == 0)
      for (int k = 0; k < 6; ++k) cbox_w[threadIdx.x >> 5][k] = v[k];
    __syncthreads();
    if (threadIdx.x < 6) {
      const int k = threadIdx.x;
      float b = cbox_w[0][k];
      for (int w = 1; w < BLOCK / 32; ++w) b = k < 3 ? fminf(b, cbox_w[w][k]) : fmaxf(b, cbox_w[w][k]);
      cbox[k] = b;
    }
    __syncthreads();
  }
  double fx = 0.0, fy = 0.0, fz = 0.0;
  for (int base = s0; base < s1; base += BLOCK) {
    if (a.boxes != nullptr) {  // CTA-uniform: the same values in every thread
      const float *tb = a.boxes + 6 * (size_t)(base / BLOCK);
      const float gx = fmaxf(0.f, fmaxf(tb[0] - cbox[3], cbox[0] - tb[3]));
      const float gy = fmaxf(0.f, fmaxf(tb[1] - cbox[4], cbox[1] - tb[4]));
      const float gz = fmaxf(0.f, fmaxf(tb[2] - cbox[5], cbox[2] - tb[5]));
      if (gx * gx + gy * gy + gz * gz >= cull2) continue;
    }
    const int j = base + threadIdx.x;
    __syncthreads();
    if (j < s1) {
      const double *xs = j < a.num_segs ? a.x_segs + 3 * (size_t)j
                                        : a.x_blobs + 3 * (size_t)(j - a.num_segs);
      sxd[threadIdx.x][0] = xs[0];
      sxd[threadIdx.x][1] = xs[1];
      sxd[threadIdx.x][2] = xs[2];
      sxf[threadIdx.x][0] = float(xs[0] - o0);
      sxf[threadIdx.x][1] = float(xs[1] - o1);
      sxf[threadIdx.x][2] = float(xs[2] - o2);
    }
    __syncthreads();
    if (!active) continue;
    const int cnt = min(BLOCK, s1 - base);
    for (int q = 0; q < cnt; ++q) {
      const int jj = base + q;
      const bool src_is_seg = jj < a.num_segs;
      const float dxf = xif - sxf[q][0], dyf = yif - sxf[q][1], dzf = zif - sxf[q][2];
      const float d2f = dxf * dxf + dyf * dyf + dzf * dzf;
      if (d2f >= (src_is_seg ? thr2_seg : thr2_blob)) continue;
      const double asum = src_is_seg ? asum_seg : asum_blob;
      // exclusions, :1319 and :1410
      if (a.target_blobs) {
        if (i + a.num_segs == jj) continue;
      } else if (src_is_seg) {
        const int fil_j = jj / a.nseg;
        if (fil_i == fil_j && (i - jj <= 1 && jj - i <= 1)) continue;
      }
      const double dx = xi - sxd[q][0], dy = yi - sxd[q][1], dz = zi - sxd[q][2];
      const double dist = sqrt(dx * dx + dy * dy + dz * dz);
      if (dist < 1.1 * asum) {
        const double chi = 10.0 / asum;
        double fac = fmin(1.0, 1.0 - chi * (dist - asum));
        fac *= emag * fac * fac * fac;
        const double dm1 = 1.0 / dist;
        fx += fac * dx * dm1;
        fy += fac * dy * dm1;
        fz += fac * dz * dm1;
      }
    }
  }
  if (!active) return;
  if (a.splits > 1) {
    double *o = a.scratch + ((size_t)blockIdx.y * n_tgt + i) * 3;
    o[0] = fx;
    o[1] = fy;
    o[2] = fz;
    return;
  }
  if (a.target_blobs) {
    a.f_blobs_repulsion[3 * (size_t)i] = fx;
    a.f_blobs_repulsion[3 * (size_t)i + 1] = fy;
    a.f_blobs_repulsion[3 * (size_t)i + 2] = fz;
  } else {
    a.f_segs[6 * (size_t)i] += fx;
    a.f_segs[6 * (size_t)i + 1] += fy;
    a.f_segs[6 * (size_t)i + 2] += fz;
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
  for (int pass = 0; pass < 2; ++pass) {
    origin_kernel<<<ctas, 256, 0, st>>>(xa, na, xb, nb, out, counter, pass);
    count_launch();
  }
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

// Split barrier forces: out[stride * i + k] (+= or =) sum over splits s in
// order of partial[s][i][k], k < 3.
__global__ void barrier_reduce_kernel(double *__restrict__ out, int stride, int accumulate,
                                      const double *__restrict__ partial, int n_tgt,
                                      int splits) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= 3 * n_tgt) return;
  const int i = e / 3, k = e - 3 * i;
  double s = 0.0;
  for (int p = 0; p < splits; ++p) s += partial[(size_t)p * 3 * n_tgt + e];
  double *o = out + (size_t)stride * i + k;
  *o = accumulate ? *o + s : s;
}

// One target kind: grid = target CTAs x source splits, the split count chosen
// for about eight CTAs per SM; partial forces summed in split order.
static cudaError_t barrier_launch(BarrierArgs a, int target_blobs, cudaStream_t st) {
  constexpr int B = 128;
  a.target_blobs = target_blobs;
  const int n_tgt = target_blobs ? a.num_blobs : a.num_segs;
  const int n_src = a.num_segs + a.num_blobs;
  const int ctas = (n_tgt + B - 1) / B;
  int splits = std::max(1, (8 * num_sms() + ctas - 1) / ctas);
  splits = std::min(splits, kMaxSplits);
  splits = std::min(splits, std::max(1, n_src / (2 * B)));
  if (a.scratch == nullptr || (size_t)splits * 3 * n_tgt > a.scratch_elems) splits = 1;
  int chunk = (n_src + splits - 1) / splits;
  chunk = std::max(B, ((chunk + B - 1) / B) * B);
  splits = std::max(1, (n_src + chunk - 1) / chunk);
  a.chunk = chunk;
  a.splits = splits;
  barrier_kernel<B><<<dim3(ctas, splits), B, 0, st>>>(a);
  count_launch();
  if (splits > 1) {
    barrier_reduce_kernel<<<(3 * n_tgt + 255) / 256, 256, 0, st>>>(
        target_blobs ? a.f_blobs_repulsion : a.f_segs, target_blobs ? 3 : 6,
        target_blobs ? 0 : 1, a.scratch, n_tgt, splits);
    count_launch();
  }
  return cudaGetLastError();
}

cudaError_t launch_barrier(const BarrierArgs &a, cudaStream_t st) {
  cudaError_t e = cudaSuccess;
  const int n_src = a.num_segs + a.num_blobs;
  if (a.boxes != nullptr && n_src > 0) {
    tile_box_kernel<128><<<(n_src + 127) / 128, 128, 0, st>>>(a, n_src);
    count_launch();
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  if (a.num_segs > 0 && (e = barrier_launch(a, 0, st)) != cudaSuccess) return e;
  if (a.free_body && a.num_blobs > 0) e = barrier_launch(a, 1, st);
  return e;
}

}  // namespace tfs
