// rpy_ff.cu -- the blob-blob product M_bb f in float-float arithmetic: the
// product FP32C iterative refinement computes its residuals with.
//
// The refinement's inner solves run on FP32 pair sums (relative error ~1e-7),
// so its residual r = b - A x must be computed to well below the 1e-8 target
// of the linear solve. Plain FP64 pair arithmetic does that at the FP64 rate
// (1/64 of FP32 on this GPU); here every pair quantity is carried as an
// unevaluated sum of two FP32 numbers (h + l, about 48 significant bits),
// with the error-free transformations of Knuth (TwoSum), Dekker
// (Fast2Sum) and the FMA-based exact product, as in the double-word
// arithmetic of Dekker (1971) and the DSFUN library (Bailey), whose error
// bounds are analysed by Joldes, Muller and Popescu (2017). A pair costs about
// 230 FP32 instructions instead of about 45 FP64 ones. Each pair term is
// accurate to about 2^-46 relative (positions carry 48 bits relative to the
// centring origin) and sums are accumulated compensated, so the product's
// error is a small multiple of 2^-46 times the sum of |pair terms|: measured
// 4e-14 of the largest component on 642 overlapping blobs and 2e-12 on 10 242
// blobs with random forces, against FP64 -- far below the 1e-8 relative
// residual the refinement works to.
//
// Pair formula: the reference's blob-blob RPY pair (cuda_functions.cu:476-549
// with the pair function :205-356, equal radii a), in units of 1/(8 pi mu):
//   far  (r > 2a):  v += (1/r + s/r^3) F + (1/r^3 - 3 s/r^5) (d.F) d,  s = 2a^2/3
//   near (0 < r <= 2a): v += (4/(3a) - 3r/(8a^2)) F + (d.F) d / (8 a^2 r)
//   self (r = 0):   v += 4/(3a) F
// with d = x_target - x_source.
//
// The reciprocal square root: the FP32 hardware estimate y0 of r^-2 refined
// by one Newton-type step y = y0 (1 + e/2 + 3e^2/8), e = 1 - r^2 y0^2, where
// 1 - r^2 y0^2 is formed exactly enough from the exact products y0^2 and
// r^2 y0^2 (Markstein's refinement of the reciprocal square root).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "ff_arith.cuh"
#include "tfs_kernels.h"

namespace tfs {

namespace {

using namespace ff;

// One source record: position (relative to the origin) and force, as three
// float4: (xh, yh, zh, fxh), (fyh, fzh, xl, yl), (zl, fxl, fyl, fzl).
__global__ void pack_ff_kernel(float4 *__restrict__ rec, const double *__restrict__ x,
                               const double *__restrict__ f, const double *__restrict__ origin,
                               int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  FF p[3], q[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    p[k] = ff_split(x[3 * (size_t)i + k] - origin[k]);
    q[k] = ff_split(f[3 * (size_t)i + k]);
  }
  rec[3 * (size_t)i + 0] = make_float4(p[0].h, p[1].h, p[2].h, q[0].h);
  rec[3 * (size_t)i + 1] = make_float4(q[1].h, q[2].h, p[0].l, p[1].l);
  rec[3 * (size_t)i + 2] = make_float4(p[2].l, q[0].l, q[1].l, q[2].l);
}

struct FFConst {
  FF s, s3;       // 2a^2/3, -2a^2
  FF asum2;       // (2a)^2: r^2 above it is the far field
  FF self;        // 4/(3a)
  FF near_r;      // -3/(8a^2): the near-field coefficient of r
  FF near_d;      // 1/(8a^2): the near-field coefficient of (d.F) d / r
};

struct FFArgs {
  const double *x;       // targets: blob positions (3 n)
  const float4 *rec;     // sources: 3 n float4
  const double *origin;  // [3]
  int n, chunk;
  FFConst k;
  double scale;          // 1 / (8 pi mu)
  double *out;           // [gridDim.y][n][3]
};

// One pair into v (units of 1/(8 pi mu)).
__device__ __forceinline__ void ff_pair(FF (&v)[3], const FF (&xt)[3], const FF (&xs)[3],
                                        const FF (&f)[3], const FFConst &k) {
  const FF dx = ff_sub(xt[0], xs[0]), dy = ff_sub(xt[1], xs[1]), dz = ff_sub(xt[2], xs[2]);
  // r^2 (all terms positive)
  const float px = __fmul_rn(dx.h, dx.h), py = __fmul_rn(dy.h, dy.h), pz = __fmul_rn(dz.h, dz.h);
  const float ex = fmaf(__fadd_rn(dx.h, dx.h), dx.l, fmaf(dx.h, dx.h, -px));
  const float ey = fmaf(__fadd_rn(dy.h, dy.h), dy.l, fmaf(dy.h, dy.h, -py));
  const float ez = fmaf(__fadd_rn(dz.h, dz.h), dz.l, fmaf(dz.h, dz.h, -pz));
  FF r2 = ff_two_sum(px, py);
  const float t = __fadd_rn(r2.l, __fadd_rn(ex, ey));
  r2 = ff_two_sum(r2.h, pz);
  r2 = ff_fast_two_sum(r2.h, __fadd_rn(r2.l, __fadd_rn(t, ez)));
  FF A, B;
  const bool far = r2.h > k.asum2.h || (r2.h == k.asum2.h && r2.l > k.asum2.l);
  if (r2.h == 0.f) {  // self
    A = k.self;
    B = {0.f, 0.f};
  } else {
    // 1/r
    const float y0 = rsqrtf(r2.h);
    const float qh = __fmul_rn(y0, y0);
    const float ql = fmaf(y0, y0, -qh);
    const float uh = __fmul_rn(r2.h, qh);
    const float ul = fmaf(r2.h, ql, fmaf(r2.l, qh, fmaf(r2.h, qh, -uh)));
    const float e = __fsub_rn(__fsub_rn(1.0f, uh), ul);
    const float c = __fmul_rn(__fmul_rn(y0, e), fmaf(e, 0.375f, 0.5f));
    const FF rm1 = ff_fast_two_sum(y0, c);
    if (far) {
      const FF rm2 = ff_mul(rm1, rm1);
      const FF rm3 = ff_mul(rm1, rm2);
      const FF rm5 = ff_mul(rm3, rm2);
      A = ff_add(rm1, ff_mul(k.s, rm3));
      B = ff_add(rm3, ff_mul(k.s3, rm5));
    } else {
      const FF r = ff_mul(r2, rm1);
      A = ff_add(k.self, ff_mul(k.near_r, r));
      B = ff_mul(k.near_d, rm1);
    }
  }
  const FF dF = ff_add(ff_add(ff_mul(dx, f[0]), ff_mul(dy, f[1])), ff_mul(dz, f[2]));
  const FF Bd = ff_mul(B, dF);
  ff_acc(v[0], ff_mul(A, f[0]));
  ff_acc(v[0], ff_mul(Bd, dx));
  ff_acc(v[1], ff_mul(A, f[1]));
  ff_acc(v[1], ff_mul(Bd, dy));
  ff_acc(v[2], ff_mul(A, f[2]));
  ff_acc(v[2], ff_mul(Bd, dz));
}

// grid = (target CTAs, source splits); BLOCK threads, TPT targets each;
// sources staged TS at a time in shared memory (read by all threads alike).
template <int BLOCK, int TPT, int TS>
__global__ void __launch_bounds__(BLOCK) bb_ff_kernel(const FFArgs a) {
  __shared__ float4 src[3 * TS];
  const int n = a.n;
  const int tile0 = blockIdx.x * BLOCK * TPT;
  FF xt[TPT][3], v[TPT][3];
#pragma unroll
  for (int t = 0; t < TPT; ++t) {
    int i = tile0 + t * BLOCK + threadIdx.x;
    i = i < n ? i : n - 1;  // duplicate the last target; not written
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      xt[t][k] = ff_split(a.x[3 * (size_t)i + k] - a.origin[k]);
      v[t][k] = {0.f, 0.f};
    }
  }
  const int s0 = blockIdx.y * a.chunk;
  const int s1 = min(s0 + a.chunk, n);
  for (int base = s0; base < s1; base += TS) {
    const int m = min(TS, s1 - base);
    __syncthreads();
    for (int q = threadIdx.x; q < 3 * m; q += BLOCK) src[q] = a.rec[3 * (size_t)base + q];
    __syncthreads();
    for (int j = 0; j < m; ++j) {
      const float4 r0 = src[3 * j], r1 = src[3 * j + 1], r2 = src[3 * j + 2];
      const FF xs[3] = {{r0.x, r1.z}, {r0.y, r1.w}, {r0.z, r2.x}};
      const FF f[3] = {{r0.w, r2.y}, {r1.x, r2.z}, {r1.y, r2.w}};
#pragma unroll
      for (int t = 0; t < TPT; ++t) ff_pair(v[t], xt[t], xs, f, a.k);
    }
  }
#pragma unroll
  for (int t = 0; t < TPT; ++t) {
    const int i = tile0 + t * BLOCK + threadIdx.x;
    if (i >= n) continue;
    double *o = a.out + ((size_t)blockIdx.y * n + i) * 3;
#pragma unroll
    for (int k = 0; k < 3; ++k) o[k] = a.scale * ((double)v[t][k].h + (double)v[t][k].l);
  }
}

constexpr int kFFBlock = 128, kFFTpt = 2, kFFTs = 128;

FF host_split(double x) {
  const float h = (float)x;
  return {h, (float)(x - (double)h)};
}

}  // namespace

size_t ff_record_bytes() { return 3 * sizeof(float4); }

cudaError_t launch_bb_ff(const double *x_blobs, const double *f_blobs, int nb,
                         const double *origin, double a_blob, double scale, void *rec, double *out,
                         double *scratch, size_t scratch_elems, cudaStream_t st, cudaEvent_t *ev) {
  if (nb <= 0) return cudaSuccess;
  float4 *r = static_cast<float4 *>(rec);
  pack_ff_kernel<<<(nb + 255) / 256, 256, 0, st>>>(r, x_blobs, f_blobs, origin, nb);
  count_launch();
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  FFArgs a{};
  a.x = x_blobs;
  a.rec = r;
  a.origin = origin;
  a.n = nb;
  a.scale = scale;
  const double a2 = a_blob * a_blob;
  a.k.s = host_split(2.0 * a2 / 3.0);
  a.k.s3 = host_split(-2.0 * a2);
  a.k.asum2 = host_split(4.0 * a2);
  a.k.self = host_split(4.0 / (3.0 * a_blob));
  a.k.near_r = host_split(-3.0 / (8.0 * a2));
  a.k.near_d = host_split(1.0 / (8.0 * a2));
  // source splits: about four CTAs per SM in all, sources per split a
  // multiple of the tile, partial sums within the scratch
  const int ctas = (nb + kFFBlock * kFFTpt - 1) / (kFFBlock * kFFTpt);
  int splits = std::max(1, (4 * num_sms() + ctas - 1) / ctas);
  splits = (int)std::min<size_t>({(size_t)splits, (size_t)kMaxSplits,
                                  scratch_elems / (3 * (size_t)nb)});
  splits = std::max(1, splits);
  int chunk = (nb + splits - 1) / splits;
  chunk = ((chunk + 31) / 32) * 32;
  splits = (nb + chunk - 1) / chunk;
  a.chunk = chunk;
  a.out = splits == 1 ? out : scratch;
  if (ev) cudaEventRecord(ev[0], st);
  bb_ff_kernel<kFFBlock, kFFTpt, kFFTs><<<dim3(ctas, splits), kFFBlock, 0, st>>>(a);
  count_launch();
  if (ev) cudaEventRecord(ev[1], st);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if (splits == 1) return cudaSuccess;
  return launch_reduce_partials(out, scratch, 3 * nb, splits, 0, st);
}

}  // namespace tfs
