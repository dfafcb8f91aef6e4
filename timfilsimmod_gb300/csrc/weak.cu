// weak.cu -- the weakly coupled filaments' segment product (the reference's
// weakly_coupled_filaments_rpy_mobility_solver: filament means and total
// forces computed on upload, weakly_coupled_filaments_rpy_mobility_solver.cu:
// 50-89, then Msf_mult, cuda_functions.cu:1129-1229, free space).
//
// Segment i of filament f receives, over the filaments j in order, the
// translation-only RPY pairs of its own filament's segments (j = f) or the
// Stokeslet of filament j's total force at its mean position (j != f):
//   v_i = (1/8 pi mu) [ sum_{k in f} RPY_tt(x_i - x_k) F_k
//                       + sum_{j != f} (Ftot_j / r + (r.Ftot_j) r / r^3) ],
// r = x_i - Z_j; the rotational velocities are zero. FP64, as the reference.
//
// Layout: the means and totals (one warp per filament, segments in order, a
// fixed shuffle tree: the reference sums them with atomic adds, in no fixed
// order) are staged per CTA in shared memory in tiles of BLOCK filaments;
// each thread owns one target segment.
#include <cuda_runtime.h>

#include "tfs_device.cuh"
#include "tfs_kernels.h"

namespace tfs {

namespace {

__device__ __forceinline__ double wc_warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Z[3 f] = sum_k x_{f,k} / nseg and Ft[3 f] = sum_k F_{f,k} (forces only),
// one warp per filament.
__global__ void fil_means_kernel(const double *__restrict__ x, const double *__restrict__ f,
                                 int nfil, int nseg, double *__restrict__ Z,
                                 double *__restrict__ Ft) {
  const int w = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (w >= nfil) return;
  double z[3] = {0.0, 0.0, 0.0}, t[3] = {0.0, 0.0, 0.0};
  for (int k = lane; k < nseg; k += 32) {
    const size_t s = (size_t)w * nseg + k;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      z[d] += x[3 * s + d] / (double)nseg;
      t[d] += f[6 * s + d];
    }
  }
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    z[d] = wc_warp_sum(z[d]);
    t[d] = wc_warp_sum(t[d]);
  }
  if (lane == 0)
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      Z[3 * (size_t)w + d] = z[d];
      Ft[3 * (size_t)w + d] = t[d];
    }
}

template <int BLOCK>
__global__ void __launch_bounds__(BLOCK) msf_kernel(const double *__restrict__ x,
                                                    const double *__restrict__ f,
                                                    const double *__restrict__ Z,
                                                    const double *__restrict__ Ft, int ns,
                                                    int nseg, int nfil, PairConst<double> pc,
                                                    double scale, double *__restrict__ v_out) {
  __shared__ double zs[BLOCK][3], fts[BLOCK][3];
  const int i = blockIdx.x * BLOCK + threadIdx.x;
  const bool active = i < ns;
  const int ii = active ? i : ns - 1;
  const int fil = ii / nseg;
  const double xi = x[3 * (size_t)ii], yi = x[3 * (size_t)ii + 1], zi = x[3 * (size_t)ii + 2];
  double v[3] = {0.0, 0.0, 0.0};
  for (int base = 0; base < nfil; base += BLOCK) {
    __syncthreads();
    const int jl = base + threadIdx.x;
    if (jl < nfil)
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        zs[threadIdx.x][d] = Z[3 * (size_t)jl + d];
        fts[threadIdx.x][d] = Ft[3 * (size_t)jl + d];
      }
    __syncthreads();
    const int cnt = min(BLOCK, nfil - base);
    for (int q = 0; q < cnt; ++q) {
      if (base + q == fil) {  // the own filament: RPY pairs, segments in order
        for (int k = 0; k < nseg; ++k) {
          const size_t jj = (size_t)fil * nseg + k;
          rpy_pair<double, 3, 3>(v, xi - x[3 * jj], yi - x[3 * jj + 1], zi - x[3 * jj + 2],
                                 f + 6 * jj, pc);
        }
      } else {  // another filament: the Stokeslet of its total force
        const double rx = xi - zs[q][0], ry = yi - zs[q][1], rz = zi - zs[q][2];
        const double rm1 = rsqrt_far(fma(rx, rx, fma(ry, ry, rz * rz)));
        const double rm3 = rm1 * rm1 * rm1;
        const double rF = fma(rx, fts[q][0], fma(ry, fts[q][1], rz * fts[q][2]));
        const double b = rm3 * rF;
        v[0] = fma(rm1, fts[q][0], fma(b, rx, v[0]));
        v[1] = fma(rm1, fts[q][1], fma(b, ry, v[1]));
        v[2] = fma(rm1, fts[q][2], fma(b, rz, v[2]));
      }
    }
  }
  if (!active) return;
  double *o = v_out + 6 * (size_t)i;
  o[0] = scale * v[0];
  o[1] = scale * v[1];
  o[2] = scale * v[2];
  o[3] = o[4] = o[5] = 0.0;
}

}  // namespace

cudaError_t launch_msf(const double *x_segs, const double *f_segs, int nfil, int nseg,
                       double a_seg, double mu, double *Z, double *Ft, double *v_segs,
                       cudaStream_t st) {
  if (nfil <= 0 || nseg <= 0) return cudaSuccess;
  const int warps_per_cta = 8;
  fil_means_kernel<<<(nfil + warps_per_cta - 1) / warps_per_cta, 32 * warps_per_cta, 0, st>>>(
      x_segs, f_segs, nfil, nseg, Z, Ft);
  count_launch();
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  PairConst<double> pc;
  pc.ai = pc.aj = a_seg;
  pc.asum2 = 4.0 * a_seg * a_seg;
  pc.s = 2.0 * a_seg * a_seg / 3.0;
  pc.s3 = -2.0 * a_seg * a_seg;
  constexpr int B = 128;
  const int ns = nfil * nseg;
  msf_kernel<B><<<(ns + B - 1) / B, B, 0, st>>>(x_segs, f_segs, Z, Ft, ns, nseg, nfil, pc,
                                              1.0 / (8.0 * kPi * mu), v_segs);
  count_launch();
  return cudaGetLastError();
}

}  // namespace tfs
