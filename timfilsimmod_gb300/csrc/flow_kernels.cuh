// flow_kernels.cuh -- the flow-field tile kernel template and its launch
// variants (instantiated in flow_f32.cu and flow_f64.cu, driven by flow.cu).
//
//   u(x) = prefac [ sum_segs ( F/r + (r.F) r / r^3 + (T x r) / r^3 )
//                 + sum_points ( F/r + (r.F) r / r^3 ) ],      r = x - x_j,
// (flow_velocities, src/flow_field/flow_field_evaluator.cu:13-228). With
// WALL the segment Stokeslet becomes the Blakelet of a no-slip wall at
// z = 0 (:83-116). "Points" are the blobs plus, when the net-force Stokeslet
// is removed (:125-143, :189-203), one point per body at its centre carrying
// minus the body's total source force: the reference subtracts
// S(x - X_b) f_j for every source j of body b, and since S(x - X_b) is the
// same for all of them that sum is S(x - X_b) (sum_j f_j).
#pragma once

#include <atomic>

#include <cuda_runtime.h>

#include "rpy_tile.cuh"

namespace tfs {

struct FlowArgs {
  const double *x_flow;
  int n_flow;
  const void *rec_segs;    // segment records (Rec<T,6>)
  int n_segs;
  const void *rec_points;  // blob and body-centre records (Rec<T,3>)
  int n_points;
  const double *origin;    // FP32 centring origin (z = 0 with the wall)
  double prefac;
  double *out;             // 3 * n_flow, or split partials
  int mode;                // OUT_ASSIGN or OUT_PARTIAL
  int chunk;               // sources per split
};

struct FlowVariant {
  int block, tpt, ts;  // threads per CTA, targets per thread, sources per tile
};
// Launch (grid.x > 0) or, with grid.x == 0, report resident CTAs per SM.
typedef cudaError_t (*FlowFn)(const FlowArgs &, dim3, cudaStream_t, int *resident);
constexpr int kFlowVariantsF32 = 4;
constexpr int kFlowVariantsF64 = 3;
extern const FlowVariant g_flow_variants_f32[kFlowVariantsF32];
extern const FlowVariant g_flow_variants_f64[kFlowVariantsF64];
extern const FlowFn g_flow_f32[kFlowVariantsF32][2];  // [variant][wall]
extern const FlowFn g_flow_f64[kFlowVariantsF64][2];

// v += sgn (rm1 f + rm3 (d.f) d): the Stokeslet of f at separation d
template <typename T>
__device__ __forceinline__ void stokeslet(T *v, T dx, T dy, T dz, T rm1, const T *f) {
  const T rm3 = rm1 * rm1 * rm1;
  const T w = rm3 * fma(dx, f[0], fma(dy, f[1], dz * f[2]));
  v[0] = fma(rm1, f[0], fma(w, dx, v[0]));
  v[1] = fma(rm1, f[1], fma(w, dy, v[1]));
  v[2] = fma(rm1, f[2], fma(w, dz, v[2]));
}

// One segment source: Stokeslet (Blakelet with WALL) + rotlet.
template <typename T, bool WALL>
__device__ __forceinline__ void flow_seg_pair(T *v, T xi, T yi, T zi, T sx, T sy, T sz,
                                              const T *f) {
  const T dx = xi - sx, dy = yi - sy, dz = zi - sz;
  const T rm1 = rsqrt_far(fma(dx, dx, fma(dy, dy, dz * dz)));
  const T rm3 = rm1 * rm1 * rm1;
  const T w = rm3 * fma(dx, f[0], fma(dy, f[1], dz * f[2]));
  // Stokeslet and rotlet (T x r) / r^3 (:118-123) share rm3
  v[0] = fma(rm1, f[0], fma(w, dx, fma(rm3, f[4] * dz - f[5] * dy, v[0])));
  v[1] = fma(rm1, f[1], fma(w, dy, fma(rm3, f[5] * dx - f[3] * dz, v[1])));
  v[2] = fma(rm1, f[2], fma(w, dz, fma(rm3, f[3] * dy - f[4] * dx, v[2])));
  if (WALL) {
    // minus the image Stokeslet at (sx, sy, -sz), then the source-doublet /
    // stresslet correction (:83-116); zi and sz are heights above the wall
    const T Rz = zi + sz;
    const T R2 = fma(dx, dx, fma(dy, dy, Rz * Rz));
    const T Rm1 = rsqrt_far(R2);
    const T Rm2 = Rm1 * Rm1;
    const T W = Rm2 * Rm1 * fma(dx, f[0], fma(dy, f[1], Rz * f[2]));
    v[0] = fma(-Rm1, f[0], fma(-W, dx, v[0]));
    v[1] = fma(-Rm1, f[1], fma(-W, dy, v[1]));
    v[2] = fma(-Rm1, f[2], fma(-W, Rz, v[2]));
    const T three_rz_zi = T(3) * Rz * zi;
    const T Dxx = (T(3) * dx * dx - R2) * zi;
    const T Dxy = T(3) * dx * dy * zi;
    const T Dxz = (R2 - three_rz_zi) * dx;
    const T Dyy = (T(3) * dy * dy - R2) * zi;
    const T Dyz = (R2 - three_rz_zi) * dy;
    const T Dzx = (three_rz_zi + R2) * dx;
    const T Dzy = (three_rz_zi + R2) * dy;
    const T Dzz = (R2 - T(3) * Rz * Rz) * zi;
    const T Dfac = T(2) * sz * Rm2 * Rm2 * Rm1;
    v[0] = fma(Dfac, Dxx * f[0] + Dxy * f[1] + Dxz * f[2], v[0]);
    v[1] = fma(Dfac, Dxy * f[0] + Dyy * f[1] + Dyz * f[2], v[1]);
    v[2] = fma(Dfac, Dzx * f[0] + Dzy * f[1] + Dzz * f[2], v[2]);
  }
}

template <typename T, int FD, bool WALL, int BLOCK, int TPT, int TS>
__device__ __forceinline__ void flow_range(T (&v)[TPT][3], const T (&xt)[TPT], const T (&yt)[TPT],
                                           const T (&zt)[TPT], const T *__restrict__ rec, int lo,
                                           int hi, T *smem, float *hl) {
  constexpr int L = Rec<T, FD>::len;
  constexpr int VEC_PER_REC = L * (int)sizeof(T) / 16;
  for (int base = lo; base < hi; base += TS) {
    const int cnt = min(TS, hi - base);
    __syncthreads();
    const int4 *src = reinterpret_cast<const int4 *>(rec + (size_t)base * L);
    int4 *dst = reinterpret_cast<int4 *>(smem);
    for (int q = threadIdx.x; q < cnt * VEC_PER_REC; q += BLOCK) dst[q] = __ldg(src + q);
    __syncthreads();
#pragma unroll 2
    for (int j = 0; j < cnt; ++j) {
      T sx, sy, sz, f[FD];
      RecLoad<T, FD>::get(smem + j * L, sx, sy, sz, f);
#pragma unroll
      for (int t = 0; t < TPT; ++t) {
        if (FD == 6) {
          flow_seg_pair<T, WALL>(v[t], xt[t], yt[t], zt[t], sx, sy, sz, f);
        } else {
          const T dx = xt[t] - sx, dy = yt[t] - sy, dz = zt[t] - sz;
          stokeslet(v[t], dx, dy, dz, rsqrt_far(fma(dx, dx, fma(dy, dy, dz * dz))), f);
        }
      }
    }
    Comp<T, 3, BLOCK, TPT>::fold(v, hl);
  }
}

template <typename T, bool WALL, int BLOCK, int TPT, int TS>
__global__ void __launch_bounds__(BLOCK) flow_kernel(const FlowArgs a) {
  constexpr int LMAX = Rec<T, 6>::len;
  constexpr bool kComp = sizeof(T) == 4;
  __shared__ __align__(16) T smem[TS * LMAX];
  __shared__ float hl[kComp ? 2 * TPT * 3 * BLOCK : 1];
  const double *origin = kComp ? a.origin : nullptr;
  const int tile0 = blockIdx.x * BLOCK * TPT;
  T xt[TPT], yt[TPT], zt[TPT], v[TPT][3];
#pragma unroll
  for (int t = 0; t < TPT; ++t) {
    int i = tile0 + t * BLOCK + threadIdx.x;
    i = i < a.n_flow ? i : a.n_flow - 1;
    xt[t] = load_target<T>(a.x_flow, i, 0, origin);
    yt[t] = load_target<T>(a.x_flow, i, 1, origin);
    zt[t] = load_target<T>(a.x_flow, i, 2, origin);
    v[t][0] = v[t][1] = v[t][2] = T(0);
  }
  if (kComp)
    for (int q = threadIdx.x; q < 2 * TPT * 3 * BLOCK; q += BLOCK) hl[q] = 0.f;
  const int n_src = a.n_segs + a.n_points;
  const int s0 = blockIdx.y * a.chunk, s1 = min(s0 + a.chunk, n_src);
  {
    const int lo = min(s0, a.n_segs), hi = min(s1, a.n_segs);
    if (lo < hi)
      flow_range<T, 6, WALL, BLOCK, TPT, TS>(v, xt, yt, zt,
                                             reinterpret_cast<const T *>(a.rec_segs), lo, hi,
                                             smem, hl);
  }
  {
    const int lo = max(s0 - a.n_segs, 0), hi = max(s1 - a.n_segs, 0);
    if (lo < hi)
      flow_range<T, 3, false, BLOCK, TPT, TS>(v, xt, yt, zt,
                                              reinterpret_cast<const T *>(a.rec_points), lo, hi,
                                              smem, hl);
  }
#pragma unroll
  for (int t = 0; t < TPT; ++t) {
    const int i = tile0 + t * BLOCK + threadIdx.x;
    if (i >= a.n_flow) continue;
    double *o = a.mode == OUT_PARTIAL ? a.out + ((size_t)blockIdx.y * a.n_flow + i) * 3
                                      : a.out + (size_t)i * 3;
#pragma unroll
    for (int k = 0; k < 3; ++k) o[k] = a.prefac * Comp<T, 3, BLOCK, TPT>::get(v, hl, t, k);
  }
}

template <typename T, bool WALL, int BLOCK, int TPT, int TS>
cudaError_t flow_launch_fn(const FlowArgs &a, dim3 grid, cudaStream_t st, int *resident) {
  static std::atomic<int> occupancy[kMaxDevices];  // set once per device; threads may race
  auto kern = flow_kernel<T, WALL, BLOCK, TPT, TS>;
  int dev = 0;
  cudaError_t e0 = cudaGetDevice(&dev);
  if (e0 != cudaSuccess) return e0;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  if (occupancy[dev].load() == 0) {
    int occ = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, BLOCK, 0);
    if (e != cudaSuccess) return e;
    occupancy[dev].store(occ < 1 ? 1 : occ);
  }
  if (resident) *resident = occupancy[dev].load();
  if (grid.x == 0) return cudaSuccess;  // query only
  kern<<<grid, BLOCK, 0, st>>>(a);
  return cudaGetLastError();
}

#define TFS_FLOW_ROW(T, B, P, S) \
  { flow_launch_fn<T, false, B, P, S>, flow_launch_fn<T, true, B, P, S> }

}  // namespace tfs
