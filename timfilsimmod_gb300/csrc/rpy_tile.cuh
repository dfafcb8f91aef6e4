// rpy_tile.cuh -- the all-pairs RPY tile kernel template (see rpy_kernels.cu
// for the layout and work decomposition) and the source-record formats.
#pragma once

#include <atomic>

#include <cuda_runtime.h>

#include "tfs_device.cuh"
#include "tfs_kernels.h"

namespace tfs {

template <typename T, int FD>
struct Rec;
template <>
struct Rec<double, 6> {
  static constexpr int len = 10;
};
template <>
struct Rec<double, 3> {
  static constexpr int len = 6;
};
template <>
struct Rec<float, 6> {
  static constexpr int len = 12;
};
template <>
struct Rec<float, 3> {
  static constexpr int len = 8;
};

// ---------------------------------------------------------------------------
// Source records from shared memory, with 16-byte vector loads (records are
// 16-byte aligned; every lane of a warp reads the same record: broadcast).
// ---------------------------------------------------------------------------
template <typename T, int FD>
struct RecLoad;

template <>
struct RecLoad<float, 6> {
  __device__ static void get(const float *r, float &x, float &y, float &z, float (&f)[6]) {
    const float4 a = reinterpret_cast<const float4 *>(r)[0];
    const float4 b = reinterpret_cast<const float4 *>(r)[1];
    const float4 c = reinterpret_cast<const float4 *>(r)[2];
    x = a.x; y = a.y; z = a.z; f[0] = a.w;
    f[1] = b.x; f[2] = b.y; f[3] = b.z; f[4] = b.w;
    f[5] = c.x;
  }
};
template <>
struct RecLoad<float, 3> {
  __device__ static void get(const float *r, float &x, float &y, float &z, float (&f)[3]) {
    const float4 a = reinterpret_cast<const float4 *>(r)[0];
    const float4 b = reinterpret_cast<const float4 *>(r)[1];
    x = a.x; y = a.y; z = a.z; f[0] = a.w;
    f[1] = b.x; f[2] = b.y;
  }
};
template <>
struct RecLoad<double, 6> {
  __device__ static void get(const double *r, double &x, double &y, double &z, double (&f)[6]) {
    const double2 *q = reinterpret_cast<const double2 *>(r);
    const double2 a = q[0], b = q[1], c = q[2], d = q[3], e = q[4];
    x = a.x; y = a.y; z = b.x; f[0] = b.y;
    f[1] = c.x; f[2] = c.y; f[3] = d.x; f[4] = d.y; f[5] = e.x;
  }
};
template <>
struct RecLoad<double, 3> {
  __device__ static void get(const double *r, double &x, double &y, double &z, double (&f)[3]) {
    const double2 *q = reinterpret_cast<const double2 *>(r);
    const double2 a = q[0], b = q[1], c = q[2];
    x = a.x; y = a.y; z = b.x; f[0] = b.y;
    f[1] = c.x; f[2] = c.y;
  }
};

template <typename T>
__device__ __forceinline__ T load_target(const double *x, int i, int k, const double *origin) {
  return T(x[3 * (size_t)i + k] - (origin ? origin[k] : 0.0));
}

// Compensated running sums of the FP32 path live in shared memory (they are
// touched once per tile), laid out [TPT][VD][BLOCK] so a warp's accesses are
// conflict-free. The FP64 path accumulates straight into its registers.
template <typename T, int VD, int BLOCK, int TPT>
struct Comp {
  __device__ static void fold(T (&)[TPT][VD], float *) {}
  __device__ static double get(const T (&v)[TPT][VD], const float *, int t, int k) {
    return (double)v[t][k];
  }
};
template <int VD, int BLOCK, int TPT>
struct Comp<float, VD, BLOCK, TPT> {
  __device__ static void fold(float (&v)[TPT][VD], float *hl) {
#pragma unroll
    for (int t = 0; t < TPT; ++t)
#pragma unroll
      for (int k = 0; k < VD; ++k) {
        float *hi = hl + ((t * VD + k) * 2) * BLOCK + threadIdx.x;
        float *lo = hi + BLOCK;
        float h = *hi, l = *lo;
        two_sum(h, l, v[t][k]);
        *hi = h;
        *lo = l;
        v[t][k] = 0.f;
      }
  }
  __device__ static double get(const float (&)[TPT][VD], const float *hl, int t, int k) {
    const float *hi = hl + ((t * VD + k) * 2) * BLOCK + threadIdx.x;
    return (double)hi[0] + (double)hi[BLOCK];
  }
};

// The exact three-regime pairs of one tile that the far-field pass skipped
// (r^2 <= (ai+aj)^2: self, overlapping or touching particles): a lane whose
// target met one rescans the tile and evaluates them in source order.
template <typename T, int VD, int FD, int TPT>
__device__ __forceinline__ void near_pass(T (&v)[TPT][VD], const T (&xt)[TPT], const T (&yt)[TPT],
                                          const T (&zt)[TPT], const unsigned (&nf)[TPT],
                                          const T *smem, int cnt, const PairConst<T> &pc) {
  constexpr int L = Rec<T, FD>::len;
#pragma unroll
  for (int t = 0; t < TPT; ++t) {
    if (nf[t] == 0u) continue;
    for (int j = 0; j < cnt; ++j) {
      T sx, sy, sz, f[FD];
      RecLoad<T, FD>::get(smem + j * L, sx, sy, sz, f);
      const T dx = xt[t] - sx, dy = yt[t] - sy, dz = zt[t] - sz;
      const T r2 = fma(dx, dx, fma(dy, dy, dz * dz));
      if (!(r2 > pc.asum2)) near_pair<T, VD, FD>(v[t], dx, dy, dz, r2, f, pc);
    }
  }
}

// Sum the sources [lo, hi) of one record array into v.
//
// Far-field pass (every pair): the far-field formula without a branch; pairs
// inside the contact distance (r^2 <= (ai+aj)^2, which includes self pairs)
// get 1/r = 0, which zeroes every far-field term, and set a per-target flag
// (one logic op per pair). After the tile, a flagged lane rescans it and adds
// those pairs with the exact three-regime formula (near_pass). In the swimmer
// configurations only the tiles that hold a target's own particle or a
// touching neighbour flag anything.
//
// compute = false (warp-uniform): the warp has no target of its own and only
// helps stage the tiles.
template <typename T, int VD, int FD, int BLOCK, int TPT, int TS>
__device__ __forceinline__ void sum_source_range(T (&v)[TPT][VD], const T (&xt)[TPT],
                                                 const T (&yt)[TPT], const T (&zt)[TPT],
                                                 const T *__restrict__ rec, int lo, int hi,
                                                 const PairConst<T> &pc, T *smem, float *hl,
                                                 bool compute = true) {
  static_assert(TS <= 256, "near-pair indices are 8-bit");
  constexpr int L = Rec<T, FD>::len;
  constexpr int VEC_PER_REC = L * (int)sizeof(T) / 16;
  for (int base = lo; base < hi; base += TS) {
    const int cnt = min(TS, hi - base);
    __syncthreads();  // previous tile fully consumed
    const int4 *src = reinterpret_cast<const int4 *>(rec + (size_t)base * L);
    int4 *dst = reinterpret_cast<int4 *>(smem);
    const int nvec = cnt * VEC_PER_REC;
    for (int q = threadIdx.x; q < nvec; q += BLOCK) dst[q] = __ldg(src + q);
    __syncthreads();
    if (!compute) continue;
    unsigned nf[TPT];
#pragma unroll
    for (int t = 0; t < TPT; ++t) nf[t] = 0u;
#pragma unroll 2
    for (int j = 0; j < cnt; ++j) {
      T sx, sy, sz, f[FD];
      RecLoad<T, FD>::get(smem + j * L, sx, sy, sz, f);
#pragma unroll
      for (int t = 0; t < TPT; ++t) {
        const T dx = xt[t] - sx, dy = yt[t] - sy, dz = zt[t] - sz;
        const T r2 = fma(dx, dx, fma(dy, dy, dz * dz));
        const bool far = r2 > pc.asum2;
        nf[t] |= far ? 0u : 1u;
        const T rs = rsqrt_far(r2);
        far_pair<T, VD, FD>(v[t], dx, dy, dz, far ? rs : T(0), f, pc);
      }
    }
    unsigned any = 0u;
#pragma unroll
    for (int t = 0; t < TPT; ++t) any |= nf[t];
    if (__any_sync(0xffffffffu, any != 0u)) near_pass<T, VD, FD, TPT>(v, xt, yt, zt, nf, smem, cnt, pc);
    Comp<T, VD, BLOCK, TPT>::fold(v, hl);
  }
}

template <typename T, int VD, int FDA, int FDB, int BLOCK, int TPT, int TS, int MINB>
__global__ void __launch_bounds__(BLOCK, MINB) rpy_tile_kernel(const TileArgs args) {
  constexpr int LA = Rec<T, FDA>::len;
  constexpr int LB = FDB > 0 ? Rec<T, (FDB > 0 ? FDB : 3)>::len : 0;
  constexpr int LMAX = LA > LB ? LA : LB;
  constexpr bool kComp = sizeof(T) == 4;
  extern __shared__ __align__(16) unsigned char tile_smem[];
  T *smem = reinterpret_cast<T *>(tile_smem);
  float *hl = reinterpret_cast<float *>(tile_smem + sizeof(T) * TS * LMAX);

  if (args.skip != nullptr && *args.skip) return;
  const int n_tgt = args.n_tgt;
  const double *origin = args.fp32 ? args.origin : nullptr;
  const int tile0 = blockIdx.x * BLOCK * TPT;

  T xt[TPT], yt[TPT], zt[TPT];
  T v[TPT][VD];
#pragma unroll
  for (int t = 0; t < TPT; ++t) {
    int i = tile0 + t * BLOCK + threadIdx.x;
    i = i < n_tgt ? i : n_tgt - 1;  // duplicate the last target; not written
    xt[t] = load_target<T>(args.x_tgt, i, 0, origin);
    yt[t] = load_target<T>(args.x_tgt, i, 1, origin);
    zt[t] = load_target<T>(args.x_tgt, i, 2, origin);
#pragma unroll
    for (int k = 0; k < VD; ++k) v[t][k] = T(0);
  }
  if (kComp) {
    for (int q = threadIdx.x; q < 2 * TPT * VD * BLOCK; q += BLOCK) hl[q] = 0.f;
  }

  const int n_src = args.n_a + args.n_b;
  const int s0 = blockIdx.y * args.chunk;
  const int s1 = min(s0 + args.chunk, n_src);

  {
    PairConst<T> pc;
    pc.ai = T(args.a_tgt);
    pc.aj = T(args.a_a);
    pc.asum2 = T((args.a_tgt + args.a_a) * (args.a_tgt + args.a_a));
    pc.s = T((args.a_tgt * args.a_tgt + args.a_a * args.a_a) / 3.0);
    pc.s3 = T(-(args.a_tgt * args.a_tgt + args.a_a * args.a_a));
    const int lo = min(s0, args.n_a), hi = min(s1, args.n_a);
    if (lo < hi)
      sum_source_range<T, VD, FDA, BLOCK, TPT, TS>(
          v, xt, yt, zt, reinterpret_cast<const T *>(args.src_a), lo, hi, pc, smem, hl);
  }
  if constexpr (FDB > 0) {
    PairConst<T> pc;
    pc.ai = T(args.a_tgt);
    pc.aj = T(args.a_b);
    pc.asum2 = T((args.a_tgt + args.a_b) * (args.a_tgt + args.a_b));
    pc.s = T((args.a_tgt * args.a_tgt + args.a_b * args.a_b) / 3.0);
    pc.s3 = T(-(args.a_tgt * args.a_tgt + args.a_b * args.a_b));
    const int lo = max(s0 - args.n_a, 0), hi = max(s1 - args.n_a, 0);
    if (lo < hi)
      sum_source_range<T, VD, (FDB > 0 ? FDB : 3), BLOCK, TPT, TS>(
          v, xt, yt, zt, reinterpret_cast<const T *>(args.src_b), lo, hi, pc, smem, hl);
  }

  const double c = args.scale;
#pragma unroll
  for (int t = 0; t < TPT; ++t) {
    const int i = tile0 + t * BLOCK + threadIdx.x;
    if (i >= n_tgt) continue;
    double r[VD];
#pragma unroll
    for (int k = 0; k < VD; ++k) r[k] = c * Comp<T, VD, BLOCK, TPT>::get(v, hl, t, k);
    if (args.mode == OUT_PARTIAL) {
      double *o = args.out + ((size_t)blockIdx.y * n_tgt + i) * VD;
#pragma unroll
      for (int k = 0; k < VD; ++k) o[k] = r[k];
    } else if (args.mode == OUT_ACCUMULATE) {
      double *o = args.out + (size_t)i * VD;
#pragma unroll
      for (int k = 0; k < VD; ++k) o[k] += r[k];
    } else {
      double *o = args.out + (size_t)i * VD;
#pragma unroll
      for (int k = 0; k < VD; ++k) o[k] = r[k];
    }
  }
}

// Dynamic shared memory of one instantiation: the source tile plus, for
// FP32, the compensated running sums.
template <typename T, int VD, int FDA, int FDB, int BLOCK, int TPT, int TS>
constexpr size_t tile_smem_bytes() {
  constexpr int LA = Rec<T, FDA>::len;
  constexpr int LB = FDB > 0 ? Rec<T, (FDB > 0 ? FDB : 3)>::len : 0;
  constexpr int LMAX = LA > LB ? LA : LB;
  return sizeof(T) * TS * LMAX + (sizeof(T) == 4 ? sizeof(float) * 2 * TPT * VD * BLOCK : 0);
}

// Launch one instantiation. With grid.x == 0 it only reports (in *resident)
// how many CTAs of it fit on one SM.
template <typename T, int VD, int FDA, int FDB, int BLOCK, int TPT, int TS, int MINB>
cudaError_t tile_launch_fn(const TileArgs &a, dim3 grid, cudaStream_t st, int *resident) {
  constexpr size_t smem = tile_smem_bytes<T, VD, FDA, FDB, BLOCK, TPT, TS>();
  // set once per device (the shared-memory attribute is per device too);
  // host threads may race to set it
  static std::atomic<int> occupancy[kMaxDevices];
  auto kern = rpy_tile_kernel<T, VD, FDA, FDB, BLOCK, TPT, TS, MINB>;
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
  if (grid.x == 0) return cudaSuccess;  // query only
  kern<<<grid, BLOCK, smem, st>>>(a);
  return cudaGetLastError();
}

// One row of the dispatch table: the six (target, source-set) combinations
// in the order of TileCombo.
#define TFS_TILE_ROW(T, B, P, S, M)                                                        \
  {                                                                                        \
    tile_launch_fn<T, 6, 6, 0, B, P, S, M>, tile_launch_fn<T, 6, 3, 0, B, P, S, M>,        \
        tile_launch_fn<T, 3, 3, 0, B, P, S, M>, tile_launch_fn<T, 3, 6, 0, B, P, S, M>,    \
        tile_launch_fn<T, 6, 6, 3, B, P, S, M>, tile_launch_fn<T, 3, 6, 3, B, P, S, M>     \
  }

}  // namespace tfs
