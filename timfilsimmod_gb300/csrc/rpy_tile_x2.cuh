// rpy_tile_x2.cuh -- FP32 tile kernel on Blackwell's packed FP32x2 pipe
// (FFMA2/FADD2/FMUL2 via __ffma2_rn/__fadd2_rn/__fmul2_rn).
//
// Each float2 holds the same quantity for two targets of one thread, so one
// packed instruction advances two pairs and the issue slots per pair halve.
// Source records are stored with every value duplicated and the position
// negated ({-x,-x,-y,-y,-z,-z,f0,f0,...}), so a 16-byte shared load yields
// two ready-made float2 operands and the separation is one packed add:
//   FP32x2 segment record: 9 pairs + 1 pad pair = 80 B
//   FP32x2 blob record:    6 pairs             = 48 B
// Accumulation, near-pair replay and compensation follow rpy_tile.cuh.
#pragma once

#include <atomic>

#include <cuda_runtime.h>

#include "rpy_tile.cuh"

namespace tfs {

template <int FD>
struct RecX2 {
  static constexpr int len = FD == 6 ? 20 : 12;  // floats
};

__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

template <int FD>
__device__ __forceinline__ void load_rec_x2(const float *r, float2 &mx, float2 &my, float2 &mz,
                                            float2 (&f)[FD]) {
  const float4 *q = reinterpret_cast<const float4 *>(r);
  const float4 a = q[0], b = q[1], c = q[2];
  mx = make_float2(a.x, a.y);
  my = make_float2(a.z, a.w);
  mz = make_float2(b.x, b.y);
  f[0] = make_float2(b.z, b.w);
  f[1] = make_float2(c.x, c.y);
  f[2] = make_float2(c.z, c.w);
  if constexpr (FD == 6) {
    const float4 d = q[3], e = q[4];
    f[3] = make_float2(d.x, d.y);
    f[4] = make_float2(d.z, d.w);
    f[5] = make_float2(e.x, e.y);
  }
}

// Far-field pair for two targets at once; the packed twin of far_pair
// (tfs_device.cuh), same formulas and units.
template <int VD, int FD>
__device__ __forceinline__ void far_pair_x2(float2 *__restrict__ v, float2 dx, float2 dy,
                                            float2 dz, float2 rm1, const float2 *__restrict__ f,
                                            float2 s, float2 s3) {
  const float2 rm2 = mul2(rm1, rm1);
  const float2 rm3 = mul2(rm1, rm2);
  const float2 rm5 = mul2(rm3, rm2);
  const float2 A = fma2(s, rm3, rm1);
  const float2 B = fma2(s3, rm5, rm3);
  const float2 dF = fma2(dx, f[0], fma2(dy, f[1], mul2(dz, f[2])));
  const float2 Bd = mul2(B, dF);
  v[0] = fma2(A, f[0], fma2(Bd, dx, v[0]));
  v[1] = fma2(A, f[1], fma2(Bd, dy, v[1]));
  v[2] = fma2(A, f[2], fma2(Bd, dz, v[2]));
  if (FD == 6 || VD == 6) {
    // e = rm3 d and its negation: the packed FMA has no operand negation, so
    // the cross products use -e instead of negated source components.
    const float2 nrm3 = mul2(make_float2(-1.f, -1.f), rm3);
    const float2 ex = mul2(rm3, dx), ey = mul2(rm3, dy), ez = mul2(rm3, dz);
    const float2 nx = mul2(nrm3, dx), ny = mul2(nrm3, dy), nz = mul2(nrm3, dz);
    if (FD == 6) {
      v[0] = fma2(f[4], ez, fma2(f[5], ny, v[0]));
      v[1] = fma2(f[5], ex, fma2(f[3], nz, v[1]));
      v[2] = fma2(f[3], ey, fma2(f[4], nx, v[2]));
    }
    if (VD == 6) {
      v[3] = fma2(f[1], ez, fma2(f[2], ny, v[3]));
      v[4] = fma2(f[2], ex, fma2(f[0], nz, v[4]));
      v[5] = fma2(f[0], ey, fma2(f[1], nx, v[5]));
      if (FD == 6) {
        const float2 h = mul2(make_float2(-0.5f, -0.5f), rm3);
        const float2 dT = fma2(dx, f[3], fma2(dy, f[4], mul2(dz, f[5])));
        const float2 q = mul2(mul2(make_float2(1.5f, 1.5f), rm5), dT);
        v[3] = fma2(h, f[3], fma2(q, dx, v[3]));
        v[4] = fma2(h, f[4], fma2(q, dy, v[4]));
        v[5] = fma2(h, f[5], fma2(q, dz, v[5]));
      }
    }
  }
}

template <int VD, int FD, int BLOCK, int TP2, int TS>
__device__ __forceinline__ void sum_source_range_x2(float2 (&v)[TP2][VD], const float2 (&xt)[TP2],
                                                    const float2 (&yt)[TP2],
                                                    const float2 (&zt)[TP2],
                                                    const float *__restrict__ rec, int lo, int hi,
                                                    const PairConst<float> &pc, float *smem,
                                                    float *hl) {
  constexpr int L = RecX2<FD>::len;
  constexpr int VEC_PER_REC = L * 4 / 16;
  const float2 s2 = make_float2(pc.s, pc.s), s32 = make_float2(pc.s3, pc.s3);
  for (int base = lo; base < hi; base += TS) {
    const int cnt = min(TS, hi - base);
    __syncthreads();
    const int4 *src = reinterpret_cast<const int4 *>(rec + (size_t)base * L);
    int4 *dst = reinterpret_cast<int4 *>(smem);
    const int nvec = cnt * VEC_PER_REC;
    for (int q = threadIdx.x; q < nvec; q += BLOCK) dst[q] = __ldg(src + q);
    __syncthreads();
    bool near = false;
#pragma unroll 1
    for (int j = 0; j < cnt; ++j) {
      float2 mx, my, mz, f[FD];
      load_rec_x2<FD>(smem + j * L, mx, my, mz, f);
#pragma unroll
      for (int p = 0; p < TP2; ++p) {
        const float2 dx = add2(xt[p], mx), dy = add2(yt[p], my), dz = add2(zt[p], mz);
        const float2 r2 = fma2(dx, dx, fma2(dy, dy, mul2(dz, dz)));
        const bool f0 = r2.x > pc.asum2, f1 = r2.y > pc.asum2;
        near |= !(f0 && f1);
        const float2 rm1 = make_float2(f0 ? rsqrtf(r2.x) : 0.f, f1 ? rsqrtf(r2.y) : 0.f);
        far_pair_x2<VD, FD>(v[p], dx, dy, dz, rm1, f, s2, s32);
      }
    }
    if (__any_sync(0xffffffffu, near)) {
      if (near) {
        for (int j = 0; j < cnt; ++j) {
          float2 mx, my, mz, f2[FD];
          load_rec_x2<FD>(smem + j * L, mx, my, mz, f2);
          float f[FD];
#pragma unroll
          for (int k = 0; k < FD; ++k) f[k] = f2[k].x;
#pragma unroll
          for (int p = 0; p < TP2; ++p) {
#pragma unroll
            for (int h = 0; h < 2; ++h) {
              const float dx = (h ? xt[p].y : xt[p].x) + mx.x;
              const float dy = (h ? yt[p].y : yt[p].x) + my.x;
              const float dz = (h ? zt[p].y : zt[p].x) + mz.x;
              const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
              if (!(r2 > pc.asum2)) {
                float tmp[VD];
#pragma unroll
                for (int k = 0; k < VD; ++k) tmp[k] = 0.f;
                near_pair<float, VD, FD>(tmp, dx, dy, dz, r2, f, pc);
#pragma unroll
                for (int k = 0; k < VD; ++k) {
                  if (h) v[p][k].y += tmp[k];
                  else v[p][k].x += tmp[k];
                }
              }
            }
          }
        }
      }
    }
    // fold the tile sums into the compensated running sums
#pragma unroll
    for (int p = 0; p < TP2; ++p)
#pragma unroll
      for (int k = 0; k < VD; ++k) {
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          float *hip = hl + (((p * VD + k) * 2 + h) * 2) * BLOCK + threadIdx.x;
          float *lop = hip + BLOCK;
          float hv = *hip, lv = *lop;
          two_sum(hv, lv, h ? v[p][k].y : v[p][k].x);
          *hip = hv;
          *lop = lv;
        }
        v[p][k] = make_float2(0.f, 0.f);
      }
  }
}

// TPT targets per thread (TPT even), packed in TPT/2 float2 pairs: pair p
// holds targets 2p and 2p+1 of the thread (target i = tile0 + t*BLOCK + tid).
template <int VD, int FDA, int FDB, int BLOCK, int TPT, int TS>
__global__ void __launch_bounds__(BLOCK) rpy_tile_x2_kernel(const TileArgs args) {
  static_assert(TPT % 2 == 0, "packed kernel needs an even number of targets per thread");
  constexpr int TP2 = TPT / 2;
  constexpr int LA = RecX2<FDA>::len;
  constexpr int LB = FDB > 0 ? RecX2<(FDB > 0 ? FDB : 3)>::len : 0;
  constexpr int LMAX = LA > LB ? LA : LB;
  extern __shared__ __align__(16) unsigned char tile_smem[];
  float *smem = reinterpret_cast<float *>(tile_smem);
  float *hl = smem + TS * LMAX;

  if (args.skip != nullptr && *args.skip) return;
  const int n_tgt = args.n_tgt;
  const double *origin = args.origin;
  const int tile0 = blockIdx.x * BLOCK * TPT;

  float2 xt[TP2], yt[TP2], zt[TP2];
  float2 v[TP2][VD];
#pragma unroll
  for (int p = 0; p < TP2; ++p) {
    float c[2][3];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      int i = tile0 + (2 * p + h) * BLOCK + threadIdx.x;
      i = i < n_tgt ? i : n_tgt - 1;  // duplicate the last target; not written
#pragma unroll
      for (int k = 0; k < 3; ++k) c[h][k] = load_target<float>(args.x_tgt, i, k, origin);
    }
    xt[p] = make_float2(c[0][0], c[1][0]);
    yt[p] = make_float2(c[0][1], c[1][1]);
    zt[p] = make_float2(c[0][2], c[1][2]);
#pragma unroll
    for (int k = 0; k < VD; ++k) v[p][k] = make_float2(0.f, 0.f);
  }
  for (int q = threadIdx.x; q < 2 * TPT * VD * BLOCK; q += BLOCK) hl[q] = 0.f;

  const int n_src = args.n_a + args.n_b;
  const int s0 = blockIdx.y * args.chunk;
  const int s1 = min(s0 + args.chunk, n_src);
  {
    PairConst<float> pc;
    pc.ai = float(args.a_tgt);
    pc.aj = float(args.a_a);
    pc.asum2 = float((args.a_tgt + args.a_a) * (args.a_tgt + args.a_a));
    pc.s = float((args.a_tgt * args.a_tgt + args.a_a * args.a_a) / 3.0);
    pc.s3 = float(-(args.a_tgt * args.a_tgt + args.a_a * args.a_a));
    const int lo = min(s0, args.n_a), hi = min(s1, args.n_a);
    if (lo < hi)
      sum_source_range_x2<VD, FDA, BLOCK, TP2, TS>(
          v, xt, yt, zt, reinterpret_cast<const float *>(args.src_a2), lo, hi, pc, smem, hl);
  }
  if constexpr (FDB > 0) {
    PairConst<float> pc;
    pc.ai = float(args.a_tgt);
    pc.aj = float(args.a_b);
    pc.asum2 = float((args.a_tgt + args.a_b) * (args.a_tgt + args.a_b));
    pc.s = float((args.a_tgt * args.a_tgt + args.a_b * args.a_b) / 3.0);
    pc.s3 = float(-(args.a_tgt * args.a_tgt + args.a_b * args.a_b));
    const int lo = max(s0 - args.n_a, 0), hi = max(s1 - args.n_a, 0);
    if (lo < hi)
      sum_source_range_x2<VD, (FDB > 0 ? FDB : 3), BLOCK, TP2, TS>(
          v, xt, yt, zt, reinterpret_cast<const float *>(args.src_b2), lo, hi, pc, smem, hl);
  }

  const double c = args.scale;
#pragma unroll
  for (int p = 0; p < TP2; ++p)
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int i = tile0 + (2 * p + h) * BLOCK + threadIdx.x;
      if (i >= n_tgt) continue;
      double r[VD];
#pragma unroll
      for (int k = 0; k < VD; ++k) {
        const float *hip = hl + (((p * VD + k) * 2 + h) * 2) * BLOCK + threadIdx.x;
        r[k] = c * ((double)hip[0] + (double)hip[BLOCK]);
      }
      double *o = args.mode == OUT_PARTIAL ? args.out + ((size_t)blockIdx.y * n_tgt + i) * VD
                                           : args.out + (size_t)i * VD;
      if (args.mode == OUT_ACCUMULATE) {
#pragma unroll
        for (int k = 0; k < VD; ++k) o[k] += r[k];
      } else {
#pragma unroll
        for (int k = 0; k < VD; ++k) o[k] = r[k];
      }
    }
}

template <int VD, int FDA, int FDB, int BLOCK, int TPT, int TS>
constexpr size_t tile_x2_smem_bytes() {
  constexpr int LA = RecX2<FDA>::len;
  constexpr int LB = FDB > 0 ? RecX2<(FDB > 0 ? FDB : 3)>::len : 0;
  constexpr int LMAX = LA > LB ? LA : LB;
  return sizeof(float) * (TS * LMAX + 2 * TPT * VD * BLOCK);
}

template <int VD, int FDA, int FDB, int BLOCK, int TPT, int TS>
cudaError_t tile_x2_launch_fn(const TileArgs &a, dim3 grid, cudaStream_t st, int *resident) {
  constexpr size_t smem = tile_x2_smem_bytes<VD, FDA, FDB, BLOCK, TPT, TS>();
  static std::atomic<int> occupancy[kMaxDevices];  // set once per device; threads may race
  auto kern = rpy_tile_x2_kernel<VD, FDA, FDB, BLOCK, TPT, TS>;
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

#define TFS_TILE_X2_ROW(B, P, S)                                                         \
  {                                                                                      \
    tile_x2_launch_fn<6, 6, 0, B, P, S>, tile_x2_launch_fn<6, 3, 0, B, P, S>,            \
        tile_x2_launch_fn<3, 3, 0, B, P, S>, tile_x2_launch_fn<3, 6, 0, B, P, S>,        \
        tile_x2_launch_fn<6, 6, 3, B, P, S>, tile_x2_launch_fn<3, 6, 3, B, P, S>         \
  }

}  // namespace tfs
