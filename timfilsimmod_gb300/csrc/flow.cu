// flow.cu -- the flow-field evaluator: fluid velocity at arbitrary points due
// to the segment forces/torques and blob forces of saved swimmer states
// (the reference's flow_velocities kernel, src/flow_field/flow_field_evaluator.cu
// :13-228, and flow_field_evaluator::velocities :546-579).
//
//   u(x) = prefac [ sum_segs ( F/r + (r.F) r / r^3 + (T x r) / r^3 )
//                 + sum_blobs ( F/r + (r.F) r / r^3 ) ],      r = x - x_j,
// point Stokeslets and rotlets without the RPY finite-size terms. With no
// blobs the segment Stokeslet becomes the Blakelet of a no-slip wall at z = 0
// (image Stokeslet plus the source-doublet/stresslet correction, :83-116);
// optionally the Stokeslet of every source force placed at its body's centre
// is subtracted (remove_net_force, :125-143, :189-203).
//
// Same tile machinery as the mobility product (rpy_tile.cuh): sources packed
// into 16-byte records and staged through shared memory, targets register
// blocked, FP32 sums compensated per tile, deterministic source splits.
#include <cuda_runtime.h>

#include <algorithm>
#include <new>

#include "../../include/tfs_gb300.h"
#include "rpy_tile.cuh"
#include "tfs_kernels.h"

namespace tfs {
int fail(int code, const char *fmt, ...);
int cuda_fail(cudaError_t e, const char *what);
int alloc_dev(void **p, size_t bytes);

struct FlowArgs {
  const double *x_flow;
  int n_flow;
  const void *rec_segs;   // segment records (Rec<T,6>)
  int n_segs, segs_per_body;
  const void *rec_blobs;  // blob records (Rec<T,3>)
  int n_blobs, blobs_per_body;
  const double *x_bodies;  // body centres (remove_net_force)
  int n_bodies;
  const double *origin;    // FP32 centring origin (z = 0 when the wall is on)
  double prefac;
  double *out;             // 3 * n_flow, or partials
  int mode;                // OUT_ASSIGN or OUT_PARTIAL
  int chunk;               // sources per split
};

// Stokeslet of force f at separation d: v += rm1 f + rm3 (d.f) d
template <typename T>
__device__ __forceinline__ void stokeslet(T *v, T dx, T dy, T dz, T rm1, const T *f, T sgn) {
  const T rm3 = rm1 * rm1 * rm1;
  const T w = rm3 * fma(dx, f[0], fma(dy, f[1], dz * f[2]));
  const T a = sgn * rm1, b = sgn * w;
  v[0] = fma(a, f[0], fma(b, dx, v[0]));
  v[1] = fma(a, f[1], fma(b, dy, v[1]));
  v[2] = fma(a, f[2], fma(b, dz, v[2]));
}

template <typename T>
__device__ __forceinline__ T rsq(T r2) {
  return rsqrt_far(r2);
}

// One segment source: Stokeslet (or Blakelet, WALL) + rotlet (+ net-force removal).
template <typename T, bool WALL, bool RNF>
__device__ __forceinline__ void flow_seg_pair(T *v, T xi, T yi, T zi, T sx, T sy, T sz,
                                              const T *f, T bx, T by, T bz) {
  const T dx = xi - sx, dy = yi - sy, dz = zi - sz;
  const T r2 = fma(dx, dx, fma(dy, dy, dz * dz));
  const T rm1 = rsq(r2);
  stokeslet(v, dx, dy, dz, rm1, f, T(1));
  if (WALL) {
    // minus the image Stokeslet at (sx, sy, -sz), then the higher-order
    // correction (flow_field_evaluator.cu:83-116)
    const T Rz = zi + sz;
    const T R2 = fma(dx, dx, fma(dy, dy, Rz * Rz));
    const T Rm1 = rsq(R2);
    stokeslet(v, dx, dy, Rz, Rm1, f, T(-1));
    const T Dxx = (T(3) * dx * dx - R2) * zi;
    const T Dxy = T(3) * dx * dy * zi;
    const T Dxz = (R2 - T(3) * Rz * zi) * dx;
    const T Dyy = (T(3) * dy * dy - R2) * zi;
    const T Dyz = (R2 - T(3) * Rz * zi) * dy;
    const T Dzx = (T(3) * Rz * zi + R2) * dx;
    const T Dzy = (T(3) * Rz * zi + R2) * dy;
    const T Dzz = (R2 - T(3) * Rz * Rz) * zi;
    const T Rm2 = Rm1 * Rm1;
    const T Dfac = T(2) * sz * Rm2 * Rm2 * Rm1;
    v[0] += Dfac * (Dxx * f[0] + Dxy * f[1] + Dxz * f[2]);
    v[1] += Dfac * (Dxy * f[0] + Dyy * f[1] + Dyz * f[2]);
    v[2] += Dfac * (Dzx * f[0] + Dzy * f[1] + Dzz * f[2]);
  }
  // rotlet (:118-123)
  const T rm3 = rm1 * rm1 * rm1;
  v[0] = fma(rm3, f[4] * dz - f[5] * dy, v[0]);
  v[1] = fma(rm3, f[5] * dx - f[3] * dz, v[1]);
  v[2] = fma(rm3, f[3] * dy - f[4] * dx, v[2]);
  if (RNF) {
    const T ex = xi - bx, ey = yi - by, ez = zi - bz;
    stokeslet(v, ex, ey, ez, rsq(fma(ex, ex, fma(ey, ey, ez * ez))), f, T(-1));
  }
}

template <typename T, bool RNF>
__device__ __forceinline__ void flow_blob_pair(T *v, T xi, T yi, T zi, T sx, T sy, T sz,
                                               const T *f, T bx, T by, T bz) {
  const T dx = xi - sx, dy = yi - sy, dz = zi - sz;
  stokeslet(v, dx, dy, dz, rsq(fma(dx, dx, fma(dy, dy, dz * dz))), f, T(1));
  if (RNF) {
    const T ex = xi - bx, ey = yi - by, ez = zi - bz;
    stokeslet(v, ex, ey, ez, rsq(fma(ex, ex, fma(ey, ey, ez * ez))), f, T(-1));
  }
}

template <typename T, int FD, bool WALL, bool RNF, int BLOCK, int TPT, int TS>
__device__ __forceinline__ void flow_range(T (&v)[TPT][3], const T (&xt)[TPT], const T (&yt)[TPT],
                                           const T (&zt)[TPT], const T *__restrict__ rec, int lo,
                                           int hi, int per_body, const double *x_bodies,
                                           const double *origin, T *smem, float *hl) {
  constexpr int L = Rec<T, FD>::len;
  constexpr int VEC_PER_REC = L * (int)sizeof(T) / 16;
  for (int base = lo; base < hi; base += TS) {
    const int cnt = min(TS, hi - base);
    __syncthreads();
    const int4 *src = reinterpret_cast<const int4 *>(rec + (size_t)base * L);
    int4 *dst = reinterpret_cast<int4 *>(smem);
    for (int q = threadIdx.x; q < cnt * VEC_PER_REC; q += BLOCK) dst[q] = __ldg(src + q);
    __syncthreads();
    int body = -1;
    T bx = 0, by = 0, bz = 0;
#pragma unroll 2
    for (int j = 0; j < cnt; ++j) {
      T sx, sy, sz, f[FD];
      RecLoad<T, FD>::get(smem + j * L, sx, sy, sz, f);
      if (RNF) {
        const int b = (base + j) / per_body;  // warp-uniform
        if (b != body) {
          body = b;
          const double *xb = x_bodies + 3 * (size_t)b;
          bx = T(xb[0] - (origin ? origin[0] : 0.0));
          by = T(xb[1] - (origin ? origin[1] : 0.0));
          bz = T(xb[2] - (origin ? origin[2] : 0.0));
        }
      }
#pragma unroll
      for (int t = 0; t < TPT; ++t) {
        if (FD == 6)
          flow_seg_pair<T, WALL, RNF>(v[t], xt[t], yt[t], zt[t], sx, sy, sz, f, bx, by, bz);
        else
          flow_blob_pair<T, RNF>(v[t], xt[t], yt[t], zt[t], sx, sy, sz, f, bx, by, bz);
      }
    }
    Comp<T, 3, BLOCK, TPT>::fold(v, hl);
  }
}

template <typename T, bool WALL, bool RNF, int BLOCK, int TPT, int TS>
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
  const int n_src = a.n_segs + a.n_blobs;
  const int s0 = blockIdx.y * a.chunk, s1 = min(s0 + a.chunk, n_src);
  {
    const int lo = min(s0, a.n_segs), hi = min(s1, a.n_segs);
    if (lo < hi)
      flow_range<T, 6, WALL, RNF, BLOCK, TPT, TS>(v, xt, yt, zt,
                                                  reinterpret_cast<const T *>(a.rec_segs), lo,
                                                  hi, a.segs_per_body, a.x_bodies, origin, smem,
                                                  hl);
  }
  {
    const int lo = max(s0 - a.n_segs, 0), hi = max(s1 - a.n_segs, 0);
    if (lo < hi)
      flow_range<T, 3, false, RNF, BLOCK, TPT, TS>(v, xt, yt, zt,
                                                   reinterpret_cast<const T *>(a.rec_blobs), lo,
                                                   hi, a.blobs_per_body, a.x_bodies, origin,
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

template <typename T, bool WALL, bool RNF>
static cudaError_t flow_launch_t(FlowArgs a, double *scratch, size_t scratch_elems,
                                 cudaStream_t st) {
  constexpr int BLOCK = 128, TPT = sizeof(T) == 4 ? 2 : 1, TS = sizeof(T) == 4 ? 256 : 128;
  const int per_cta = BLOCK * TPT;
  const int ctas = (a.n_flow + per_cta - 1) / per_cta;
  const int n_src = a.n_segs + a.n_blobs;
  int splits = std::max(1, (8 * num_sms() + ctas - 1) / ctas);
  splits = std::min({splits, kMaxSplits, std::max(1, n_src / 128)});
  if ((size_t)splits * 3 * a.n_flow > scratch_elems) splits = 1;
  int chunk = (n_src + splits - 1) / splits;
  chunk = std::max(64, ((chunk + 63) / 64) * 64);
  splits = std::max(1, (n_src + chunk - 1) / chunk);
  a.chunk = chunk;
  double *final_out = a.out;
  if (splits > 1) {
    a.mode = OUT_PARTIAL;
    a.out = scratch;
  } else {
    a.mode = OUT_ASSIGN;
  }
  flow_kernel<T, WALL, RNF, BLOCK, TPT, TS><<<dim3(ctas, splits), BLOCK, 0, st>>>(a);
  count_launch();
  if (splits > 1) return launch_reduce_partials(final_out, scratch, 3 * a.n_flow, splits, 0, st);
  return cudaGetLastError();
}

cudaError_t launch_flow(const FlowArgs &a, int fp32, int wall, int rnf, double *scratch,
                        size_t scratch_elems, cudaStream_t st) {
  if (a.n_flow <= 0) return cudaSuccess;
  if (fp32) {
    if (wall) return rnf ? flow_launch_t<float, true, true>(a, scratch, scratch_elems, st)
                         : flow_launch_t<float, true, false>(a, scratch, scratch_elems, st);
    return rnf ? flow_launch_t<float, false, true>(a, scratch, scratch_elems, st)
               : flow_launch_t<float, false, false>(a, scratch, scratch_elems, st);
  }
  if (wall) return rnf ? flow_launch_t<double, true, true>(a, scratch, scratch_elems, st)
                       : flow_launch_t<double, true, false>(a, scratch, scratch_elems, st);
  return rnf ? flow_launch_t<double, false, true>(a, scratch, scratch_elems, st)
             : flow_launch_t<double, false, false>(a, scratch, scratch_elems, st);
}

}  // namespace tfs

using namespace tfs;

// ---------------------------------------------------------------------------
// C ABI: the flow evaluator object (flow_field_evaluator, flow_field_evaluator.hpp:8-61)
// ---------------------------------------------------------------------------
struct tfs_flow {
  int nflow = 0, nbod = 0, segs_per_body = 0, blobs_per_body = 0, precision = 0;
  int ns = 0, nb = 0;
  cudaStream_t own_stream = nullptr, stream = nullptr;
  double *x_flow = nullptr, *v_flow = nullptr, *x_segs = nullptr, *f_segs = nullptr,
         *x_blobs = nullptr, *f_blobs = nullptr, *x_bodies = nullptr, *origin = nullptr;
  void *rec_segs = nullptr, *rec_blobs = nullptr;
  double *scratch = nullptr;
  size_t scratch_elems = 0;
  double origin_host[4] = {0, 0, 0, 0};
};

static void flow_free(tfs_flow *f) {
  cudaFree(f->x_flow);
  cudaFree(f->v_flow);
  cudaFree(f->x_segs);
  cudaFree(f->f_segs);
  cudaFree(f->x_blobs);
  cudaFree(f->f_blobs);
  cudaFree(f->x_bodies);
  cudaFree(f->origin);
  cudaFree(f->rec_segs);
  cudaFree(f->rec_blobs);
  cudaFree(f->scratch);
  if (f->own_stream) cudaStreamDestroy(f->own_stream);
}

extern "C" {

int tfs_flow_create(int num_flow, int num_bodies, int segs_per_body, int blobs_per_body,
                    int precision, tfs_flow **out) {
  if (out == nullptr) return fail(TFS_EINVAL, "null output");
  *out = nullptr;
  if (num_flow < 0 || num_bodies < 1 || segs_per_body < 0 || blobs_per_body < 0)
    return fail(TFS_EINVAL, "bad sizes");
  if (precision != TFS_FP64 && precision != TFS_FP32C)
    return fail(TFS_EINVAL, "unknown precision %d", precision);
  const long long ns = (long long)num_bodies * segs_per_body;
  const long long nb = (long long)num_bodies * blobs_per_body;
  if (ns > (1LL << 26) || nb > (1LL << 26) || num_flow > (1 << 28))
    return fail(TFS_EINVAL, "sizes too large");
  tfs_flow *f = new (std::nothrow) tfs_flow;
  if (f == nullptr) return fail(TFS_ENOMEM, "host allocation failed");
  f->nflow = num_flow;
  f->nbod = num_bodies;
  f->segs_per_body = segs_per_body;
  f->blobs_per_body = blobs_per_body;
  f->precision = precision;
  f->ns = (int)ns;
  f->nb = (int)nb;
  cudaError_t e = cudaStreamCreateWithFlags(&f->own_stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete f;
    return cuda_fail(e, "cudaStreamCreate");
  }
  f->stream = f->own_stream;
  // split partials (source splits are only used while the points fill few
  // waves; the launcher drops to one split when they do not fit)
  f->scratch_elems = std::max((size_t)1, std::min((size_t)kMaxSplits * 3 * num_flow,
                                                  (size_t)3 << 20));
  int rc;
  if ((rc = alloc_dev((void **)&f->x_flow, 24 * (size_t)num_flow)) ||
      (rc = alloc_dev((void **)&f->v_flow, 24 * (size_t)num_flow)) ||
      (rc = alloc_dev((void **)&f->x_segs, 24 * (size_t)ns)) ||
      (rc = alloc_dev((void **)&f->f_segs, 48 * (size_t)ns)) ||
      (rc = alloc_dev((void **)&f->x_blobs, 24 * (size_t)nb)) ||
      (rc = alloc_dev((void **)&f->f_blobs, 24 * (size_t)nb)) ||
      (rc = alloc_dev((void **)&f->x_bodies, 24 * (size_t)num_bodies)) ||
      (rc = alloc_dev((void **)&f->origin, 32)) ||
      (rc = alloc_dev(&f->rec_segs, record_bytes(0, 6) * (size_t)ns)) ||
      (rc = alloc_dev(&f->rec_blobs, record_bytes(0, 3) * (size_t)nb)) ||
      (rc = alloc_dev((void **)&f->scratch, 8 * f->scratch_elems))) {
    flow_free(f);
    delete f;
    return rc;
  }
  *out = f;
  return TFS_OK;
}

int tfs_flow_destroy(tfs_flow *f) {
  if (f == nullptr) return TFS_OK;
  cudaStreamSynchronize(f->stream);
  flow_free(f);
  delete f;
  return TFS_OK;
}

int tfs_flow_set_stream(tfs_flow *f, void *stream) {
  if (f == nullptr) return fail(TFS_EINVAL, "null flow handle");
  f->stream = stream ? (cudaStream_t)stream : f->own_stream;
  return TFS_OK;
}

// read_positions_and_forces (flow_field_evaluator.cu:401-544) from host
// arrays: evaluation points x_flow[3 nflow], segment positions/forces
// (x_segs[3 ns], f_segs[6 ns]), blob positions/forces (x_blobs[3 nb],
// f_blobs[3 nb]; NULL when there are no blobs) and body centres x_bodies[3 nbod].
int tfs_flow_copy_inputs_to_device(tfs_flow *f, const double *x_flow, const double *x_segs,
                                   const double *f_segs, const double *x_blobs,
                                   const double *f_blobs, const double *x_bodies) {
  if (f == nullptr) return fail(TFS_EINVAL, "null flow handle");
  struct {
    double *dst;
    const double *src;
    size_t n;
  } c[] = {{f->x_flow, x_flow, 3 * (size_t)f->nflow}, {f->x_segs, x_segs, 3 * (size_t)f->ns},
           {f->f_segs, f_segs, 6 * (size_t)f->ns},    {f->x_blobs, x_blobs, 3 * (size_t)f->nb},
           {f->f_blobs, f_blobs, 3 * (size_t)f->nb},  {f->x_bodies, x_bodies, 3 * (size_t)f->nbod}};
  for (auto &k : c) {
    if (k.n == 0) continue;
    if (k.src == nullptr) return fail(TFS_EINVAL, "null host array");
    cudaError_t e = cudaMemcpyAsync(k.dst, k.src, 8 * k.n, cudaMemcpyHostToDevice, f->stream);
    if (e != cudaSuccess) return cuda_fail(e, "flow inputs");
  }
  // FP32 centring origin: the mean body centre; z stays 0 for the wall form,
  // whose image terms need absolute heights above z = 0
  double o[4] = {0, 0, 0, 0};
  for (int b = 0; b < f->nbod; ++b)
    for (int k = 0; k < 3; ++k) o[k] += x_bodies[3 * (size_t)b + k] / f->nbod;
  if (f->blobs_per_body == 0) o[2] = 0.0;
  for (int k = 0; k < 4; ++k) f->origin_host[k] = o[k];
  cudaError_t e = cudaMemcpyAsync(f->origin, f->origin_host, 32, cudaMemcpyHostToDevice,
                                  f->stream);
  if (e != cudaSuccess) return cuda_fail(e, "flow origin");
  e = cudaStreamSynchronize(f->stream);  // the origin staging buffer is reused
  if (e != cudaSuccess) return cuda_fail(e, "flow inputs");
  return TFS_OK;
}

// velocities() (flow_field_evaluator.cu:546-579): v_flow = prefac * (...)
// with prefac = 1 / (8 pi mu); remove_net_force as the reference's
// REMOVE_NET_FORCE_STOKESLET. The wall (Blakelet) form is used when the
// bodies have no blobs, as in the reference.
int tfs_flow_velocities(tfs_flow *f, double mu, int remove_net_force) {
  if (f == nullptr) return fail(TFS_EINVAL, "null flow handle");
  if (!(mu > 0.0)) return fail(TFS_EINVAL, "mu must be positive");
  const int fp32 = f->precision == TFS_FP32C;
  cudaError_t e;
  const double *origin = fp32 ? f->origin : nullptr;  // FP64 records stay absolute
  if (f->ns > 0 && (e = launch_pack(fp32, 6, f->rec_segs, f->x_segs, f->f_segs, f->ns, origin,
                                    f->stream)) != cudaSuccess)
    return cuda_fail(e, "pack kernel");
  if (f->nb > 0 && (e = launch_pack(fp32, 3, f->rec_blobs, f->x_blobs, f->f_blobs, f->nb, origin,
                                    f->stream)) != cudaSuccess)
    return cuda_fail(e, "pack kernel");
  FlowArgs a{};
  a.x_flow = f->x_flow;
  a.n_flow = f->nflow;
  a.rec_segs = f->rec_segs;
  a.n_segs = f->ns;
  a.segs_per_body = std::max(1, f->segs_per_body);
  a.rec_blobs = f->rec_blobs;
  a.n_blobs = f->nb;
  a.blobs_per_body = std::max(1, f->blobs_per_body);
  a.x_bodies = f->x_bodies;
  a.n_bodies = f->nbod;
  a.origin = f->origin;
  a.prefac = 1.0 / (8.0 * 3.14159265358979323846264338327950288 * mu);
  a.out = f->v_flow;
  e = launch_flow(a, fp32, f->blobs_per_body == 0, remove_net_force != 0, f->scratch,
                  f->scratch_elems, f->stream);
  if (e != cudaSuccess) return cuda_fail(e, "flow kernel");
  return TFS_OK;
}

int tfs_flow_copy_velocities_to_host(tfs_flow *f, double *v_flow) {
  if (f == nullptr) return fail(TFS_EINVAL, "null flow handle");
  if (f->nflow == 0) return TFS_OK;
  if (v_flow == nullptr) return fail(TFS_EINVAL, "null host pointer");
  cudaError_t e = cudaMemcpyAsync(v_flow, f->v_flow, 24 * (size_t)f->nflow,
                                  cudaMemcpyDeviceToHost, f->stream);
  if (e != cudaSuccess) return cuda_fail(e, "copy flow velocities");
  e = cudaStreamSynchronize(f->stream);
  if (e != cudaSuccess) return cuda_fail(e, "copy flow velocities");
  return TFS_OK;
}

int tfs_flow_device_buffers(tfs_flow *f, double **x_flow, double **v_flow) {
  if (f == nullptr) return fail(TFS_EINVAL, "null flow handle");
  if (x_flow) *x_flow = f->x_flow;
  if (v_flow) *v_flow = f->v_flow;
  return TFS_OK;
}

int tfs_flow_wait(tfs_flow *f) {
  if (f == nullptr) return fail(TFS_EINVAL, "null flow handle");
  cudaError_t e = cudaStreamSynchronize(f->stream);
  if (e != cudaSuccess) return cuda_fail(e, "flow wait");
  return TFS_OK;
}

}  // extern "C"
