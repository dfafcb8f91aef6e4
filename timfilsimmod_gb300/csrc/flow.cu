// flow.cu -- the flow-field evaluator: fluid velocity at arbitrary points due
// to the segment forces/torques and blob forces of saved swimmer states
// (the reference's flow_field_evaluator, src/flow_field/flow_field_evaluator.cu;
// kernel flow_velocities :13-228, velocities() :546-579). The tile kernel is
// in flow_kernels.cuh; this file holds its launcher, the body-centre points
// of the net-force Stokeslet, the launch-variant autotuner and the C ABI.
#include <cuda_runtime.h>

#include <algorithm>
#include <new>

#include "../../include/tfs_gb300.h"
#include "flow_kernels.cuh"
#include "tfs_kernels.h"

namespace tfs {
int fail(int code, const char *fmt, ...);
int cuda_fail(cudaError_t e, const char *what);
int alloc_dev(void **p, size_t bytes);

// One record per body b, appended after the blob records: the body centre
// (minus the FP32 origin) carrying minus the sum of the forces of the body's
// segments and blobs. One CTA per body; each thread sums a fixed strided
// subset, then a fixed-shape tree: the result does not depend on timing.
template <typename T>
__global__ void __launch_bounds__(256) body_points_kernel(
    T *__restrict__ rec, const double *__restrict__ f_segs, int segs_per_body,
    const double *__restrict__ f_blobs, int blobs_per_body, const double *__restrict__ x_bodies,
    const double *__restrict__ origin) {
  constexpr int L = Rec<T, 3>::len;
  __shared__ double red[3][256];
  const int b = blockIdx.x;
  double s0 = 0.0, s1 = 0.0, s2 = 0.0;
  const double *fs = f_segs + 6 * (size_t)b * segs_per_body;
  for (int j = threadIdx.x; j < segs_per_body; j += 256) {
    s0 += fs[6 * (size_t)j];
    s1 += fs[6 * (size_t)j + 1];
    s2 += fs[6 * (size_t)j + 2];
  }
  const double *fb = f_blobs + 3 * (size_t)b * blobs_per_body;
  for (int j = threadIdx.x; j < blobs_per_body; j += 256) {
    s0 += fb[3 * (size_t)j];
    s1 += fb[3 * (size_t)j + 1];
    s2 += fb[3 * (size_t)j + 2];
  }
  red[0][threadIdx.x] = s0;
  red[1][threadIdx.x] = s1;
  red[2][threadIdx.x] = s2;
  for (int h = 128; h > 0; h >>= 1) {
    __syncthreads();
    if (threadIdx.x < h)
      for (int k = 0; k < 3; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + h];
  }
  if (threadIdx.x == 0) {
    T *r = rec + (size_t)b * L;
    for (int k = 0; k < 3; ++k) {
      r[k] = T(x_bodies[3 * (size_t)b + k] - (origin ? origin[k] : 0.0));
      r[3 + k] = T(-red[k][0]);
    }
    for (int k = 6; k < L; ++k) r[k] = T(0);
  }
}

static cudaError_t launch_body_points(int fp32, void *rec, const double *f_segs,
                                      int segs_per_body, const double *f_blobs,
                                      int blobs_per_body, const double *x_bodies, int nbod,
                                      const double *origin, cudaStream_t st) {
  if (fp32)
    body_points_kernel<float><<<nbod, 256, 0, st>>>(static_cast<float *>(rec), f_segs,
                                                    segs_per_body, f_blobs, blobs_per_body,
                                                    x_bodies, origin);
  else
    body_points_kernel<double><<<nbod, 256, 0, st>>>(static_cast<double *>(rec), f_segs,
                                                     segs_per_body, f_blobs, blobs_per_body,
                                                     x_bodies, origin);
  count_launch();
  return cudaGetLastError();
}

// Source splits: while the point set fills less than one wave of resident
// CTAs, split the sources so that the grid does (partials summed in split
// order by launch_reduce_partials); sources per split a multiple of 64.
static cudaError_t launch_flow(FlowArgs a, int fp32, int wall, int variant, double *scratch,
                               size_t scratch_elems, cudaStream_t st) {
  if (a.n_flow <= 0) return cudaSuccess;
  const int nvar = fp32 ? kFlowVariantsF32 : kFlowVariantsF64;
  if (variant < 0 || variant >= nvar) variant = 0;
  const FlowVariant var = fp32 ? g_flow_variants_f32[variant] : g_flow_variants_f64[variant];
  const FlowFn fn = fp32 ? g_flow_f32[variant][wall ? 1 : 0] : g_flow_f64[variant][wall ? 1 : 0];
  const int per_cta = var.block * var.tpt;
  const int ctas = (a.n_flow + per_cta - 1) / per_cta;
  const int n_src = a.n_segs + a.n_points;
  int resident = 1;
  cudaError_t e = fn(a, dim3(0), st, &resident);
  if (e != cudaSuccess) return e;
  const long slots = (long)resident * num_sms();
  int splits = (int)std::max(1L, slots / std::max(1, ctas));
  splits = std::min({splits, kMaxSplits, std::max(1, n_src / 64)});
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
  e = fn(a, dim3(ctas, splits), st, nullptr);
  count_launch();
  if (e != cudaSuccess) return e;
  if (splits > 1) return launch_reduce_partials(final_out, scratch, 3 * a.n_flow, splits, 0, st);
  return cudaSuccess;
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
  int variant[2] = {0, 0};  // launch variant per precision (TFS_FP64, TFS_FP32C)
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
      (rc = alloc_dev(&f->rec_blobs, record_bytes(0, 3) * ((size_t)nb + num_bodies))) ||
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
  const double *origin = fp32 ? f->origin : nullptr;  // FP64 records stay absolute
  cudaError_t e;
  if (f->ns > 0 && (e = launch_pack(fp32, 6, f->rec_segs, f->x_segs, f->f_segs, f->ns, origin,
                                    f->stream)) != cudaSuccess)
    return cuda_fail(e, "pack kernel");
  if (f->nb > 0 && (e = launch_pack(fp32, 3, f->rec_blobs, f->x_blobs, f->f_blobs, f->nb, origin,
                                    f->stream)) != cudaSuccess)
    return cuda_fail(e, "pack kernel");
  int n_points = f->nb;
  if (remove_net_force) {
    char *body_rec = static_cast<char *>(f->rec_blobs) + record_bytes(fp32, 3) * (size_t)f->nb;
    e = launch_body_points(fp32, body_rec, f->f_segs, f->segs_per_body, f->f_blobs,
                           f->blobs_per_body, f->x_bodies, f->nbod, origin, f->stream);
    if (e != cudaSuccess) return cuda_fail(e, "body-point kernel");
    n_points += f->nbod;
  }
  FlowArgs a{};
  a.x_flow = f->x_flow;
  a.n_flow = f->nflow;
  a.rec_segs = f->rec_segs;
  a.n_segs = f->ns;
  a.rec_points = f->rec_blobs;
  a.n_points = n_points;
  a.origin = f->origin;
  a.prefac = 1.0 / (8.0 * 3.14159265358979323846264338327950288 * mu);
  a.out = f->v_flow;
  e = launch_flow(a, fp32, f->blobs_per_body == 0, f->variant[fp32], f->scratch,
                  f->scratch_elems, f->stream);
  if (e != cudaSuccess) return cuda_fail(e, "flow kernel");
  return TFS_OK;
}

int tfs_flow_num_variants(int precision) {
  return precision == TFS_FP32C ? kFlowVariantsF32 : kFlowVariantsF64;
}

int tfs_flow_set_variant(tfs_flow *f, int variant) {
  if (f == nullptr) return fail(TFS_EINVAL, "null flow handle");
  if (variant < 0 || variant >= tfs_flow_num_variants(f->precision))
    return fail(TFS_EINVAL, "variant %d out of range", variant);
  f->variant[f->precision == TFS_FP32C] = variant;
  return TFS_OK;
}

int tfs_flow_autotune(tfs_flow *f, double mu, int remove_net_force, int reps, int *best,
                      double *best_ms) {
  if (f == nullptr) return fail(TFS_EINVAL, "null flow handle");
  if (reps < 1) reps = 1;
  const int fp32 = f->precision == TFS_FP32C;
  const int nvar = tfs_flow_num_variants(f->precision);
  cudaEvent_t ev[2];
  cudaError_t e = cudaEventCreate(&ev[0]);
  if (e != cudaSuccess) return cuda_fail(e, "cudaEventCreate");
  e = cudaEventCreate(&ev[1]);
  if (e != cudaSuccess) {
    cudaEventDestroy(ev[0]);
    return cuda_fail(e, "cudaEventCreate");
  }
  int chosen = 0, rc = TFS_OK;
  float chosen_ms = 0.f;
  for (int v = 0; v < nvar && rc == TFS_OK; ++v) {
    f->variant[fp32] = v;
    if ((rc = tfs_flow_velocities(f, mu, remove_net_force)) != TFS_OK) break;  // warm-up
    cudaEventRecord(ev[0], f->stream);
    for (int r = 0; r < reps && rc == TFS_OK; ++r) rc = tfs_flow_velocities(f, mu, remove_net_force);
    cudaEventRecord(ev[1], f->stream);
    if ((e = cudaEventSynchronize(ev[1])) != cudaSuccess) {
      rc = cuda_fail(e, "flow autotune");
      break;
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ev[0], ev[1]);
    ms /= reps;
    if (v == 0 || ms < chosen_ms) {
      chosen = v;
      chosen_ms = ms;
    }
  }
  cudaEventDestroy(ev[0]);
  cudaEventDestroy(ev[1]);
  f->variant[fp32] = chosen;
  if (rc != TFS_OK) return rc;
  if (best) *best = chosen;
  if (best_ms) *best_ms = chosen_ms;
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
