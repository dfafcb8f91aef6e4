// tfs_api.cu -- the C ABI of libtfs_gb300.so (include/tfs_gb300.h): the
// solver object that stands in for the reference's rpy_mobility_solver
// (src/cilia/mobility/rpy_mobility_solver.{hpp,cu}).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <map>
#include <mutex>
#include <tuple>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/tfs_gb300.h"
#include "tfs_kernels.h"

namespace tfs {

static constexpr double kPiHost = 3.14159265358979323846264338327950288;

static std::atomic<long long> g_launches{0};
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
void count_launch_n(long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
long long launch_count() { return g_launches.load(std::memory_order_relaxed); }

static thread_local std::string g_last_error;

// Process-wide tuning results: (precision, combination, Ns, Nb) -> tuning, so
// solvers created after an autotune of the same sizes start tuned.
static std::mutex g_tune_mutex;
// queue kinds are cached under kQueueTuneKey + kind
static constexpr int kQueueTuneKey = 100;
static std::map<std::tuple<int, int, int, int>, TileTuning> g_tune_cache;

void tune_cache_store(int precision, int combo, int ns, int nb, TileTuning t) {
  std::lock_guard<std::mutex> lock(g_tune_mutex);
  g_tune_cache[std::make_tuple(precision, combo, ns, nb)] = t;
}

bool tune_cache_lookup(int precision, int combo, int ns, int nb, TileTuning *t) {
  std::lock_guard<std::mutex> lock(g_tune_mutex);
  auto it = g_tune_cache.find(std::make_tuple(precision, combo, ns, nb));
  if (it == g_tune_cache.end()) return false;
  *t = it->second;
  return true;
}

int fail(int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

int cuda_fail(cudaError_t e, const char *what) {
  return fail(TFS_ECUDA, "%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
}

}  // namespace tfs

using namespace tfs;

#include "tfs_solver.h"

// Next free event pair for the timing hook (nullptr when timing is off).
static cudaEvent_t *next_events(tfs_solver *s) {
  if (!s->timing) return nullptr;
  if (s->events_used + 2 > s->events.size()) {
    if (s->events.size() >= 2 * 4096) return nullptr;  // bounded
    for (int k = 0; k < 2; ++k) {
      cudaEvent_t e;
      if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
      s->events.push_back(e);
    }
  }
  cudaEvent_t *p = &s->events[s->events_used];
  s->events_used += 2;
  return p;
}

static void free_all(tfs_solver *s) {
  for (cudaEvent_t e : s->events) cudaEventDestroy(e);
  s->events.clear();
  if (s->pready_ev) cudaEventDestroy(s->pready_ev);
  if (s->pdone_ev) cudaEventDestroy(s->pdone_ev);
  pres_free(s);
  solve_free(s);
  cudaFree(s->x_segs);
  cudaFree(s->f_segs);
  cudaFree(s->v_segs);
  cudaFree(s->x_blobs);
  cudaFree(s->f_blobs);
  cudaFree(s->v_blobs);
  cudaFree(s->f_rep);
  cudaFree(s->origin);
  cudaFree(s->origin_cnt);
  cudaFree(s->rec_segs);
  cudaFree(s->rec_blobs);
  cudaFree(s->rec_segs_x2);
  cudaFree(s->rec_blobs_x2);
  cudaFree(s->rec_ff);
  cudaFree(s->bar_grid);
  cudaFree(s->wc_z);
  cudaFree(s->wc_f);
  cudaFree(s->scratch);
  cudaFree(s->stage32);
  cudaFree(s->qjobs_dev);
  cudaFree(s->qcount);
  if (s->own_stream) cudaStreamDestroy(s->own_stream);
}

int tfs::alloc_dev(void **p, size_t bytes) {
  if (bytes == 0) bytes = 16;
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(TFS_ENOMEM, "cudaMalloc(%zu bytes): %s", bytes, cudaGetErrorString(e));
  }
  return TFS_OK;
}

int tfs::ensure_origin(tfs_solver *s) {
  if (!s->origin_dirty) return TFS_OK;
  cudaError_t e = launch_origin(s->x_segs, s->ns, s->x_blobs, s->nb, s->origin, s->origin_cnt,
                                s->stream);
  if (e != cudaSuccess) return cuda_fail(e, "origin kernel");
  s->origin_dirty = false;
  return TFS_OK;
}

int tfs::pack(tfs_solver *s, int segs) {
  const int fp32 = s->cfg.precision == TFS_FP32C;
  cudaError_t e = segs ? launch_pack(fp32, 6, s->rec_segs, s->x_segs, s->f_segs, s->ns,
                                     s->origin, s->stream)
                       : launch_pack(fp32, 3, s->rec_blobs, s->x_blobs, s->f_blobs, s->nb,
                                     s->origin, s->stream);
  if (e != cudaSuccess) return cuda_fail(e, "pack kernel");
  if (fp32) {
    e = segs ? launch_pack_x2(6, s->rec_segs_x2, s->x_segs, s->f_segs, s->ns, s->origin, s->stream)
             : launch_pack_x2(3, s->rec_blobs_x2, s->x_blobs, s->f_blobs, s->nb, s->origin,
                              s->stream);
    if (e != cudaSuccess) return cuda_fail(e, "pack kernel");
  }
  return TFS_OK;
}

TileArgs tfs::base_args(tfs_solver *s) {
  TileArgs a{};
  a.origin = s->origin;
  a.fp32 = s->cfg.precision == TFS_FP32C;
  a.scale = 1.0 / (8.0 * 3.14159265358979323846264338327950288 * s->cfg.mu);
  a.splits = 0;
  return a;
}

// ---------------------------------------------------------------------------
// Work-queue products: the solver's job lists and one launch per product.
// ---------------------------------------------------------------------------
static QueueJob make_job(tfs_solver *s, bool tgt_segs, bool src_segs, bool src_blobs, int mode) {
  QueueJob j{};
  j.tgt_rec = tgt_segs ? s->rec_segs : s->rec_blobs;
  j.n_tgt = tgt_segs ? s->ns : s->nb;
  j.a_tgt = tgt_segs ? s->cfg.a_seg : s->cfg.a_blob;
  j.out = tgt_segs ? s->v_segs : s->v_blobs;
  j.vd = tgt_segs ? 6 : 3;
  j.mode = mode;
  j.scale = 1.0 / (8.0 * kPiHost * s->cfg.mu);
  if (src_segs) {
    j.src_a = s->rec_segs;
    j.n_a = s->ns;
    j.a_a = s->cfg.a_seg;
    if (src_blobs) {
      j.src_b = s->rec_blobs;
      j.n_b = s->nb;
      j.a_b = s->cfg.a_blob;
    }
  } else {
    j.src_a = s->rec_blobs;
    j.n_a = s->nb;
    j.a_a = s->cfg.a_blob;
  }
  // the pair constants exactly as the tile kernel forms them (in FP64, then
  // rounded to the kernel's precision)
  for (int set = 0; set < 2; ++set) {
    const double ai = j.a_tgt, aj = set == 0 ? j.a_a : j.a_b;
    const double q[5] = {ai, aj, (ai + aj) * (ai + aj), (ai * ai + aj * aj) / 3.0,
                         -(ai * ai + aj * aj)};
    for (int k = 0; k < 5; ++k) {
      j.pc64[set][k] = q[k];
      j.pc32[set][k] = (float)q[k];
    }
  }
  queue_chunking(j.n_a + j.n_b, s->ns + s->nb, &j.chunk, &j.n_chunks);
  // segment-target and blob-target jobs of one launch use disjoint partials
  // and arrival counters
  j.partial = s->scratch + (tgt_segs ? (size_t)0 : (size_t)kMaxSplits * 6 * s->ns);
  j.block_done = s->qcount + 2 + (tgt_segs ? 0 : (s->ns + 31) / 32);
  return j;
}

static void add_job(tfs_solver *s, int kind, bool tgt_segs, bool src_segs, bool src_blobs,
                    int mode) {
  const QueueJob j = make_job(s, tgt_segs, src_segs, src_blobs, mode);
  if (j.n_tgt > 0 && j.n_a + j.n_b > 0) s->qjobs[kind][s->qjobs_n[kind]++] = j;
}

// Job lists of every launch kind (segment-target jobs first: their pairs cost
// more), copied to the device once.
static int build_queue_jobs(tfs_solver *s) {
  for (int k = 0; k < kNumQueueKinds; ++k) s->qjobs_n[k] = 0;
  add_job(s, QK_MSS, true, true, false, OUT_ASSIGN);
  add_job(s, QK_MBS, false, true, false, OUT_ASSIGN);
  add_job(s, QK_SEGSRC, true, true, false, OUT_ASSIGN);
  add_job(s, QK_SEGSRC, false, true, false, OUT_ASSIGN);
  add_job(s, QK_MSB, true, false, true, OUT_ACCUMULATE);
  add_job(s, QK_MBB, false, false, true, OUT_ASSIGN);
  add_job(s, QK_GRAND, true, true, true, OUT_ASSIGN);
  add_job(s, QK_GRAND, false, true, true, OUT_ASSIGN);
  TFS_CUDA(cudaMemcpy(s->qjobs_dev, s->qjobs, sizeof s->qjobs, cudaMemcpyHostToDevice),
           "copy queue jobs");
  return TFS_OK;
}

static int queue_sources(int kind) {
  return kind == QK_GRAND ? Q_SEG_BLOB : (kind == QK_MSB || kind == QK_MBB) ? Q_BLOB : Q_SEG;
}

int tfs::queue_product(tfs_solver *s, int kind) {
  const int fp32 = s->cfg.precision == TFS_FP32C;
  const int src = queue_sources(kind);
  int rc;
  if (fp32 && (rc = ensure_origin(s)) != TFS_OK) return rc;
  // the records of both particle kinds: sources, and the targets' positions
  cudaError_t e;
  if (s->ns > 0) {
    e = launch_pack(fp32, 6, s->rec_segs, s->x_segs, s->f_segs, s->ns, s->origin, s->stream);
    if (e != cudaSuccess) return cuda_fail(e, "pack kernel");
  }
  if (s->nb > 0) {
    e = launch_pack(fp32, 3, s->rec_blobs, s->x_blobs, s->f_blobs, s->nb, s->origin, s->stream);
    if (e != cudaSuccess) return cuda_fail(e, "pack kernel");
  }
  if (s->product_service != nullptr)  // one launch shared with other swimmers' products
    return product_service_run(s->product_service, s, kind, fp32, src);
  e = launch_queue(fp32, s->qtune[fp32][kind], src, s->qjobs_dev + 2 * kind, s->qjobs[kind],
                   s->qjobs_n[kind], s->qcount, s->stream, next_events(s));
  if (e != cudaSuccess) return cuda_fail(e, "RPY work-queue kernel");
  return TFS_OK;
}

// Product of one block into `out` (assign or accumulate).
int tfs::product(tfs_solver *s, bool tgt_segs, bool src_segs, bool src_blobs, int mode) {
  int rc;
  if (src_segs == src_blobs) return fail(TFS_EINVAL, "one source set per block product");
  const int n_tgt = tgt_segs ? s->ns : s->nb;
  const int n_src = src_segs ? s->ns : s->nb;
  if (n_tgt == 0) return TFS_OK;
  if (n_src == 0) {
    if (mode == OUT_ASSIGN)
      TFS_CUDA(cudaMemsetAsync(tgt_segs ? s->v_segs : s->v_blobs, 0,
                               sizeof(double) * (tgt_segs ? 6 : 3) * n_tgt, s->stream),
               "cudaMemsetAsync");
    return TFS_OK;
  }
  const int kind = tgt_segs ? (src_segs ? QK_MSS : QK_MSB) : (src_segs ? QK_MBS : QK_MBB);
  if ((kind == QK_MSB) != (mode == OUT_ACCUMULATE))
    return fail(TFS_EINVAL, "M_sb accumulates, the other blocks assign");
  if ((rc = queue_product(s, kind)) != TFS_OK) return rc;
  return TFS_OK;
}

extern "C" {

int tfs_config_default(tfs_config *cfg, int nswim, int nfil, int nseg, int nblob) {
  if (cfg == nullptr) return fail(TFS_EINVAL, "null config");
  std::memset(cfg, 0, sizeof *cfg);
  cfg->nswim = nswim;
  cfg->nfil = nfil;
  cfg->nseg = nseg;
  cfg->nblob = nblob;
  cfg->mu = 1.0;
  cfg->a_seg = 1.0;
  cfg->a_blob = 1.0;
  // END_FORCE_MAGNITUDE = DIMENSIONLESS_FORCE*KB/(DL*DL*NSEG*NSEG) with the
  // default DL = 2.6 (globals.cu:14-18, config.hpp:261,275), truncated to int.
  cfg->end_force_magnitude =
      nseg > 0 ? (int)(220.0 * 1800.0 / (2.6 * 2.6 * (double)nseg * (double)nseg)) : 0;
  cfg->repulsive_force_factor = 2.0;
  cfg->free_body = 1;
  cfg->precision = TFS_FP64;
  return TFS_OK;
}

int tfs_solver_create(const tfs_config *cfg, tfs_solver **out) {
  if (cfg == nullptr || out == nullptr) return fail(TFS_EINVAL, "null argument");
  *out = nullptr;
  if (cfg->nswim < 0 || cfg->nfil < 0 || cfg->nseg < 0 || cfg->nblob < 0)
    return fail(TFS_EINVAL, "negative size");
  const long long ns = (long long)cfg->nswim * cfg->nfil * cfg->nseg;
  const long long nb = (long long)cfg->nswim * cfg->nblob;
  if (ns > (1LL << 26) || nb > (1LL << 26))
    return fail(TFS_EINVAL, "too many particles (%lld segments, %lld blobs; max 2^26 each)", ns, nb);
  if (!(cfg->mu > 0) || !(cfg->a_seg > 0) || !(cfg->a_blob > 0))
    return fail(TFS_EINVAL, "mu and radii must be positive");
  if (cfg->precision != TFS_FP64 && cfg->precision != TFS_FP32C)
    return fail(TFS_EINVAL, "unknown precision %d", cfg->precision);
  if (ns > 0 && cfg->nseg <= 0) return fail(TFS_EINVAL, "nseg must be positive");

  tfs_solver *s = new (std::nothrow) tfs_solver;
  if (s == nullptr) return fail(TFS_ENOMEM, "host allocation failed");
  s->cfg = *cfg;
  for (int p = 0; p < 2; ++p) {
    for (int c = 0; c < kNumCombos; ++c) {
      s->tune[p][c] = TileTuning{0, 1};
      tune_cache_lookup(p, c, (int)ns, (int)nb, &s->tune[p][c]);
    }
    for (int k = 0; k < kNumQueueKinds; ++k) {
      TileTuning t{0, 1};
      tune_cache_lookup(p, kQueueTuneKey + k, (int)ns, (int)nb, &t);
      s->qtune[p][k] = t.variant;
    }
  }
  s->ns = (int)ns;
  s->nb = (int)nb;
  cudaGetDevice(&s->device);
  int rc = TFS_OK;
  cudaError_t e = cudaStreamCreateWithFlags(&s->own_stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete s;
    return cuda_fail(e, "cudaStreamCreate");
  }
  s->stream = s->own_stream;
  const size_t dsz = sizeof(double);
  // split partials: tile launches need kMaxSplits x the larger target set,
  // a queue launch up to kMaxSplits chunks of both target sets at once
  s->scratch_elems = (size_t)kMaxSplits * (size_t)(6 * ns + 3 * nb);
  const size_t qcount_elems = 2 + (size_t)(ns + 31) / 32 + (size_t)(nb + 31) / 32;
  if ((rc = alloc_dev((void **)&s->x_segs, dsz * 3 * ns)) ||
      (rc = alloc_dev((void **)&s->f_segs, dsz * 6 * ns)) ||
      (rc = alloc_dev((void **)&s->v_segs, dsz * 6 * ns)) ||
      (rc = alloc_dev((void **)&s->x_blobs, dsz * 3 * nb)) ||
      (rc = alloc_dev((void **)&s->f_blobs, dsz * 3 * nb)) ||
      (rc = alloc_dev((void **)&s->v_blobs, dsz * 3 * nb)) ||
      (rc = alloc_dev((void **)&s->f_rep, dsz * 3 * nb)) ||
      (rc = alloc_dev((void **)&s->origin, dsz * origin_elems())) ||
      (rc = alloc_dev((void **)&s->origin_cnt, 2 * sizeof(unsigned))) ||
      (rc = alloc_dev(&s->rec_segs, record_bytes(0, 6) * ns)) ||
      (rc = alloc_dev(&s->rec_blobs, record_bytes(0, 3) * nb)) ||
      (rc = alloc_dev(&s->rec_segs_x2, 80 * (size_t)ns)) ||
      (rc = alloc_dev(&s->rec_blobs_x2, 48 * (size_t)nb)) ||
      (rc = alloc_dev(&s->rec_ff, ff_record_bytes() * nb)) ||
      (rc = alloc_dev(&s->bar_grid, barrier_grid_bytes(ns, nb))) ||
      (rc = alloc_dev((void **)&s->scratch, dsz * s->scratch_elems)) ||
      (rc = alloc_dev((void **)&s->qjobs_dev, sizeof s->qjobs)) ||
      (rc = alloc_dev((void **)&s->qcount, sizeof(unsigned) * qcount_elems)) ||
      (rc = solve_alloc(s))) {
    free_all(s);
    delete s;
    return rc;
  }
  // GMRES warm starts read f_blobs before any force is written
  // (mobility_solver.cpp:35-39 zeroes the host copy), and the FP32 origin
  // (the mean particle position) reads the segment positions even before a
  // caller sets them (the body reference matrices need only the blobs):
  // zero every particle array, so that no earlier allocation's contents can
  // leak into a result.
  cudaMemsetAsync(s->x_segs, 0, dsz * 3 * ns, s->stream);
  cudaMemsetAsync(s->f_segs, 0, dsz * 6 * ns, s->stream);
  cudaMemsetAsync(s->v_segs, 0, dsz * 6 * ns, s->stream);
  cudaMemsetAsync(s->x_blobs, 0, dsz * 3 * nb, s->stream);
  cudaMemsetAsync(s->v_blobs, 0, dsz * 3 * nb, s->stream);
  cudaMemsetAsync(s->f_blobs, 0, dsz * 3 * nb, s->stream);
  cudaMemsetAsync(s->f_rep, 0, dsz * 3 * nb, s->stream);
  cudaMemsetAsync(s->origin, 0, dsz * origin_elems(), s->stream);
  cudaMemsetAsync(s->origin_cnt, 0, 2 * sizeof(unsigned), s->stream);
  cudaMemsetAsync(s->qcount, 0, sizeof(unsigned) * qcount_elems, s->stream);
  e = cudaStreamSynchronize(s->stream);
  if (e == cudaSuccess && (rc = build_queue_jobs(s)) != TFS_OK) {
    free_all(s);
    delete s;
    return rc;
  }
  if (e != cudaSuccess) {
    free_all(s);
    delete s;
    return cuda_fail(e, "solver initialisation");
  }
  *out = s;
  return TFS_OK;
}

int tfs_solver_destroy(tfs_solver *s) {
  if (s == nullptr) return TFS_OK;
  cudaStreamSynchronize(s->stream);
  free_all(s);
  delete s;
  return TFS_OK;
}

int tfs_solver_set_stream(tfs_solver *s, void *stream) {
  TFS_CHECK_SOLVER(s);
  s->stream = stream ? (cudaStream_t)stream : s->own_stream;
  return TFS_OK;
}

int tfs_solver_set_precision(tfs_solver *s, int precision) {
  TFS_CHECK_SOLVER(s);
  if (precision != TFS_FP64 && precision != TFS_FP32C)
    return fail(TFS_EINVAL, "unknown precision %d", precision);
  s->cfg.precision = precision;
  return TFS_OK;
}

int tfs_solver_device_buffers(tfs_solver *s, tfs_device_buffers *out) {
  TFS_CHECK_SOLVER(s);
  if (out == nullptr) return fail(TFS_EINVAL, "null output");
  out->x_segs = s->x_segs;
  out->f_segs = s->f_segs;
  out->v_segs = s->v_segs;
  out->x_blobs = s->x_blobs;
  out->f_blobs = s->f_blobs;
  out->v_blobs = s->v_blobs;
  out->f_blobs_repulsion = s->f_rep;
  // the caller may write positions directly
  s->origin_dirty = true;
  return TFS_OK;
}

int tfs_solver_positions_updated(tfs_solver *s) {
  TFS_CHECK_SOLVER(s);
  s->origin_dirty = true;
  return TFS_OK;
}

static int h2d(tfs_solver *s, double *dst, const double *src, size_t n, const char *what) {
  TFS_CHECK_SOLVER(s);
  if (n == 0) return TFS_OK;
  if (src == nullptr) return fail(TFS_EINVAL, "%s: null host pointer", what);
  TFS_CUDA(cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyHostToDevice, s->stream), what);
  return TFS_OK;
}

static int d2h(tfs_solver *s, double *dst, const double *src, size_t n, const char *what) {
  TFS_CHECK_SOLVER(s);
  if (n == 0) return TFS_OK;
  if (dst == nullptr) return fail(TFS_EINVAL, "%s: null host pointer", what);
  TFS_CUDA(cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyDeviceToHost, s->stream), what);
  return TFS_OK;
}

}  // extern "C"

namespace {
__global__ void widen_kernel(double *__restrict__ dst, const float *__restrict__ src, size_t n) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = (double)src[i];
}
__global__ void narrow_kernel(float *__restrict__ dst, const double *__restrict__ src, size_t n) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = (float)src[i];
}
int ensure_stage32(tfs_solver *s) {
  if (s->stage32 != nullptr) return TFS_OK;
  return alloc_dev((void **)&s->stage32,
                   sizeof(float) * std::max<size_t>(6 * (size_t)s->ns, 3 * (size_t)s->nb));
}
}  // namespace

int tfs::h2d_f32(tfs_solver *s, double *dst, const float *src, size_t n, const char *what) {
  if (n == 0) return TFS_OK;
  if (src == nullptr) return fail(TFS_EINVAL, "%s: null host pointer", what);
  int rc = ensure_stage32(s);
  if (rc != TFS_OK) return rc;
  TFS_CUDA(cudaMemcpyAsync(s->stage32, src, n * sizeof(float), cudaMemcpyHostToDevice, s->stream),
           what);
  widen_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s->stream>>>(dst, s->stage32, n);
  count_launch();
  TFS_CUDA(cudaGetLastError(), what);
  return TFS_OK;
}

int tfs::d2h_f32(tfs_solver *s, float *dst, const double *src, size_t n, const char *what) {
  if (n == 0) return TFS_OK;
  if (dst == nullptr) return fail(TFS_EINVAL, "%s: null host pointer", what);
  int rc = ensure_stage32(s);
  if (rc != TFS_OK) return rc;
  narrow_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s->stream>>>(s->stage32, src, n);
  count_launch();
  TFS_CUDA(cudaGetLastError(), what);
  TFS_CUDA(cudaMemcpyAsync(dst, s->stage32, n * sizeof(float), cudaMemcpyDeviceToHost, s->stream),
           what);
  return TFS_OK;
}

extern "C" {

int tfs_copy_segment_positions_to_device_f32(tfs_solver *s, const float *x) {
  TFS_CHECK_SOLVER(s);
  s->origin_dirty = true;
  return h2d_f32(s, s->x_segs, x, 3 * (size_t)s->ns, "copy_segment_positions_to_device");
}
int tfs_copy_segment_forces_to_device_f32(tfs_solver *s, const float *f) {
  TFS_CHECK_SOLVER(s);
  return h2d_f32(s, s->f_segs, f, 6 * (size_t)s->ns, "copy_segment_forces_to_device");
}
int tfs_copy_blob_positions_to_device_f32(tfs_solver *s, const float *x) {
  TFS_CHECK_SOLVER(s);
  s->origin_dirty = true;
  return h2d_f32(s, s->x_blobs, x, 3 * (size_t)s->nb, "copy_blob_positions_to_device");
}
int tfs_copy_blob_forces_to_device_f32(tfs_solver *s, const float *f) {
  TFS_CHECK_SOLVER(s);
  return h2d_f32(s, s->f_blobs, f, 3 * (size_t)s->nb, "copy_blob_forces_to_device");
}
int tfs_copy_interparticle_blob_forces_to_host_f32(tfs_solver *s, float *f) {
  TFS_CHECK_SOLVER(s);
  return d2h_f32(s, f, s->f_rep, 3 * (size_t)s->nb, "copy_interparticle_blob_forces_to_host");
}
int tfs_copy_blob_velocities_to_host_f32(tfs_solver *s, float *v) {
  TFS_CHECK_SOLVER(s);
  return d2h_f32(s, v, s->v_blobs, 3 * (size_t)s->nb, "copy_blob_velocities_to_host");
}
int tfs_copy_segment_velocities_to_host_f32(tfs_solver *s, float *v) {
  TFS_CHECK_SOLVER(s);
  return d2h_f32(s, v, s->v_segs, 6 * (size_t)s->ns, "copy_segment_velocities_to_host");
}

int tfs_copy_segment_positions_to_device(tfs_solver *s, const double *x) {
  TFS_CHECK_SOLVER(s);
  s->origin_dirty = true;
  return h2d(s, s->x_segs, x, 3 * (size_t)s->ns, "copy_segment_positions_to_device");
}
int tfs_copy_segment_forces_to_device(tfs_solver *s, const double *f) {
  TFS_CHECK_SOLVER(s);
  return h2d(s, s->f_segs, f, 6 * (size_t)s->ns, "copy_segment_forces_to_device");
}
int tfs_copy_blob_positions_to_device(tfs_solver *s, const double *x) {
  TFS_CHECK_SOLVER(s);
  s->origin_dirty = true;
  return h2d(s, s->x_blobs, x, 3 * (size_t)s->nb, "copy_blob_positions_to_device");
}
int tfs_copy_blob_forces_to_device(tfs_solver *s, const double *f) {
  TFS_CHECK_SOLVER(s);
  return h2d(s, s->f_blobs, f, 3 * (size_t)s->nb, "copy_blob_forces_to_device");
}
int tfs_copy_interparticle_blob_forces_to_host(tfs_solver *s, double *f) {
  TFS_CHECK_SOLVER(s);
  return d2h(s, f, s->f_rep, 3 * (size_t)s->nb, "copy_interparticle_blob_forces_to_host");
}
int tfs_copy_blob_velocities_to_host(tfs_solver *s, double *v) {
  TFS_CHECK_SOLVER(s);
  return d2h(s, v, s->v_blobs, 3 * (size_t)s->nb, "copy_blob_velocities_to_host");
}
int tfs_copy_segment_velocities_to_host(tfs_solver *s, double *v) {
  TFS_CHECK_SOLVER(s);
  return d2h(s, v, s->v_segs, 6 * (size_t)s->ns, "copy_segment_velocities_to_host");
}

int tfs_apply_interparticle_forces(tfs_solver *s) {
  TFS_CHECK_SOLVER(s);
  int rc = ensure_origin(s);
  if (rc != TFS_OK) return rc;
  BarrierArgs a{};
  a.f_segs = s->f_segs;
  a.f_blobs_repulsion = s->f_rep;
  a.x_segs = s->x_segs;
  a.x_blobs = s->x_blobs;
  a.origin = s->origin;
  a.num_segs = s->ns;
  a.num_blobs = s->nb;
  a.nseg = s->cfg.nseg > 0 ? s->cfg.nseg : 1;
  a.a_seg = s->cfg.a_seg;
  a.a_blob = s->cfg.a_blob;
  a.end_force_magnitude = s->cfg.end_force_magnitude;
  a.repulsive_force_factor = s->cfg.repulsive_force_factor;
  a.free_body = s->cfg.free_body;
  a.grid = s->bar_grid;
  cudaError_t e = launch_barrier(a, s->stream);
  if (e != cudaSuccess) return cuda_fail(e, "barrier kernel");
  return TFS_OK;
}

int tfs_wait_for_device(tfs_solver *s) {
  TFS_CHECK_SOLVER(s);
  TFS_CUDA(cudaStreamSynchronize(s->stream), "wait_for_device");
  TFS_CUDA(cudaGetLastError(), "wait_for_device");
  return TFS_OK;
}

int tfs_evaluate_segment_segment_mobility(tfs_solver *s) {
  TFS_CHECK_SOLVER(s);
  if (s->pres != nullptr) return pres_hook(s, true, true);
  return product(s, true, true, false, OUT_ASSIGN);
}
int tfs_evaluate_segment_blob_mobility(tfs_solver *s) {
  TFS_CHECK_SOLVER(s);
  if (s->pres != nullptr) return pres_hook(s, true, false);
  return product(s, true, false, true, OUT_ACCUMULATE);
}
int tfs_evaluate_blob_blob_mobility(tfs_solver *s) {
  TFS_CHECK_SOLVER(s);
  if (s->pres != nullptr) return pres_hook(s, false, false);
  return product(s, false, false, true, OUT_ASSIGN);
}
int tfs_evaluate_weakly_coupled_segment_mobility(tfs_solver *s) {
  TFS_CHECK_SOLVER(s);
  const int nseg = s->cfg.nseg;
  if (nseg < 1 || s->ns % nseg != 0)
    return fail(TFS_EINVAL, "the segments must form whole filaments of nseg = %d", nseg);
  const int nfil = s->ns / nseg;
  int rc;
  if (s->wc_z == nullptr &&
      ((rc = alloc_dev((void **)&s->wc_z, sizeof(double) * 3 * nfil)) != TFS_OK ||
       (rc = alloc_dev((void **)&s->wc_f, sizeof(double) * 3 * nfil)) != TFS_OK))
    return rc;
  cudaError_t e = launch_msf(s->x_segs, s->f_segs, nfil, nseg, s->cfg.a_seg, s->cfg.mu, s->wc_z,
                             s->wc_f, s->v_segs, s->stream);
  if (e != cudaSuccess) return cuda_fail(e, "weakly coupled segment product");
  return TFS_OK;
}

int tfs_evaluate_blob_blob_mobility_ff(tfs_solver *s) {
  TFS_CHECK_SOLVER(s);
  int rc;
  if ((rc = ensure_origin(s)) != TFS_OK) return rc;
  cudaError_t e = launch_bb_ff(s->x_blobs, s->f_blobs, s->nb, s->origin, s->cfg.a_blob,
                               1.0 / (8.0 * 3.14159265358979323846264338327950288 * s->cfg.mu), s->rec_ff, s->v_blobs, s->scratch,
                               s->scratch_elems, s->stream);
  if (e != cudaSuccess) return cuda_fail(e, "float-float blob-blob product");
  return TFS_OK;
}
int tfs_evaluate_blob_segment_mobility(tfs_solver *s) {
  TFS_CHECK_SOLVER(s);
  if (s->pres != nullptr) return pres_hook(s, false, true);
  return product(s, false, true, false, OUT_ASSIGN);
}

int tfs_evaluate_full_mobility(tfs_solver *s, double *v_segs_host, double *v_blobs_host) {
  TFS_CHECK_SOLVER(s);
  int rc;
  if ((rc = tfs_evaluate_segment_segment_mobility(s)) != TFS_OK) return rc;
  if ((rc = tfs_evaluate_segment_blob_mobility(s)) != TFS_OK) return rc;
  if (v_segs_host && (rc = tfs_copy_segment_velocities_to_host(s, v_segs_host)) != TFS_OK)
    return rc;
  if ((rc = tfs_evaluate_blob_blob_mobility(s)) != TFS_OK) return rc;
  if ((rc = tfs_evaluate_blob_segment_mobility(s)) != TFS_OK) return rc;
  if (v_blobs_host && (rc = tfs_copy_blob_velocities_to_host(s, v_blobs_host)) != TFS_OK)
    return rc;
  return TFS_OK;
}

int tfs_apply_grand_mobility(tfs_solver *s) {
  TFS_CHECK_SOLVER(s);
  // both target kinds against both source sets in one work-queue launch
  if (s->ns > 0 && s->nb > 0) return queue_product(s, QK_GRAND);
  if (s->ns > 0) return product(s, true, true, false, OUT_ASSIGN);
  if (s->nb > 0) return product(s, false, false, true, OUT_ASSIGN);
  return TFS_OK;
}

int tfs_solver_enable_kernel_timing(tfs_solver *s, int enable) {
  TFS_CHECK_SOLVER(s);
  s->timing = enable != 0;
  s->events_used = 0;
  return TFS_OK;
}

int tfs_solver_kernel_timing(tfs_solver *s, double *ms, int capacity, int *launches) {
  TFS_CHECK_SOLVER(s);
  if (launches == nullptr || (ms == nullptr && capacity > 0)) return fail(TFS_EINVAL, "null output");
  TFS_CUDA(cudaStreamSynchronize(s->stream), "kernel timing");
  const int n = (int)(s->events_used / 2);
  for (int k = 0; k < n && k < capacity; ++k) {
    float t = 0.f;
    TFS_CUDA(cudaEventElapsedTime(&t, s->events[2 * k], s->events[2 * k + 1]),
             "cudaEventElapsedTime");
    ms[k] = t;
  }
  *launches = n;
  s->events_used = 0;
  return TFS_OK;
}

static const char *queue_kind_name(int k) {
  static const char *names[kNumQueueKinds] = {"seg<-seg", "blob<-seg", "seg,blob<-seg",
                                              "seg<-blob", "blob<-blob", "grand"};
  return names[k];
}

static const char *combo_name(int c) {
  static const char *names[kNumCombos] = {"seg<-seg", "seg<-blob", "blob<-blob", "blob<-seg",
                                          "seg<-seg+blob", "blob<-seg+blob"};
  return names[c];
}

// Time every (variant, CTAs-per-SM) candidate of every combination the
// solver uses, on its current positions and forces, and keep the fastest.
int tfs_solver_autotune(tfs_solver *s, int precision_mask, int reps) {
  TFS_CHECK_SOLVER(s);
  if (reps <= 0) reps = 2;
  const int saved_precision = s->cfg.precision;
  const bool saved_timing = s->timing;
  s->timing = false;
  static const int kWaves[] = {1, 2, 4};
  cudaEvent_t e0, e1;
  TFS_CUDA(cudaEventCreate(&e0), "cudaEventCreate");
  TFS_CUDA(cudaEventCreate(&e1), "cudaEventCreate");
  std::string report = "{";
  int rc = TFS_OK;
  for (int p = 0; p < 2 && rc == TFS_OK; ++p) {
    if (!(precision_mask & (1 << p))) continue;
    s->cfg.precision = p;  // TFS_FP64 = 0, TFS_FP32C = 1
    if (p == TFS_FP32C && (rc = ensure_origin(s)) != TFS_OK) break;
    if (s->ns > 0 && (rc = pack(s, 1)) != TFS_OK) break;
    if (s->nb > 0 && (rc = pack(s, 0)) != TFS_OK) break;
    if (report.size() > 1) report += ",";
    report += std::string("\"") + (p ? "fp32c" : "fp64") + "\":{";
    bool first_combo = true;
    // tile launches serve only the blob-blob product of the kernel-sequence
    // GMRES now; every other product goes through the work queue (below)
    for (int c = C_BB; c == C_BB && rc == TFS_OK; ++c) {
      const bool tgt_segs = (c == C_SS || c == C_SB || c == C_SX);
      const bool src_segs = (c != C_SB && c != C_BB);
      const bool src_blobs = (c == C_SB || c == C_BB || c == C_SX || c == C_BX);
      if ((tgt_segs ? s->ns : s->nb) == 0 || (src_segs && s->ns == 0) ||
          (src_blobs && s->nb == 0))
        continue;
      TileArgs a = base_args(s);
      a.x_tgt = tgt_segs ? s->x_segs : s->x_blobs;
      a.n_tgt = tgt_segs ? s->ns : s->nb;
      a.a_tgt = tgt_segs ? s->cfg.a_seg : s->cfg.a_blob;
      a.out = tgt_segs ? s->v_segs : s->v_blobs;
      int fda, fdb = 0;
      if (src_segs) {
        a.src_a = s->rec_segs; a.src_a2 = s->rec_segs_x2; a.n_a = s->ns; a.a_a = s->cfg.a_seg;
        fda = 6;
        if (src_blobs) {
          a.src_b = s->rec_blobs; a.src_b2 = s->rec_blobs_x2; a.n_b = s->nb;
          a.a_b = s->cfg.a_blob; fdb = 3;
        }
      } else {
        a.src_a = s->rec_blobs; a.src_a2 = s->rec_blobs_x2; a.n_a = s->nb; a.a_a = s->cfg.a_blob;
        fda = 3;
      }
      const int vd = tgt_segs ? 6 : 3;
      const int nvar = p ? kNumVariantsF32 : kNumVariantsF64;
      float best_ms = 1e30f;
      TileTuning best{0, 1};
      std::string cands;
      for (int v = 0; v < nvar && rc == TFS_OK; ++v) {
        for (int cps : kWaves) {
          TileTuning t{v, cps};
          cudaError_t e = launch_tile(a, vd, fda, fdb, t, s->scratch, s->scratch_elems, OUT_ASSIGN,
                                      s->stream);  // warm-up
          // the best of three timed groups of reps launches (less sensitive
          // to another process's work on the GPU than one group)
          float ms = 1e30f;
          for (int trial = 0; trial < 3 && e == cudaSuccess; ++trial) {
            cudaEventRecord(e0, s->stream);
            for (int r = 0; r < reps && e == cudaSuccess; ++r)
              e = launch_tile(a, vd, fda, fdb, t, s->scratch, s->scratch_elems, OUT_ASSIGN,
                              s->stream);
            cudaEventRecord(e1, s->stream);
            if (e == cudaSuccess) e = cudaEventSynchronize(e1);
            float tm = 0.f;
            if (e == cudaSuccess) cudaEventElapsedTime(&tm, e0, e1);
            ms = std::min(ms, tm / reps);
          }
          if (e != cudaSuccess) {
            rc = cuda_fail(e, "autotune launch");
            break;
          }
          const TileVariant tv = p ? g_variants_f32[v] : g_variants_f64[v];
          char buf[96];
          snprintf(buf, sizeof buf, "%s[%d,%d,%d,%d,%d,%.4f]", cands.empty() ? "" : ",",
                   tv.block, tv.tpt, tv.ts, tv.x2, cps, ms);
          cands += buf;
          if (ms < best_ms) {
            best_ms = ms;
            best = t;
          }
        }
      }
      if (rc != TFS_OK) break;
      s->tune[p][c] = best;
      tune_cache_store(p, c, s->ns, s->nb, best);
      const TileVariant bv = p ? g_variants_f32[best.variant] : g_variants_f64[best.variant];
      char buf[256];
      snprintf(buf, sizeof buf,
               "%s\"%s\":{\"block\":%d,\"tpt\":%d,\"ts\":%d,\"x2\":%d,\"waves\":%d,"
               "\"ms\":%.4f,\"candidates\":[",
               first_combo ? "" : ",", combo_name(c), bv.block, bv.tpt, bv.ts, bv.x2,
               best.waves, best_ms);
      report += buf;
      report += cands + "]}";
      first_combo = false;
    }
    // work-queue launches: every variant of every kind the solver has
    for (int k = 0; k < kNumQueueKinds && rc == TFS_OK; ++k) {
      if (s->qjobs_n[k] == 0) continue;
      const int nvar = p ? kNumQueueVariantsF32 : kNumQueueVariantsF64;
      const int src = queue_sources(k);
      float best_ms = 1e30f;
      int best = 0;
      std::string cands;
      for (int v = 0; v < nvar && rc == TFS_OK; ++v) {
        cudaError_t e = launch_queue(p, v, src, s->qjobs_dev + 2 * k, s->qjobs[k], s->qjobs_n[k],
                                     s->qcount, s->stream);  // warm-up
        float ms = 1e30f;
        for (int trial = 0; trial < 3 && e == cudaSuccess; ++trial) {
          cudaEventRecord(e0, s->stream);
          for (int r = 0; r < reps && e == cudaSuccess; ++r)
            e = launch_queue(p, v, src, s->qjobs_dev + 2 * k, s->qjobs[k], s->qjobs_n[k],
                             s->qcount, s->stream);
          cudaEventRecord(e1, s->stream);
          if (e == cudaSuccess) e = cudaEventSynchronize(e1);
          float tm = 0.f;
          if (e == cudaSuccess) cudaEventElapsedTime(&tm, e0, e1);
          ms = std::min(ms, tm / reps);
        }
        if (e != cudaSuccess) {
          rc = cuda_fail(e, "autotune queue launch");
          break;
        }
        const QueueVariant qv = p ? g_qvariants_f32[v] : g_qvariants_f64[v];
        char buf[96];
        snprintf(buf, sizeof buf, "%s[%d,%d,%d,0,0,%.4f]", cands.empty() ? "" : ",", qv.block,
                 qv.tpt, qv.ts, ms);
        cands += buf;
        if (ms < best_ms) {
          best_ms = ms;
          best = v;
        }
      }
      if (rc != TFS_OK) break;
      s->qtune[p][k] = best;
      tune_cache_store(p, kQueueTuneKey + k, s->ns, s->nb, TileTuning{best, 1});
      const QueueVariant bq = p ? g_qvariants_f32[best] : g_qvariants_f64[best];
      char buf[256];
      snprintf(buf, sizeof buf,
               "%s\"queue %s\":{\"block\":%d,\"tpt\":%d,\"ts\":%d,\"x2\":0,\"waves\":0,"
               "\"ms\":%.4f,\"candidates\":[",
               first_combo ? "" : ",", queue_kind_name(k), bq.block, bq.tpt, bq.ts, best_ms);
      report += buf;
      report += cands + "]}";
      first_combo = false;
    }
    report += "}";
  }
  report += "}";
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  s->cfg.precision = saved_precision;
  s->timing = saved_timing;
  if (rc == TFS_OK) s->tuning_report = report;
  return rc;
}

int tfs_solver_set_tuning(tfs_solver *s, int precision, int combo, int variant, int waves) {
  TFS_CHECK_SOLVER(s);
  if (precision != TFS_FP64 && precision != TFS_FP32C)
    return fail(TFS_EINVAL, "unknown precision %d", precision);
  if (combo < 0 || combo >= kNumCombos) return fail(TFS_EINVAL, "combination %d out of range", combo);
  const int nvar = precision == TFS_FP32C ? kNumVariantsF32 : kNumVariantsF64;
  if (variant < 0 || variant >= nvar) return fail(TFS_EINVAL, "variant %d out of range", variant);
  if (waves < 1 || waves > 64) return fail(TFS_EINVAL, "waves out of range");
  s->tune[precision][combo] = TileTuning{variant, waves};
  return TFS_OK;
}

int tfs_solver_set_queue_variant(tfs_solver *s, int precision, int kind, int variant) {
  TFS_CHECK_SOLVER(s);
  if (precision != TFS_FP64 && precision != TFS_FP32C)
    return fail(TFS_EINVAL, "unknown precision %d", precision);
  if (kind < 0 || kind >= kNumQueueKinds) return fail(TFS_EINVAL, "kind %d out of range", kind);
  if (variant < 0 || variant >= tfs_num_queue_variants(precision))
    return fail(TFS_EINVAL, "variant %d out of range", variant);
  s->qtune[precision][kind] = variant;
  return TFS_OK;
}

int tfs_num_queue_variants(int precision) {
  return precision == TFS_FP32C ? kNumQueueVariantsF32 : kNumQueueVariantsF64;
}

int tfs_num_tile_variants(int precision) {
  return precision == TFS_FP32C ? kNumVariantsF32 : kNumVariantsF64;
}

int tfs_solver_tuning_report(tfs_solver *s, char *buf, size_t len, size_t *needed) {
  TFS_CHECK_SOLVER(s);
  const size_t n = s->tuning_report.size() + 1;
  if (needed) *needed = n;
  if (buf != nullptr && len > 0) {
    const size_t k = std::min(len - 1, s->tuning_report.size());
    std::memcpy(buf, s->tuning_report.data(), k);
    buf[k] = 0;
  }
  return TFS_OK;
}

const char *tfs_last_error(void) { return g_last_error.c_str(); }

long long tfs_kernel_launch_count(void) { return g_launches.load(); }

}  // extern "C"

namespace tfs {
// Device bytes of a solver of these sizes (tfs_solver_create's and the
// solve's allocations, the cooperative-GMRES buffers at their largest),
// plus 1 MB for the small ones.
size_t solver_bytes_estimate(const tfs_config *cfg) {
  const size_t ns = (size_t)cfg->nswim * cfg->nfil * cfg->nseg, nb = (size_t)cfg->nswim * cfg->nblob;
  const size_t n = 3 * nb + 6, m = std::min<size_t>(350, n);
  const size_t doubles = 15 * ns + 12 * nb + (size_t)kMaxSplits * (6 * ns + 3 * nb) +
                         n * (m + 1) + (m + 1) * (m + 1) + 16 * n + 57 * nb + 256 * (m + 1);
  return 8 * doubles + 200 * ns + 200 * nb + ((size_t)1 << 20);
}
}  // namespace tfs
