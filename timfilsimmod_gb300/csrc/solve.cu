// solve.cu -- the free-body mobility solve behind the C ABI: body geometry
// and pose, make_body_reference_matrices, and compute_velocities
// (src/cilia/mobility/mobility_solver.cpp:2574-2659 and :2950-3047) on the
// device, with the GMRES of gmres.cu. In FP32C mode the linear solve is
// iterative refinement: FP64 residuals r = rhs - A x around inner GMRES
// solves whose blob-blob products run in FP32 with compensated sums.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>
#include <new>
#include <mutex>
#include <deque>
#include <condition_variable>
#include <chrono>

#include "tfs_solver.h"

using namespace tfs;

namespace {

void rot_mat(double *R, const double *q) {
  const double s = q[0], a = q[1], b = q[2], c = q[3];
  R[0] = 1.0 - 2.0 * b * b - 2.0 * c * c;  // (0,0)
  R[4] = 1.0 - 2.0 * a * a - 2.0 * c * c;  // (1,1)
  R[8] = 1.0 - 2.0 * a * a - 2.0 * b * b;  // (2,2)
  R[1] = 2.0 * a * b + 2.0 * s * c;        // (1,0)
  R[3] = 2.0 * a * b - 2.0 * s * c;        // (0,1)
  R[2] = 2.0 * a * c - 2.0 * s * b;        // (2,0)
  R[6] = 2.0 * a * c + 2.0 * s * b;        // (0,2)
  R[5] = 2.0 * b * c + 2.0 * s * a;        // (2,1)
  R[7] = 2.0 * b * c - 2.0 * s * a;        // (1,2)
}

// Each 3x3 block B of the 6x6 `in` becomes R B R^T (mobility_solver.cpp:1455-1467).
void rotate_blocks(double *out, const double *in, const double *R) {
  for (int bi = 0; bi < 2; ++bi)
    for (int bj = 0; bj < 2; ++bj) {
      double RB[9];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
          double t = 0.0;
          for (int k = 0; k < 3; ++k) t += R[i + 3 * k] * in[(3 * bi + k) + 6 * (3 * bj + j)];
          RB[i + 3 * j] = t;
        }
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
          double t = 0.0;
          for (int k = 0; k < 3; ++k) t += RB[i + 3 * k] * R[j + 3 * k];
          out[(3 * bi + i) + 6 * (3 * bj + j)] = t;
        }
    }
}

bool invert6(double *A) {
  double M[6][12];
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < 6; ++j) {
      M[i][j] = A[i + 6 * j];
      M[i][6 + j] = (i == j) ? 1.0 : 0.0;
    }
  for (int k = 0; k < 6; ++k) {
    int p = k;
    for (int i = k + 1; i < 6; ++i)
      if (std::fabs(M[i][k]) > std::fabs(M[p][k])) p = i;
    if (M[p][k] == 0.0) return false;
    if (p != k)
      for (int j = 0; j < 12; ++j) std::swap(M[k][j], M[p][j]);
    const double piv = M[k][k];
    for (int j = 0; j < 12; ++j) M[k][j] /= piv;
    for (int i = 0; i < 6; ++i) {
      if (i == k) continue;
      const double f = M[i][k];
      for (int j = 0; j < 12; ++j) M[i][j] -= f * M[k][j];
    }
  }
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < 6; ++j) A[i + 6 * j] = M[i][6 + j];
  return true;
}

// The 72 doubles of the rotated body matrices, passed to the device as a
// kernel argument (copied at launch, so the host needs no staging buffer that
// must outlive the copy, and no wait).
struct Mats72 {
  double v[72];
};

__global__ void set_mats_kernel(Mats72 m, double *__restrict__ dst) {
  if (threadIdx.x < 72) dst[threadIdx.x] = m.v[threadIdx.x];
}

int upload_mats(tfs_solver *s) {
  rotate_blocks(s->mats_host, s->body_mob_ref, s->pose.R);
  rotate_blocks(s->mats_host + 36, s->ktkinv_ref, s->pose.R);
  Mats72 m;
  std::memcpy(m.v, s->mats_host, sizeof m.v);
  set_mats_kernel<<<1, 96, 0, s->stream>>>(m, s->mats);
  TFS_CUDA(cudaGetLastError(), "upload body matrices");
  count_launch();
  return TFS_OK;
}

GmresArgs gmres_args(tfs_solver *s, const double *rhs, double *f_blobs, double *v_bodies,
                     GmresScalars *st, double tol, int fp32) {
  GmresArgs g{};
  g.n = s->n;
  g.nb = s->nb;
  g.max_iter = s->max_iter;
  g.tol = tol;
  g.mu = s->cfg.mu;
  g.a_blob = s->cfg.a_blob;
  g.fp32 = fp32;
  g.x_blobs = s->x_blobs;
  g.diff = s->diff;
  g.origin = s->origin;
  g.rec64 = s->rec_blobs;
  g.rec32 = s->rec_blobs;
  g.rec32x2 = s->rec_blobs_x2;
  g.mats = s->mats;
  g.rhs = rhs;
  g.soln = s->soln;
  g.Q = s->Q;
  g.H = s->H;
  g.beta = s->beta;
  g.cs = s->cs;
  g.sn = s->sn;
  g.y = s->y;
  g.z = s->z;
  g.tmp = s->tmp;
  g.v = s->vtmp;
  g.f_blobs = f_blobs;
  g.v_bodies = v_bodies;
  g.st = st;
  g.G = s->gG;
  g.blobs_per_cta = s->g_blobs_per_cta;
  g.part = s->gpart;
  g.part_stride = s->max_iter + 1;
  g.part6 = s->gpart6;
  g.counters = s->gcounters;
  g.h1 = s->gh1;
  g.h2 = s->gh2;
  return g;
}

// v = M_bb (the blob records just packed), in FP64 or FP32C; skipped when
// *skip is set.
int mbb_product(tfs_solver *s, int fp32, const int *skip) {
  TileArgs a = base_args(s);
  a.fp32 = fp32;
  a.x_tgt = s->x_blobs;
  a.n_tgt = s->nb;
  a.a_tgt = s->cfg.a_blob;
  a.src_a = s->rec_blobs;
  a.src_a2 = s->rec_blobs_x2;
  a.n_a = s->nb;
  a.a_a = s->cfg.a_blob;
  a.out = s->vtmp;
  a.skip = skip;
  cudaError_t e = launch_tile(a, 3, 3, 0, s->tune[fp32][C_BB], s->scratch, s->scratch_elems,
                              OUT_ASSIGN, s->stream);
  if (e != cudaSuccess) return cuda_fail(e, "blob-blob product");
  return TFS_OK;
}

int poll(tfs_solver *s, int which, GmresScalars *out) {
  TFS_CUDA(cudaMemcpyAsync(s->gst_host + which, s->gst + which, sizeof(GmresScalars),
                           cudaMemcpyDeviceToHost, s->stream),
           "read solver state");
  TFS_CUDA(cudaStreamSynchronize(s->stream), "read solver state");
  *out = s->gst_host[which];
  return TFS_OK;
}

// Both scalar sets (inner solve, refinement) with one copy and one wait.
int poll_both(tfs_solver *s, GmresScalars *inner, GmresScalars *outer) {
  TFS_CUDA(cudaMemcpyAsync(s->gst_host, s->gst, 2 * sizeof(GmresScalars), cudaMemcpyDeviceToHost,
                           s->stream),
           "read solver state");
  TFS_CUDA(cudaStreamSynchronize(s->stream), "read solver state");
  *inner = s->gst_host[0];
  *outer = s->gst_host[1];
  return TFS_OK;
}

// One chunk of Arnoldi steps (preconditioner, M_bb product, CGS2, norm,
// Givens) as launched by gmres_run. Every kernel reads the step index from
// the device scalars and skips once the solve is done, so a chunk is the same
// launch sequence every time for given arguments.
int launch_chunk(tfs_solver *s, const GmresArgs &g, int fp32) {
  cudaError_t e;
  int rc;
  for (int k = 0; k < s->chunk; ++k) {
    if ((e = launch_gmres_precond(g, s->stream)) != cudaSuccess)
      return cuda_fail(e, "gmres preconditioner");
    if ((rc = mbb_product(s, fp32, &s->gst->done)) != TFS_OK) return rc;
    if ((e = launch_gmres_arnoldi(g, s->stream)) != cudaSuccess) return cuda_fail(e, "gmres arnoldi");
  }
  return TFS_OK;
}

// The chunk as a CUDA graph, captured on first use for these arguments
// (nullptr: launch the kernels directly -- kernel timing on, or capture
// unavailable).
cudaGraphExec_t chunk_graph(tfs_solver *s, const GmresArgs &g, int fp32, long long *kernels) {
  if (!s->graphs_enabled || s->timing) return nullptr;
  const TileTuning tune = s->tune[fp32][C_BB];
  for (auto &c : s->chunk_graphs)
    if (c.chunk == s->chunk && c.tune.variant == tune.variant && c.tune.waves == tune.waves &&
        std::memcmp(&c.args, &g, sizeof g) == 0) {
      *kernels = c.kernels;
      return c.exec;
    }
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  const long long before = launch_count();
  if (cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    cudaGetLastError();
    s->graphs_enabled = false;
    return nullptr;
  }
  const int rc = launch_chunk(s, g, fp32);
  const cudaError_t e = cudaStreamEndCapture(s->stream, &graph);
  const long long recorded = launch_count() - before;
  count_launch_n(-recorded);  // recorded, not launched
  if (rc != TFS_OK || e != cudaSuccess || graph == nullptr ||
      cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) {
    cudaGetLastError();
    if (graph) cudaGraphDestroy(graph);
    s->graphs_enabled = false;
    return nullptr;
  }
  cudaGraphDestroy(graph);
  s->chunk_graphs.push_back({g, tune, s->chunk, exec, recorded});
  *kernels = recorded;
  return exec;
}

// GMRES on rhs with warm start / solution (f_blobs, v_bodies).
int gmres_run(tfs_solver *s, const double *rhs, double *f_blobs, double *v_bodies, double tol,
              int fp32, int *iters) {
  if (s->nb == 0) return fail(TFS_ESTATE, "the free-body solve needs blobs");
  GmresScalars *st = s->gst;
  const GmresArgs g = gmres_args(s, rhs, f_blobs, v_bodies, st, tol, fp32);
  cudaError_t e;
  if ((e = launch_gmres_start(g, s->stream)) != cudaSuccess) return cuda_fail(e, "gmres start");
  int rc = mbb_product(s, fp32, &st->done);
  if (rc) return rc;
  if ((e = launch_gmres_residual(g, s->stream)) != cudaSuccess)
    return cuda_fail(e, "gmres residual");
  GmresScalars h{};
  const int max_chunks = s->max_iter / std::max(1, s->chunk) + 2;
  for (int c = 0; c < max_chunks; ++c) {
    if ((rc = poll(s, 0, &h)) != TFS_OK) return rc;
    if (h.done) break;
    long long kernels = 0;
    if (cudaGraphExec_t exec = chunk_graph(s, g, fp32, &kernels)) {
      if ((e = cudaGraphLaunch(exec, s->stream)) != cudaSuccess) return cuda_fail(e, "gmres chunk");
      count_launch_n(kernels);
    } else if ((rc = launch_chunk(s, g, fp32)) != TFS_OK) {
      return rc;
    }
  }
  if ((rc = poll(s, 0, &h)) != TFS_OK) return rc;
  if (!h.done) return fail(TFS_ENOTCONV, "GMRES did not finish within %d steps", s->max_iter);
  if (h.status) return fail(TFS_ENAN, "GMRES residual is not finite");
  if (h.iters > 0 && (e = launch_gmres_finish(g, s->stream)) != cudaSuccess)
    return cuda_fail(e, "gmres finish");
  *iters = h.iters;
  s->last_rel = h.rel;
  return TFS_OK;
}

// Inner GMRES of the refinement as one cooperative kernel (FP32 M_bb).
// The persistent kernel's arguments for one inner solve of s in shape sh.
PgArgs persistent_args(tfs_solver *s, const PgShape &sh, const double *rhs, double *f_blobs,
                       double *v_bodies, double tol, int vec64) {
  GmresArgs g = gmres_args(s, rhs, f_blobs, v_bodies, s->gst, tol, 1);
  g.G = sh.G;
  g.blobs_per_cta = sh.blobs_per_cta;
  PgArgs p{};
  p.g = g;
  p.x32 = s->pg_x32;
  p.rec = s->pg_rec;
  p.mpart = s->pg_mpart;
  p.p6 = s->pg_p6;
  p.ps = s->pg_ps;
  p.pd1 = s->pg_pd1;
  p.pd2 = s->pg_pd2;
  p.aux = s->pg_aux;
  p.bar = s->pg_bar;
  p.P = sh.P;
  p.TB = sh.TB;
  p.tbs = sh.tbs;
  p.S = sh.S;
  p.chunk = sh.chunk;
  p.vec64 = vec64;
  p.Kr = vec64 ? sh.Kr64 : sh.Kr;
  p.dyn_smem = vec64 ? sh.dyn_smem64 : sh.dyn_smem;
  p.a = (float)s->cfg.a_blob;
  const double ab = s->cfg.a_blob;
  p.pc_asum2 = (float)((2.0 * ab) * (2.0 * ab));
  p.pc_s = (float)(2.0 * ab * ab / 3.0);
  p.pc_s3 = (float)(-2.0 * ab * ab);
  p.minv = 6.0 * 3.14159265358979323846264338327950288 * s->cfg.mu * ab;
  p.scale = 1.0 / (8.0 * 3.14159265358979323846264338327950288 * s->cfg.mu);
  // its only use is the refinement's inner solve, whose warm start (the
  // correction dx) refine_residual_kernel has just set to zero
  p.zero_start = 1;
  p.bar_extra = s->pg_stall ? 1u : 0u;
  return p;
}

// The result of a finished inner persistent solve from its scalars.
int persistent_result(const GmresScalars &h, int *iters) {
  if (h.status == 2) return fail(TFS_ETIMEOUT, "persistent GMRES: a grid barrier timed out");
  if (h.status == 1) return fail(TFS_ENAN, "GMRES residual is not finite");
  if (!h.done) return fail(TFS_ESTATE, "persistent GMRES ended without a result");
  *iters = h.iters;
  return TFS_OK;
}

// Queues an inner persistent solve on s->stream; its scalars (s->gst[0])
// are read by the caller's next poll.
int gmres_launch_persistent(tfs_solver *s, const double *rhs, double *f_blobs, double *v_bodies,
                            double tol, int vec64) {
  const PgArgs p = persistent_args(s, s->pg, rhs, f_blobs, v_bodies, tol, vec64);
  TFS_CUDA(cudaMemcpyAsync(s->pg_gp, &p, sizeof p, cudaMemcpyHostToDevice, s->stream),
           "persistent GMRES arguments");
  TFS_CUDA(cudaMemsetAsync(p.bar, 0, 4 * sizeof(unsigned), s->stream), "persistent GMRES barrier");
  cudaError_t e = launch_gmres_persistent(s->pg_gp, s->pg_cmap, p.P, p.dyn_smem, vec64, s->stream);
  if (e != cudaSuccess) return cuda_fail(e, "persistent GMRES");
  return TFS_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
// Inner solves of several swimmers in one cooperative launch. A swimmer's
// solve runs on a fixed number of CTAs chosen from its size alone, so its
// result does not depend on which others share the launch. A waiting thread
// that finds no launch being prepared becomes the leader: while the previous
// launch still runs on the GPU (and the waiting solves fill fewer CTAs than
// the SMs) it lets requests gather, then takes them in arrival order up to
// the SM count, queues their launch on the service's stream behind each
// swimmer's inputs, marks each swimmer's completion event and wakes the
// owners, who wait for that event on their own streams. Launches queue back
// to back on the service's stream; the host never waits for one to finish
// except to reuse one of its argument staging slots.
// ---------------------------------------------------------------------------
namespace tfs {

struct GmresService {
  struct Req {
    tfs_solver *s;
    PgArgs args;
    bool done;
    int rc;
  };
  static constexpr int kSlots = 8;  // host staging of the launch arguments
  struct Slot {
    PgArgs *args = nullptr;
    int2 *map = nullptr;
    cudaEvent_t copied = nullptr;
  };
  std::mutex m;
  std::condition_variable cv;
  std::deque<Req *> pending;
  bool busy = false;
  int sms = 1;
  cudaStream_t stream = nullptr;
  PgArgs *dev_args = nullptr;
  int2 *dev_map = nullptr;
  Slot slot[kSlots];
  int next_slot = 0;
  cudaEvent_t last = nullptr;  // the latest launch's completion
  bool launched = false;
  long long launches = 0, solves = 0;

  int waiting_ctas() const {
    int c = 0;
    for (const Req *q : pending) c += q->args.P;
    return c;
  }
  bool gpu_busy() const { return launched && cudaEventQuery(last) == cudaErrorNotReady; }

  // Queues one launch of the solves in batch (the leader, without the lock).
  int launch(std::vector<Req *> &batch) {
    Slot &sl = slot[next_slot];
    next_slot = (next_slot + 1) % kSlots;
    TFS_CUDA(cudaEventSynchronize(sl.copied), "service: staging slot");
    int ctas = 0;
    size_t dyn = 0;
    for (size_t q = 0; q < batch.size(); ++q) {
      Req *r = batch[q];
      TFS_CUDA(cudaStreamWaitEvent(stream, r->s->ready_ev, 0), "service: wait for inputs");
      TFS_CUDA(cudaMemsetAsync(r->args.bar, 0, 4 * sizeof(unsigned), stream), "service: barrier");
      sl.args[q] = r->args;
      for (int c = 0; c < r->args.P; ++c) sl.map[ctas + c] = make_int2((int)q, c);
      ctas += r->args.P;
      dyn = std::max(dyn, r->args.dyn_smem);
    }
    TFS_CUDA(cudaMemcpyAsync(dev_args, sl.args, sizeof(PgArgs) * batch.size(),
                             cudaMemcpyHostToDevice, stream),
             "service: arguments");
    TFS_CUDA(cudaMemcpyAsync(dev_map, sl.map, sizeof(int2) * ctas, cudaMemcpyHostToDevice, stream),
             "service: map");
    TFS_CUDA(cudaEventRecord(sl.copied, stream), "service: staging slot");
    cudaError_t e = launch_gmres_persistent(dev_args, dev_map, ctas, dyn, 0, stream);
    if (e != cudaSuccess) return cuda_fail(e, "service: persistent GMRES");
    for (Req *r : batch) TFS_CUDA(cudaEventRecord(r->s->done_ev, stream), "service: completion");
    TFS_CUDA(cudaEventRecord(last, stream), "service: completion");
    return TFS_OK;
  }

  // Queues s's inner solve in a shared launch; s->stream waits for it, and
  // its scalars (s->gst[0]) are read by the caller's next poll.
  int solve(tfs_solver *s, const double *rhs, double *f_blobs, double *v_bodies, double tol) {
    Req r{s, persistent_args(s, s->pg_group, rhs, f_blobs, v_bodies, tol, 0), false, TFS_OK};
    TFS_CUDA(cudaEventRecord(s->ready_ev, s->stream), "service: inputs ready");
    std::unique_lock<std::mutex> g(m);
    pending.push_back(&r);
    cv.notify_all();
    while (!r.done) {
      if (busy) {
        cv.wait(g);
        continue;
      }
      busy = true;
      while (waiting_ctas() < sms && gpu_busy()) cv.wait_for(g, std::chrono::microseconds(20));
      std::vector<Req *> batch;
      int ctas = 0;
      while (!pending.empty() && (batch.empty() || ctas + pending.front()->args.P <= sms)) {
        ctas += pending.front()->args.P;
        batch.push_back(pending.front());
        pending.pop_front();
      }
      g.unlock();
      const int lrc = launch(batch);
      g.lock();
      if (lrc == TFS_OK) {
        launched = true;
        ++launches;
        solves += (long long)batch.size();
      }
      for (Req *q : batch) {
        q->done = true;
        q->rc = lrc;
      }
      busy = false;
      cv.notify_all();
    }
    g.unlock();
    if (r.rc != TFS_OK) return r.rc;
    TFS_CUDA(cudaStreamWaitEvent(s->stream, s->done_ev, 0), "service: wait for the solve");
    return TFS_OK;
  }
};

GmresService *service_create() {
  GmresService *sv = new (std::nothrow) GmresService();
  if (sv == nullptr) return nullptr;
  sv->sms = num_sms();
  bool ok = cudaStreamCreateWithFlags(&sv->stream, cudaStreamNonBlocking) == cudaSuccess &&
            cudaMalloc(&sv->dev_args, sizeof(PgArgs) * kMaxPgCtas) == cudaSuccess &&
            cudaMalloc(&sv->dev_map, sizeof(int2) * kMaxPgCtas) == cudaSuccess &&
            cudaEventCreateWithFlags(&sv->last, cudaEventDisableTiming) == cudaSuccess;
  for (auto &sl : sv->slot)
    ok = ok && cudaHostAlloc(&sl.args, sizeof(PgArgs) * kMaxPgCtas, cudaHostAllocDefault) == cudaSuccess &&
         cudaHostAlloc(&sl.map, sizeof(int2) * kMaxPgCtas, cudaHostAllocDefault) == cudaSuccess &&
         cudaEventCreateWithFlags(&sl.copied, cudaEventDisableTiming) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    service_destroy(sv);
    return nullptr;
  }
  return sv;
}

void service_destroy(GmresService *sv) {
  if (sv == nullptr) return;
  if (sv->stream) cudaStreamSynchronize(sv->stream);
  if (sv->dev_args) cudaFree(sv->dev_args);
  if (sv->dev_map) cudaFree(sv->dev_map);
  for (auto &sl : sv->slot) {
    if (sl.args) cudaFreeHost(sl.args);
    if (sl.map) cudaFreeHost(sl.map);
    if (sl.copied) cudaEventDestroy(sl.copied);
  }
  if (sv->last) cudaEventDestroy(sv->last);
  if (sv->stream) cudaStreamDestroy(sv->stream);
  delete sv;
}

// CTAs of a swimmer's solve in a shared launch: the fewest the kernel allows
// (kPgServiceBlobsPerCta blobs each), at most the SMs.
int service_attach(GmresService *sv, tfs_solver *s) {
  if (sv == nullptr || s == nullptr) return fail(TFS_EINVAL, "null argument");
  if (s->cfg.precision != TFS_FP32C) return fail(TFS_ESTATE, "only FP32C inner solves are shared");
  if (!s->pg_ok) return fail(TFS_ESTATE, "the persistent GMRES kernel cannot serve this swimmer");
  const int nb = s->nb;
  const int want =
      std::min(sv->sms, (nb + kPgServiceBlobsPerCta - 1) / kPgServiceBlobsPerCta);
  PgShape sh{};
  if (!pg_grid(nb, want, s->max_iter, &sh) || sh.G > s->pg.G || sh.S > s->pg.S)
    return fail(TFS_ESTATE, "no persistent GMRES shape for %d blobs on %d CTAs", nb, want);
  for (cudaEvent_t *ev : {&s->ready_ev, &s->done_ev})
    if (*ev == nullptr && cudaEventCreateWithFlags(ev, cudaEventDisableTiming) != cudaSuccess) {
      cudaGetLastError();
      return fail(TFS_ECUDA, "event creation failed");
    }
  s->pg_group = sh;
  s->service = sv;
  return TFS_OK;
}

void service_stats(GmresService *sv, long long *launches, long long *solves) {
  std::lock_guard<std::mutex> g(sv->m);
  if (launches) *launches = sv->launches;
  if (solves) *solves = sv->solves;
}

}  // namespace tfs

namespace {

// Refinement cycles from the iterate in s->xr: the residual in float-float
// arithmetic, an inner GMRES on it, the update. The inner solve runs in the
// shared launch of s->service, else on the solver's own cooperative launch
// (when enabled), else as the kernel sequence; vec64 runs the cooperative
// solve with FP64 Arnoldi vectors (on the solver's own launch) instead of
// FP32 ones. *stalled: a cycle did not reduce the residual (the inner solves
// cannot make progress on this system).
int refine_cycles(tfs_solver *s, const GmresArgs &g64, int vec64, bool first_ready, int *total,
                  int *cycles, GmresScalars *h, bool *stalled) {
  const int vel = 3 * s->nb;
  // the solver's own cooperative launch: when enabled, and for FP64 vectors
  // of a swimmer whose FP32 solves go to a shared launch
  const bool own = s->pg_ok && (s->pg_enabled || (vec64 && s->service));
  double prev_rel = 0.0;
  int rc;
  // a queued cooperative inner solve whose scalars are read with the next
  // residual's (one host wait per cycle)
  bool pending = false;
  *stalled = false;
  for (int it = 0; it <= s->max_outer; ++it) {
    // the residual's M_bb product in float-float arithmetic (FP64-grade
    // accuracy at FP32 instruction rates); the first one may have run
    // already, beside the segment products
    cudaError_t e = cudaSuccess;
    if (!(it == 0 && first_ready) &&
        (e = launch_bb_ff(s->x_blobs, s->xr, s->nb, s->origin, s->cfg.a_blob,
                          1.0 / (8.0 * 3.14159265358979323846264338327950288 * s->cfg.mu),
                          s->rec_ff, s->vtmp, s->scratch, s->scratch_elems, s->stream)) !=
            cudaSuccess)
      return cuda_fail(e, "refinement residual product");
    if ((e = launch_refine_residual(g64, s->xr, s->r, s->dx, it, s->stream)) != cudaSuccess)
      return cuda_fail(e, "refinement residual");
    if (pending) {
      GmresScalars hin{};
      int inner = 0;
      if ((rc = poll_both(s, &hin, h)) != TFS_OK || (rc = persistent_result(hin, &inner)) != TFS_OK)
        return rc;
      *total += inner;
      pending = false;
    } else if ((rc = poll(s, 1, h)) != TFS_OK) {
      return rc;
    }
    // a non-finite residual (the kernel then marks the solve done with
    // status 1): of the input itself at the first cycle, else a stall
    if (h->status && it == 0)
      return fail(TFS_ENAN, "non-finite right-hand side or warm start in the mobility solve");
    if (h->done && !h->status) break;
    // a cycle that did not reduce the residual (or a non-finite one): the
    // inner solves cannot make progress on this system
    if (h->status || !(h->rel == h->rel) || (it > 0 && !(h->rel < prev_rel)) ||
        it == s->max_outer) {
      *stalled = true;
      break;
    }
    prev_rel = h->rel;
    // the inner solve asks only for the reduction the outer target still
    // needs (with a factor 2 to spare), at most inner_tol's: a good warm
    // start then costs a few Arnoldi steps instead of a full 1e-4 reduction
    const double itol = std::max(s->inner_tol, std::min(0.5, 0.5 * s->tol / h->rel));
    int inner = 0;
    if (s->service && !vec64) {  // a shared launch (FP32 vectors)
      if ((rc = s->service->solve(s, s->r, s->dx, s->dx + vel, itol)) != TFS_OK) return rc;
      pending = true;
    } else if (own) {
      if ((rc = gmres_launch_persistent(s, s->r, s->dx, s->dx + vel, itol, vec64)) != TFS_OK)
        return rc;
      pending = true;
    } else {
      rc = gmres_run(s, s->r, s->dx, s->dx + vel, itol, 1, &inner);
      if (rc != TFS_OK && rc != TFS_ENOTCONV) return rc;
      *total += inner;
    }
    ++*cycles;
    if ((e = launch_axpy(s->xr, s->dx, s->n, s->stream)) != cudaSuccess)
      return cuda_fail(e, "refinement update");
  }
  return TFS_OK;
}

// x = 2 a - b (the linear extrapolation of two steps' solutions)
__global__ void extrapolate_kernel(double *__restrict__ x, const double *__restrict__ a,
                                   const double *__restrict__ b, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] = 2.0 * a[i] - b[i];
}

// xr (on stream st) = the caller's warm start (f_blobs, v_bodies), or, for the first solve
// of a time step after two earlier steps, 2 x_{n-1} - x_{n-2} of their final
// solutions: the blob forces and body velocity change smoothly with time, so
// the extrapolation starts the refinement several digits closer and its
// inner solve asks for less (the refined result meets the same residual)
int refine_start(tfs_solver *s, cudaStream_t st) {
  const int vel = 3 * s->nb;
  if (s->extrap_next) {
    s->extrap_next = false;
    const double *h1 = s->whist + (size_t)s->whist_head * s->n;
    const double *h2 = s->whist + (size_t)(s->whist_head ^ 1) * s->n;
    extrapolate_kernel<<<(s->n + 255) / 256, 256, 0, st>>>(s->xr, h1, h2, s->n);
    TFS_CUDA(cudaGetLastError(), "extrapolated warm start");
    count_launch();
    return TFS_OK;
  }
  TFS_CUDA(cudaMemcpyAsync(s->xr, s->f_blobs, sizeof(double) * vel, cudaMemcpyDeviceToDevice, st),
           "refinement start");
  TFS_CUDA(cudaMemcpyAsync(s->xr + vel, s->v_bodies, sizeof(double) * 6, cudaMemcpyDeviceToDevice,
                           st),
           "refinement start");
  return TFS_OK;
}

// compute_velocities' first refinement residual product, on the solver's
// second stream beside the segment products (which it does not touch): the
// warm start into xr and M_bb xr (float-float) into vtmp, with partial sums
// in a buffer of its own. The main stream waits for it before the solve.
int early_residual_product(tfs_solver *s) {
  if (s->aux_stream == nullptr) {
    if (cudaStreamCreateWithFlags(&s->aux_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&s->aux_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&s->aux_join, cudaEventDisableTiming) != cudaSuccess) {
      cudaGetLastError();
      return fail(TFS_ECUDA, "second stream creation failed");
    }
  }
  int rc;
  TFS_CUDA(cudaEventRecord(s->aux_fork, s->stream), "second stream fork");
  TFS_CUDA(cudaStreamWaitEvent(s->aux_stream, s->aux_fork, 0), "second stream fork");
  if ((rc = refine_start(s, s->aux_stream)) != TFS_OK) return rc;
  cudaError_t e = launch_bb_ff(s->x_blobs, s->xr, s->nb, s->origin, s->cfg.a_blob,
                               1.0 / (8.0 * 3.14159265358979323846264338327950288 * s->cfg.mu),
                               s->rec_ff, s->vtmp, s->ff_scratch, s->ff_scratch_elems,
                               s->aux_stream);
  if (e != cudaSuccess) return cuda_fail(e, "refinement residual product");
  TFS_CUDA(cudaEventRecord(s->aux_join, s->aux_stream), "second stream join");
  return TFS_OK;
}

// The linear solve of compute_velocities on s->rhs: plain FP64 GMRES, or
// FP32C iterative refinement. The cooperative inner solves run with FP32
// Arnoldi vectors, except while the body mobility is still the identity
// make_body_reference_matrices starts from: that preconditioner leaves the
// body rows unscaled against the blob rows, beyond what an FP32 basis
// resolves, so those solves take FP64 vectors. A refinement that stalls
// with FP32 vectors is run again from the warm start with FP64 ones, and
// one that stalls with those finishes in plain FP64 GMRES. first_ready: xr
// and its M_bb product are already there (early_residual_product).
int linear_solve(tfs_solver *s, int *iters, bool first_ready = false) {
  const int fp32 = s->cfg.precision == TFS_FP32C;
  int rc;
  if (!fp32) {
    rc = gmres_run(s, s->rhs, s->f_blobs, s->v_bodies, s->tol, 0, iters);
    s->last_outer = 1;
    return rc;
  }
  if ((rc = ensure_origin(s)) != TFS_OK) return rc;
  const int vel = 3 * s->nb;
  GmresScalars *outer = s->gst + 1;
  const GmresArgs g64 = gmres_args(s, s->rhs, nullptr, nullptr, outer, s->tol, 0);
  int total = 0, cycles = 0;
  GmresScalars h{};
  bool stalled = false;
  int vec64 = (s->bootstrap || s->vec_mode == TFS_VECTORS_FP64) ? 1 : 0;
  if ((!first_ready && (rc = refine_start(s, s->stream)) != TFS_OK) ||
      (rc = refine_cycles(s, g64, vec64, first_ready, &total, &cycles, &h, &stalled)) != TFS_OK)
    return rc;
  if (stalled && !vec64 && s->pg_ok && (s->pg_enabled || s->service)) {
    vec64 = 1;
    ++s->vec64_retries;
    if ((rc = refine_start(s, s->stream)) != TFS_OK ||
        (rc = refine_cycles(s, g64, vec64, false, &total, &cycles, &h, &stalled)) != TFS_OK)
      return rc;
  }
  if (stalled) {
    // finish in FP64 from the caller's warm start (f_blobs, v_bodies are
    // untouched so far); reported as a negative cycle count
    int it64 = 0;
    rc = gmres_run(s, s->rhs, s->f_blobs, s->v_bodies, s->tol, 0, &it64);
    *iters = total + it64;
    s->last_outer = -std::max(1, cycles);
    return rc;
  }
  TFS_CUDA(cudaMemcpyAsync(s->f_blobs, s->xr, sizeof(double) * vel, cudaMemcpyDeviceToDevice,
                           s->stream),
           "refinement result");
  TFS_CUDA(cudaMemcpyAsync(s->v_bodies, s->xr + vel, sizeof(double) * 6,
                           cudaMemcpyDeviceToDevice, s->stream),
           "refinement result");
  *iters = total;
  s->last_outer = cycles;
  s->last_rel = h.rel;
  // a solution of a time step (not one of the body-reference solves)
  if (!s->bootstrap) s->solved = true;
  return TFS_OK;
}

}  // namespace

namespace tfs {

int solve_alloc(tfs_solver *s) {
  s->n = 3 * s->nb + 6;
  s->max_iter = std::min(350, s->n);
  const size_t n = s->n, m = s->max_iter, nb3 = 3 * (size_t)s->nb;
  int rc;
  s->ff_scratch_elems = (size_t)kMaxSplits * 3 * (size_t)s->nb;
  if ((rc = alloc_dev((void **)&s->refs, 8 * nb3)) || (rc = alloc_dev((void **)&s->diff, 8 * nb3)) ||
      (rc = alloc_dev((void **)&s->mats, 8 * 72)) ||
      (rc = alloc_dev((void **)&s->Q, 8 * n * (m + 1))) ||
      (rc = alloc_dev((void **)&s->H, 8 * (m + 1) * (m + 1))) ||
      (rc = alloc_dev((void **)&s->beta, 8 * (m + 1))) ||
      (rc = alloc_dev((void **)&s->cs, 8 * (m + 1))) ||
      (rc = alloc_dev((void **)&s->sn, 8 * (m + 1))) ||
      (rc = alloc_dev((void **)&s->y, 8 * (m + 1))) || (rc = alloc_dev((void **)&s->z, 8 * n)) ||
      (rc = alloc_dev((void **)&s->tmp, 8 * n)) || (rc = alloc_dev((void **)&s->soln, 8 * n)) ||
      (rc = alloc_dev((void **)&s->rhs, 8 * n)) || (rc = alloc_dev((void **)&s->vtmp, 8 * nb3)) ||
      (rc = alloc_dev((void **)&s->v_bodies, 8 * 6)) ||
      (rc = alloc_dev((void **)&s->swimmer_f, 8 * 6)) ||
      (rc = alloc_dev((void **)&s->xr, 8 * n)) || (rc = alloc_dev((void **)&s->r, 8 * n)) ||
      (rc = alloc_dev((void **)&s->whist, 8 * 2 * n)) ||
      (rc = alloc_dev((void **)&s->ff_scratch, 8 * s->ff_scratch_elems)) ||
      (rc = alloc_dev((void **)&s->dx, 8 * n)) ||
      (rc = alloc_dev((void **)&s->gst, 2 * sizeof(GmresScalars))))
    return rc;
  s->gG = gmres_grid(std::max(1, s->nb), num_sms(), &s->g_blobs_per_cta);
  if ((rc = alloc_dev((void **)&s->gpart, 8 * (size_t)s->gG * (m + 1))) ||
      (rc = alloc_dev((void **)&s->gpart6, 8 * 6 * (size_t)s->gG)) ||
      (rc = alloc_dev((void **)&s->gh1, 8 * (m + 1))) ||
      (rc = alloc_dev((void **)&s->gh2, 8 * (m + 1))) ||
      (rc = alloc_dev((void **)&s->gcounters, 8 * sizeof(unsigned))))
    return rc;
  cudaMemsetAsync(s->gcounters, 0, 8 * sizeof(unsigned), s->stream);
  int coop = 0;
  cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, s->device);
  if (coop && s->nb > 0 && s->max_iter <= 350 && pg_grid(s->nb, num_sms(), s->max_iter, &s->pg)) {
    const size_t nb = s->nb;
    if ((rc = alloc_dev((void **)&s->pg_x32, 4 * 3 * nb)) ||
        (rc = alloc_dev((void **)&s->pg_rec, 4 * 8 * nb)) ||
        (rc = alloc_dev((void **)&s->pg_mpart, 8 * 3 * nb * (size_t)s->pg.S)) ||
        (rc = alloc_dev((void **)&s->pg_p6, 8 * pg_p6_elems(s->pg))) ||
        (rc = alloc_dev((void **)&s->pg_ps, 8 * pg_ps_elems(s->pg))) ||
        (rc = alloc_dev((void **)&s->pg_pd1, 8 * pg_pd_elems(s->pg))) ||
        (rc = alloc_dev((void **)&s->pg_pd2, 8 * pg_pd_elems(s->pg))) ||
        (rc = alloc_dev((void **)&s->pg_aux, 8 * kPgAuxElems)) ||
        (rc = alloc_dev((void **)&s->pg_bar, 4 * sizeof(unsigned))) ||
        (rc = alloc_dev((void **)&s->pg_gp, sizeof(PgArgs))) ||
        (rc = alloc_dev((void **)&s->pg_cmap, sizeof(int2) * (size_t)s->pg.P)))
      return rc;
    std::vector<int2> cmap(s->pg.P);
    for (int c = 0; c < s->pg.P; ++c) cmap[c] = make_int2(0, c);
    TFS_CUDA(cudaMemcpy(s->pg_cmap, cmap.data(), sizeof(int2) * cmap.size(), cudaMemcpyHostToDevice),
             "persistent GMRES map");
    s->pg_ok = 1;
  }
  cudaGetLastError();
  if (cudaHostAlloc((void **)&s->gst_host, 2 * sizeof(GmresScalars), cudaHostAllocDefault) !=
          cudaSuccess ||
      cudaHostAlloc((void **)&s->f6_host, 8 * 6, cudaHostAllocDefault) != cudaSuccess) {
    cudaGetLastError();
    return fail(TFS_ENOMEM, "pinned host allocation failed");
  }
  std::memset(s->body_mob_ref, 0, sizeof s->body_mob_ref);
  std::memset(s->ktkinv_ref, 0, sizeof s->ktkinv_ref);
  for (int i = 0; i < 6; ++i) {
    // identity(6) until make_body_reference_matrices (mobility_solver.cpp:112-114)
    s->body_mob_ref[i + 6 * i] = 1.0;
    s->ktkinv_ref[i + 6 * i] = 1.0;
  }
  const double q[4] = {1, 0, 0, 0};
  rot_mat(s->pose.R, q);
  std::memset(s->pose.x, 0, sizeof s->pose.x);
  cudaMemsetAsync(s->v_bodies, 0, 8 * 6, s->stream);
  cudaMemsetAsync(s->gst, 0, 2 * sizeof(GmresScalars), s->stream);
  cudaMemsetAsync(s->diff, 0, 8 * nb3, s->stream);
  rotate_blocks(s->mats_host, s->body_mob_ref, s->pose.R);
  rotate_blocks(s->mats_host + 36, s->ktkinv_ref, s->pose.R);
  if (cudaMemcpy(s->mats, s->mats_host, sizeof s->mats_host, cudaMemcpyHostToDevice) !=
      cudaSuccess)
    return fail(TFS_ECUDA, "upload body matrices");
  return TFS_OK;
}

void solve_free(tfs_solver *s) {
  if (s->aux_stream) cudaStreamSynchronize(s->aux_stream);
  if (s->aux_fork) cudaEventDestroy(s->aux_fork);
  if (s->aux_join) cudaEventDestroy(s->aux_join);
  if (s->aux_stream) cudaStreamDestroy(s->aux_stream);
  s->aux_stream = nullptr;
  s->aux_fork = s->aux_join = nullptr;
  if (s->ready_ev) cudaEventDestroy(s->ready_ev);
  if (s->done_ev) cudaEventDestroy(s->done_ev);
  s->ready_ev = s->done_ev = nullptr;
  for (auto &g : s->chunk_graphs) cudaGraphExecDestroy(g.exec);
  s->chunk_graphs.clear();
  double *bufs[] = {s->refs, s->diff, s->mats, s->Q, s->H, s->beta, s->cs, s->sn, s->y, s->z,
                    s->tmp, s->soln, s->rhs, s->vtmp, s->v_bodies, s->swimmer_f, s->xr, s->r,
                    s->dx, s->gpart, s->gpart6, s->gh1, s->gh2, s->whist, s->ff_scratch};
  for (double *b : bufs) cudaFree(b);
  cudaFree(s->gcounters);
  cudaFree(s->pg_x32);
  cudaFree(s->pg_rec);
  cudaFree(s->pg_mpart);
  cudaFree(s->pg_p6);
  cudaFree(s->pg_ps);
  cudaFree(s->pg_pd1);
  cudaFree(s->pg_pd2);
  cudaFree(s->pg_aux);
  cudaFree(s->pg_bar);
  cudaFree(s->pg_gp);
  cudaFree(s->pg_cmap);
  cudaFree(s->gst);
  if (s->gst_host) cudaFreeHost(s->gst_host);
  if (s->f6_host) cudaFreeHost(s->f6_host);
}

}  // namespace tfs

extern "C" {

int tfs_set_blob_references(tfs_solver *s, const double *refs) {
  TFS_CHECK_SOLVER(s);
  if (refs == nullptr && s->nb > 0) return fail(TFS_EINVAL, "null blob references");
  if (s->nb > 0)
    TFS_CUDA(cudaMemcpyAsync(s->refs, refs, sizeof(double) * 3 * s->nb, cudaMemcpyHostToDevice,
                             s->stream),
             "copy blob references");
  TFS_CUDA(cudaStreamSynchronize(s->stream), "copy blob references");
  s->have_refs = true;
  return tfs_set_body_pose(s, s->pose.x, nullptr);
}

int tfs_set_body_pose(tfs_solver *s, const double *x, const double *q) {
  TFS_CHECK_SOLVER(s);
  if (x == nullptr) return fail(TFS_EINVAL, "null body position");
  for (int k = 0; k < 3; ++k) s->pose.x[k] = x[k];
  if (q != nullptr) {
    const double nq = std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
    if (!(nq > 0.0)) return fail(TFS_EINVAL, "zero quaternion");
    rot_mat(s->pose.R, q);
  }
  if (!s->have_refs) return fail(TFS_ESTATE, "set the blob references first");
  cudaError_t e = launch_blob_positions(s->x_blobs, s->diff, s->refs, s->nb, s->pose, s->stream);
  if (e != cudaSuccess) return cuda_fail(e, "blob positions");
  s->origin_dirty = true;
  return upload_mats(s);
}

int tfs_set_linear_solver(tfs_solver *s, double tol, int max_iter) {
  TFS_CHECK_SOLVER(s);
  if (!(tol > 0.0) || max_iter < 1) return fail(TFS_EINVAL, "tol must be > 0, max_iter >= 1");
  const int cap = std::min(350, s->n);
  if (max_iter > cap)
    return fail(TFS_EINVAL, "max_iter %d exceeds the Krylov storage of %d columns", max_iter, cap);
  s->tol = tol;
  s->max_iter = max_iter;
  return TFS_OK;
}

int tfs_set_refinement(tfs_solver *s, double inner_tol, int max_cycles) {
  TFS_CHECK_SOLVER(s);
  if (!(inner_tol > 0.0 && inner_tol < 1.0) || max_cycles < 1)
    return fail(TFS_EINVAL, "inner_tol in (0, 1), max_cycles >= 1");
  s->inner_tol = inner_tol;
  s->max_outer = max_cycles;
  return TFS_OK;
}

int tfs_set_refinement_vectors(tfs_solver *s, int mode) {
  TFS_CHECK_SOLVER(s);
  if (mode != TFS_VECTORS_FP32 && mode != TFS_VECTORS_FP64)
    return fail(TFS_EINVAL, "mode is TFS_VECTORS_FP32 or TFS_VECTORS_FP64");
  s->vec_mode = mode;
  return TFS_OK;
}

int tfs_set_persistent_gmres(tfs_solver *s, int enable) {
  TFS_CHECK_SOLVER(s);
  if (enable && !s->pg_ok)
    return fail(TFS_ESTATE, "the persistent GMRES kernel cannot run for this system or device");
  s->pg_enabled = enable != 0;
  return TFS_OK;
}

int tfs_inject_barrier_stall(tfs_solver *s, int on) {
  TFS_CHECK_SOLVER(s);
  s->pg_stall = on != 0;
  return TFS_OK;
}

int tfs_make_body_reference_matrices(tfs_solver *s) {
  TFS_CHECK_SOLVER(s);
  if (!s->have_refs) return fail(TFS_ESTATE, "set the blob references first");
  // (K^T K)^-1 from the body-frame references (mobility_solver.cpp:2954-2971);
  // rcross(v) a = a x v.
  std::vector<double> refs(3 * (size_t)s->nb);
  TFS_CUDA(cudaMemcpyAsync(refs.data(), s->refs, sizeof(double) * refs.size(),
                           cudaMemcpyDeviceToHost, s->stream),
           "read blob references");
  TFS_CUDA(cudaStreamSynchronize(s->stream), "read blob references");
  double KTK[36] = {0};
  KTK[0] = KTK[7] = KTK[14] = (double)s->nb;
  for (int m = 0; m < s->nb; ++m) {
    const double *v = &refs[3 * (size_t)m];
    const double rc[9] = {0, -v[2], v[1], v[2], 0, -v[0], -v[1], v[0], 0};
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        double rc2 = 0.0;
        for (int k = 0; k < 3; ++k) rc2 += rc[i + 3 * k] * rc[k + 3 * j];
        KTK[i + 6 * (3 + j)] += rc[i + 3 * j];
        KTK[(3 + i) + 6 * j] -= rc[i + 3 * j];
        KTK[(3 + i) + 6 * (3 + j)] -= rc2;
      }
  }
  if (!invert6(KTK)) return fail(TFS_EINVAL, "K^T K is singular (fewer than 3 distinct blobs?)");
  std::memcpy(s->ktkinv_ref, KTK, sizeof KTK);
  int rc;
  if ((rc = upload_mats(s)) != TFS_OK) return rc;
  // six solves with rhs = -e_{n-1-j}; each warm-starts from the last
  double cols[36];
  for (int j = 0; j < 6; ++j) {
    cudaError_t e = launch_unit_rhs(s->rhs, s->n, j, s->stream);
    if (e != cudaSuccess) return cuda_fail(e, "unit rhs");
    int iters = 0;
    s->bootstrap = true;
    rc = linear_solve(s, &iters);
    s->bootstrap = false;
    if (rc != TFS_OK) return rc;
    TFS_CUDA(cudaMemcpyAsync(s->f6_host, s->v_bodies, 8 * 6, cudaMemcpyDeviceToHost, s->stream),
             "read body velocity");
    TFS_CUDA(cudaStreamSynchronize(s->stream), "read body velocity");
    for (int i = 0; i < 6; ++i) cols[i + 6 * (5 - j)] = s->f6_host[i];
  }
  std::memcpy(s->body_mob_ref, cols, sizeof cols);
  return upload_mats(s);
}

int tfs_get_body_reference_matrices(tfs_solver *s, double *body_mobility, double *ktkinv) {
  TFS_CHECK_SOLVER(s);
  if (body_mobility) std::memcpy(body_mobility, s->body_mob_ref, sizeof s->body_mob_ref);
  if (ktkinv) std::memcpy(ktkinv, s->ktkinv_ref, sizeof s->ktkinv_ref);
  return TFS_OK;
}

int tfs_set_body_reference_matrices(tfs_solver *s, const double *body_mobility,
                                    const double *ktkinv) {
  TFS_CHECK_SOLVER(s);
  if (body_mobility) std::memcpy(s->body_mob_ref, body_mobility, sizeof s->body_mob_ref);
  if (ktkinv) std::memcpy(s->ktkinv_ref, ktkinv, sizeof s->ktkinv_ref);
  return upload_mats(s);
}

}  // extern "C"

namespace tfs {

// compute_velocities on the swimmer force already on the device
// (s->swimmer_f, updated in place with the blob repulsion's sums as the
// reference updates swimmer::f): queued on s->stream with one host wait per
// refinement cycle and none at the end.
int compute_velocities_dev(tfs_solver *s, int *gmres_iters) {
  if (s->cfg.nswim != 1) return fail(TFS_EINVAL, "compute_velocities solves one swimmer per solver");
  if (!s->have_refs) return fail(TFS_ESTATE, "set the blob references first");
  int rc;
  // read_positions_and_forces: barrier forces (device f_segs, blob repulsion)
  if ((rc = tfs_apply_interparticle_forces(s)) != TFS_OK) return rc;
  // FP32C: the refinement's first residual product runs beside the segment
  // products, on the second stream (a solver alone; in a batch or server the
  // other swimmers' work already fills the GPU)
  const bool early = s->cfg.precision == TFS_FP32C && s->nb > 0 && s->ff_scratch != nullptr &&
                     s->service == nullptr && s->product_service == nullptr;
  if (early && (rc = early_residual_product(s)) != TFS_OK) return rc;
  // v_segs = Mss f_segs, v_blobs = Mbs f_segs (one work-queue launch when
  // both target sets exist)
  if (s->ns > 0 && s->nb > 0) {
    if ((rc = queue_product(s, QK_SEGSRC)) != TFS_OK) return rc;
  } else {
    if ((rc = tfs_evaluate_segment_segment_mobility(s)) != TFS_OK) return rc;
    if ((rc = tfs_evaluate_blob_segment_mobility(s)) != TFS_OK) return rc;
  }
  const GmresArgs ga = gmres_args(s, s->rhs, s->f_blobs, s->v_bodies, s->gst, s->tol, 0);
  cudaError_t e = launch_rhs(ga, s->f_rep, s->v_blobs, s->swimmer_f, s->rhs, s->stream);
  if (e != cudaSuccess) return cuda_fail(e, "right-hand side");
  if (early) TFS_CUDA(cudaStreamWaitEvent(s->stream, s->aux_join, 0), "second stream join");
  int iters = 0;
  if ((rc = linear_solve(s, &iters, early)) != TFS_OK) return rc;
  // v_segs += Msb f_blobs (the solved blob forces)
  if ((rc = tfs_evaluate_segment_blob_mobility(s)) != TFS_OK) return rc;
  s->last_iters = iters;
  if (gmres_iters) *gmres_iters = iters;
  return TFS_OK;
}

int solver_new_step(tfs_solver *s) {
  if (s->cfg.precision != TFS_FP32C || s->whist == nullptr) return TFS_OK;
  if (s->solved) {
    const int slot = s->whist_head ^ 1;  // the older entry
    double *h = s->whist + (size_t)slot * s->n;
    const int vel = 3 * s->nb;
    TFS_CUDA(cudaMemcpyAsync(h, s->f_blobs, sizeof(double) * vel, cudaMemcpyDeviceToDevice,
                             s->stream),
             "solution history");
    TFS_CUDA(cudaMemcpyAsync(h + vel, s->v_bodies, sizeof(double) * 6, cudaMemcpyDeviceToDevice,
                             s->stream),
             "solution history");
    s->whist_head = slot;
    s->whist_n = std::min(2, s->whist_n + 1);
    s->solved = false;
  }
  s->extrap_next = s->whist_n == 2;
  return TFS_OK;
}

void solver_reset_history(tfs_solver *s) {
  s->whist_n = 0;
  s->solved = false;
  s->extrap_next = false;
}

}  // namespace tfs

extern "C" {

int tfs_compute_velocities(tfs_solver *s, double *swimmer_f, int *gmres_iters) {
  TFS_CHECK_SOLVER(s);
  if (swimmer_f == nullptr) return fail(TFS_EINVAL, "null swimmer force");
  std::memcpy(s->f6_host, swimmer_f, 8 * 6);
  TFS_CUDA(cudaMemcpyAsync(s->swimmer_f, s->f6_host, 8 * 6, cudaMemcpyHostToDevice, s->stream),
           "copy swimmer force");
  int rc = compute_velocities_dev(s, gmres_iters);
  if (rc != TFS_OK) return rc;
  TFS_CUDA(cudaMemcpyAsync(s->f6_host, s->swimmer_f, 8 * 6, cudaMemcpyDeviceToHost, s->stream),
           "read swimmer force");
  TFS_CUDA(cudaStreamSynchronize(s->stream), "compute_velocities");
  std::memcpy(swimmer_f, s->f6_host, 8 * 6);
  return TFS_OK;
}

int tfs_solve_linear_system(tfs_solver *s, const double *rhs_host, int *gmres_iters) {
  TFS_CHECK_SOLVER(s);
  if (rhs_host == nullptr) return fail(TFS_EINVAL, "null right-hand side");
  if (!s->have_refs) return fail(TFS_ESTATE, "set the blob references first");
  TFS_CUDA(cudaMemcpyAsync(s->rhs, rhs_host, sizeof(double) * s->n, cudaMemcpyHostToDevice,
                           s->stream),
           "copy right-hand side");
  int iters = 0, rc;
  if ((rc = linear_solve(s, &iters)) != TFS_OK) return rc;
  s->last_iters = iters;
  if (gmres_iters) *gmres_iters = iters;
  return tfs_wait_for_device(s);
}

int tfs_get_body_velocities(tfs_solver *s, double *v_bodies) {
  TFS_CHECK_SOLVER(s);
  if (v_bodies == nullptr) return fail(TFS_EINVAL, "null output");
  TFS_CUDA(cudaMemcpyAsync(s->f6_host, s->v_bodies, 8 * 6, cudaMemcpyDeviceToHost, s->stream),
           "read body velocity");
  TFS_CUDA(cudaStreamSynchronize(s->stream), "read body velocity");
  std::memcpy(v_bodies, s->f6_host, 8 * 6);
  return TFS_OK;
}

int tfs_set_body_velocities(tfs_solver *s, const double *v_bodies) {
  TFS_CHECK_SOLVER(s);
  if (v_bodies == nullptr) return fail(TFS_EINVAL, "null input");
  std::memcpy(s->f6_host, v_bodies, 8 * 6);
  TFS_CUDA(cudaMemcpyAsync(s->v_bodies, s->f6_host, 8 * 6, cudaMemcpyHostToDevice, s->stream),
           "write body velocity");
  TFS_CUDA(cudaStreamSynchronize(s->stream), "write body velocity");
  return TFS_OK;
}

int tfs_copy_blob_forces_to_host(tfs_solver *s, double *f_blobs_host) {
  TFS_CHECK_SOLVER(s);
  if (f_blobs_host == nullptr && s->nb > 0) return fail(TFS_EINVAL, "null host pointer");
  if (s->nb > 0)
    TFS_CUDA(cudaMemcpyAsync(f_blobs_host, s->f_blobs, sizeof(double) * 3 * s->nb,
                             cudaMemcpyDeviceToHost, s->stream),
             "copy blob forces to host");
  return TFS_OK;
}

int tfs_pg_trace(unsigned long long *stamps, int capacity, int *steps) {
  const int rc = pg_trace_read(stamps, capacity, steps);
  if (rc == -3) return fail(TFS_ESTATE, "the library was built without TFS_PG_TRACE");
  if (rc == -1) return fail(TFS_EINVAL, "capacity below 2 x steps x 8 stamps");
  if (rc != 0) return fail(TFS_ECUDA, "reading the trace failed");
  return TFS_OK;
}

int tfs_copy_blob_forces_to_host_f32(tfs_solver *s, float *f_blobs_host) {
  TFS_CHECK_SOLVER(s);
  return d2h_f32(s, f_blobs_host, s->f_blobs, 3 * (size_t)s->nb, "copy blob forces to host");
}

int tfs_refinement_retries(tfs_solver *s, long long *retries) {
  TFS_CHECK_SOLVER(s);
  if (retries == nullptr) return fail(TFS_EINVAL, "null argument");
  *retries = s->vec64_retries;
  return TFS_OK;
}

int tfs_solve_info(tfs_solver *s, int *iters, int *cycles, double *rel_residual) {
  TFS_CHECK_SOLVER(s);
  if (iters) *iters = s->last_iters;
  if (cycles) *cycles = s->last_outer;
  if (rel_residual) *rel_residual = s->last_rel;
  return TFS_OK;
}

}  // extern "C"
