// tfs_solver.h -- the solver object behind the C ABI (internal to
// libtfs_gb300.so): device buffers of one swimmer system, launch tuning,
// and the state of the free-body solve.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/tfs_gb300.h"
#include "gmres.h"
#include "tfs_kernels.h"

namespace tfs {
struct GmresService;
struct ProductService;
struct PresState;
int fail(int code, const char *fmt, ...);
int cuda_fail(cudaError_t e, const char *what);
long long launch_count();
}  // namespace tfs

struct tfs_solver {
  tfs_config cfg;
  int ns = 0, nb = 0;
  int device = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  double *x_segs = nullptr, *f_segs = nullptr, *v_segs = nullptr;
  double *x_blobs = nullptr, *f_blobs = nullptr, *v_blobs = nullptr, *f_rep = nullptr;
  double *origin = nullptr;  // [4]: mean position and extent, then partials
  unsigned *origin_cnt = nullptr;  // [2] last-CTA counters of the origin passes
  void *rec_segs = nullptr, *rec_blobs = nullptr;
  void *rec_segs_x2 = nullptr, *rec_blobs_x2 = nullptr;  // FP32x2 records
  void *rec_ff = nullptr;  // float-float blob records (the refinement residual)
  void *bar_grid = nullptr;     // barrier forces: hashed grid of the sources
  double *wc_z = nullptr, *wc_f = nullptr;  // weakly coupled filaments: means, total forces
  double *scratch = nullptr;
  size_t scratch_elems = 0;
  float *stage32 = nullptr;  // float host-array copies: staging of the largest array
  bool origin_dirty = true;

  // --- free-body solve (solve.cu) ---
  int n = 0;                 // 3 nb + 6
  int max_iter = 350;        // MAX_LINEAR_SYSTEM_ITER, capped at n
  double tol = 1e-4;         // LINEAR_SYSTEM_TOL
  double inner_tol = 1e-4;   // FP32C: inner GMRES tolerance of each refinement cycle
  bool bootstrap = false;    // the solves of make_body_reference_matrices are running
  // FP32C: the final solutions of the last two time steps (2 x n, ring of two
  // with the newest at whist_head), for the first solve of the next step to
  // start from their linear extrapolation
  double *whist = nullptr;
  int whist_n = 0, whist_head = 0;
  bool solved = false, extrap_next = false;
  // FP32C: the first refinement residual's M_bb product runs on a second
  // stream beside the segment products (its own partial sums buffer)
  cudaStream_t aux_stream = nullptr;
  cudaEvent_t aux_fork = nullptr, aux_join = nullptr;
  double *ff_scratch = nullptr;
  size_t ff_scratch_elems = 0;
  long long vec64_retries = 0;  // FP32C refinements rerun with FP64 Arnoldi vectors
  // FP32C: Arnoldi vectors of the cooperative inner solves (TFS_VECTORS_*)
  int vec_mode = 0;
  int max_outer = 12;        // FP32C: refinement cycles
  int chunk = 8;             // Arnoldi steps launched between polls of the done flag
  bool have_refs = false;
  double *refs = nullptr, *diff = nullptr;   // 3 nb: body-frame references, R ref
  tfs::BodyPose pose{};
  double body_mob_ref[36], ktkinv_ref[36];   // column-major, body frame
  double mats_host[72];
  double *mats = nullptr;    // device copy of the rotated matrices
  double *Q = nullptr, *H = nullptr, *beta = nullptr, *cs = nullptr, *sn = nullptr,
         *y = nullptr, *z = nullptr, *tmp = nullptr, *soln = nullptr, *rhs = nullptr,
         *vtmp = nullptr;
  double *v_bodies = nullptr;  // 6: warm start / solution
  double *swimmer_f = nullptr; // 6
  double *xr = nullptr, *r = nullptr, *dx = nullptr;  // FP32C refinement (n each)
  tfs::GmresScalars *gst = nullptr;   // device scalars: [0] inner, [1] outer
  int gG = 1, g_blobs_per_cta = 1;    // GMRES kernel grid
  double *gpart = nullptr, *gpart6 = nullptr, *gh1 = nullptr, *gh2 = nullptr;
  unsigned *gcounters = nullptr;
  // persistent inner GMRES (FP32C); pg_ok = 0 when it cannot run here
  int pg_ok = 0, pg_enabled = 1;
  int pg_stall = 0;  // tfs_inject_barrier_stall: barriers wait for one CTA more than run
  tfs::PgShape pg{};
  float *pg_x32 = nullptr, *pg_rec = nullptr;
  float2 *pg_mpart = nullptr;
  double *pg_p6 = nullptr, *pg_ps = nullptr, *pg_pd1 = nullptr,
         *pg_pd2 = nullptr, *pg_aux = nullptr;
  unsigned *pg_bar = nullptr;
  tfs::PgArgs *pg_gp = nullptr;  // device copy of this solve's arguments
  int2 *pg_cmap = nullptr;       // CTA c -> (0, c)
  // inner solves shared with other swimmers' (one cooperative launch for all
  // that are waiting): the service, this swimmer's fixed shape within such a
  // launch, and events marking its inputs ready and its solve ended
  tfs::GmresService *service = nullptr;
  tfs::PgShape pg_group{};
  cudaEvent_t ready_ev = nullptr, done_ev = nullptr;
  tfs::GmresScalars *gst_host = nullptr;  // pinned copies
  double *f6_host = nullptr;              // pinned 6
  int last_iters = 0, last_outer = 0;
  double last_rel = 0.0;
  // work-queue products (rpy_queue.cuh): the job list of each launch kind,
  // built once at creation (host copy and device copy), the launch counters
  // and per-target-block arrival counters, and the tuned variant per
  // (precision, kind)
  tfs::QueueJob qjobs[tfs::kNumQueueKinds][2];
  int qjobs_n[tfs::kNumQueueKinds] = {};
  tfs::QueueJob *qjobs_dev = nullptr;  // [kNumQueueKinds][2]
  unsigned *qcount = nullptr;          // [2] launch counters, then arrival counters
  int qtune[2][tfs::kNumQueueKinds] = {};
  // products shared with other swimmers' (one work-queue launch for all that
  // are waiting): the service, and events marking this swimmer's records
  // ready and its product done
  tfs::ProductService *product_service = nullptr;
  cudaEvent_t pready_ev = nullptr, pdone_ev = nullptr;
  // launch tuning per precision and (target, source-set) combination
  tfs::TileTuning tune[2][tfs::kNumCombos];
  std::string tuning_report = "{}";
  // kernel-sequence GMRES: one chunk of Arnoldi steps captured as a CUDA
  // graph per argument set (solve.cu), replayed once per chunk
  struct ChunkGraph {
    tfs::GmresArgs args;
    tfs::TileTuning tune;
    int chunk;
    cudaGraphExec_t exec;
    long long kernels;
  };
  std::vector<ChunkGraph> chunk_graphs;
  bool graphs_enabled = true;
  // the prescribed-cilia solve (prescribed.cu), made by tfs_prescribed_setup
  tfs::PresState *pres = nullptr;
  // dominant-kernel timing (tfs_solver_enable_kernel_timing)
  bool timing = false;
  std::vector<cudaEvent_t> events;  // pairs, in launch order
  size_t events_used = 0;
};


#define TFS_CHECK_SOLVER(s)                                              \
  do {                                                                   \
    if ((s) == nullptr) return tfs::fail(TFS_EINVAL, "null solver handle"); \
  } while (0)

#define TFS_CUDA(call, what)                                 \
  do {                                                       \
    cudaError_t e_ = (call);                                 \
    if (e_ != cudaSuccess) return tfs::cuda_fail(e_, what);  \
  } while (0)

namespace tfs {
// helpers shared by tfs_api.cu and solve.cu
int ensure_origin(tfs_solver *s);
int pack(tfs_solver *s, int segs);
TileArgs base_args(tfs_solver *s);
int product(tfs_solver *s, bool tgt_segs, bool src_segs, bool src_blobs, int mode);
// One work-queue launch of the given kind (QueueKind) on the solver's stream.
int queue_product(tfs_solver *s, int kind);
// Float host arrays: copy n floats to (from) a float64 device array,
// converting on the device through the solver's float staging buffer.
int h2d_f32(tfs_solver *s, double *dst, const float *src, size_t n, const char *what);
int d2h_f32(tfs_solver *s, float *dst, const double *src, size_t n, const char *what);
int alloc_dev(void **p, size_t bytes);
int solve_alloc(tfs_solver *s);
void solve_free(tfs_solver *s);
// Inner solves of FP32C swimmers batched into shared cooperative launches.
GmresService *service_create();
void service_destroy(GmresService *sv);
int service_attach(GmresService *sv, tfs_solver *s);  // TFS_ESTATE if the kernel cannot serve s
void service_stats(GmresService *sv, long long *launches, long long *solves);
// Pair products of many swimmers batched into shared work-queue launches
// (product_service.cu).
ProductService *product_service_create();
void product_service_destroy(ProductService *sv);
int product_service_attach(ProductService *sv, tfs_solver *s);
int product_service_run(ProductService *sv, tfs_solver *s, int kind, int fp32, int src);
void product_service_stats(ProductService *sv, long long *launches, long long *products);
// compute_velocities on the swimmer force already in s->swimmer_f, queued on
// s->stream without a host wait at the end (solve.cu).
int compute_velocities_dev(tfs_solver *s, int *gmres_iters);
// A new time step begins (the stepper's initial guess): FP32C solvers keep
// the last step's final solution for the extrapolated warm start of the next
// step's first solve (solve.cu).
int solver_new_step(tfs_solver *s);
// Forget the solutions of earlier steps (the stepper restarted or reloaded).
void solver_reset_history(tfs_solver *s);
// Free the prescribed-cilia solve's buffers (prescribed.cu).
void pres_free(tfs_solver *s);
// A block hook in the reference's PRESCRIBED_CILIA form (after
// tfs_prescribed_setup): forces only, 3x3 pairs, zero rotational segment
// velocities, blob <- seg adding (prescribed.cu).
int pres_hook(tfs_solver *s, bool tgt_segs, bool src_segs);
}  // namespace tfs
