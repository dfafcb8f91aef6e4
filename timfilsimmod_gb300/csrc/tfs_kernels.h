// tfs_kernels.h -- host-side declarations of the kernel launchers
// (internal to libtfs_gb300.so).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

namespace tfs {

enum OutMode { OUT_ASSIGN = 0, OUT_ACCUMULATE = 1, OUT_PARTIAL = 2 };

// Upper bound on source splits of one product (sizes the scratch buffer).
constexpr int kMaxSplits = 64;
// Devices whose per-kernel occupancy is cached.
constexpr int kMaxDevices = 64;

struct TileArgs {
  const double *x_tgt;  // target positions, AoS float64 [3*n_tgt]
  int n_tgt;
  double a_tgt;         // target radius
  const void *src_a;    // packed source records, set A
  int n_a;
  double a_a;
  const void *src_b;    // packed source records, set B (or null)
  int n_b;
  double a_b;
  const void *src_a2;   // FP32x2 records (duplicated pairs) of set A, set B
  const void *src_b2;
  const double *origin; // device [4]: FP32 centring origin (+ extent)
  int fp32;             // 1: FP32 compensated, 0: FP64
  double scale;         // 1 / (8 pi mu)
  double *out;          // velocities, AoS float64 [VD*n_tgt]
  const int *skip;      // device flag: the launch does nothing when *skip != 0 (or null)
  int splits;           // 0: automatic
  int chunk;            // set by the launcher
  int mode;             // set by the launcher
};

struct BarrierArgs {
  double *f_segs;             // += on segment targets
  double *f_blobs_repulsion;  // = on blob targets
  const double *x_segs;
  const double *x_blobs;
  const double *origin;       // device [4] origin + extent
  int num_segs, num_blobs, nseg;
  double a_seg, a_blob;
  int end_force_magnitude;
  double repulsive_force_factor;
  int free_body;
  void *grid;                 // barrier_grid_bytes(): the hashed grid of the sources
};

// The barrier forces' hashed grid (rpy_kernels.cu): T bucket counters, the
// overflow word, T buckets of source entries {x, y, z, index}, 3 sums per
// target.
struct BarGrid {
  unsigned *count, *overflow;
  float4 *entry;
  double *sum;
  unsigned T;
};

// Launch variants of the tile kernel and their dispatch tables
// (rpy_tile_f32.cu, rpy_tile_f64.cu).
struct TileVariant {
  int block, tpt, ts;  // threads per CTA, targets per thread, sources per tile
  int x2;              // 1: packed FP32x2 kernel (rpy_tile_x2.cuh)
  int min_blocks;      // __launch_bounds__ minimum resident CTAs (register cap), 0 = none
};
// (target kind, source sets): 0 = seg<-seg, 1 = seg<-blob, 2 = blob<-blob,
// 3 = blob<-seg, 4 = seg<-(seg,blob), 5 = blob<-(seg,blob)
enum TileCombo { C_SS = 0, C_SB = 1, C_BB = 2, C_BS = 3, C_SX = 4, C_BX = 5 };
constexpr int kNumCombos = 6;
constexpr int kNumVariantsF32Scalar = 8;
constexpr int kNumVariantsF32X2 = 3;
constexpr int kNumVariantsF32 = kNumVariantsF32Scalar + kNumVariantsF32X2;
constexpr int kNumVariantsF64 = 5;
// Launch (grid.x > 0) or, with grid.x == 0, report resident CTAs per SM.
typedef cudaError_t (*TileFn)(const TileArgs &, dim3, cudaStream_t, int *resident);
extern const TileVariant g_variants_f32[kNumVariantsF32];
extern const TileVariant g_variants_f64[kNumVariantsF64];
extern const TileFn g_tile_f32[kNumVariantsF32Scalar][kNumCombos];
extern const TileFn g_tile_f32x2[kNumVariantsF32X2][kNumCombos];
extern const TileFn g_tile_f64[kNumVariantsF64][kNumCombos];

// ---------------------------------------------------------------------------
// Work-queue products (rpy_queue.cuh): one persistent launch over any number
// of jobs, each a target set against one or two packed source sets.
// ---------------------------------------------------------------------------
struct QueueJob {
  const void *tgt_rec;     // packed records of the targets (their positions are read)
  const void *src_a;       // packed source records, set A
  const void *src_b;       // packed source records, set B (or null)
  double *out;             // velocities, AoS float64 [vd n_tgt]
  void *partial;           // [n_chunks][n_tgt][vd] chunk sums, float2 (hi, lo) for FP32 and
                           // double for FP64 (8 B either way; unused when n_chunks == 1)
  unsigned *block_done;    // one arrival counter per target block (zero between launches)
  const int *skip;         // device flag: the job does nothing when *skip != 0 (or null)
  double a_tgt, a_a, a_b;  // radii
  double scale;            // 1 / (8 pi mu)
  // pair constants of (target, set A) and (target, set B), in both precisions:
  // {a_tgt, a_src, (a_tgt + a_src)^2, (a_tgt^2 + a_src^2)/3, -(a_tgt^2 + a_src^2)}
  double pc64[2][5];
  float pc32[2][5];
  int n_tgt, n_a, n_b;
  int vd;                  // 6 (segment targets) or 3 (blob targets)
  int mode;                // OUT_ASSIGN or OUT_ACCUMULATE
  int chunk, n_chunks;     // sources per unit (a multiple of kQueueQuantum), chunks
  int pad;
};
struct QueueArgs {
  const QueueJob *jobs;    // device array, costliest pairs first
  int n_jobs;
  unsigned *counters;      // [2]: units handed out, CTAs finished (zero between launches)
};
// Source sets of a queue launch (every job of one launch has the same).
enum QueueSources { Q_SEG = 0, Q_BLOB = 1, Q_SEG_BLOB = 2 };
constexpr int kNumQueueSources = 3;
struct QueueVariant {
  int block, tpt, ts, min_blocks;
};
constexpr int kNumQueueVariantsF32 = 5;
constexpr int kNumQueueVariantsF64 = 3;
typedef cudaError_t (*QueueFn)(const QueueArgs &, int ctas, cudaStream_t, int *resident);
extern const QueueVariant g_qvariants_f32[kNumQueueVariantsF32];
extern const QueueVariant g_qvariants_f64[kNumQueueVariantsF64];
extern const QueueFn g_queue_f32[kNumQueueVariantsF32][kNumQueueSources];
extern const QueueFn g_queue_f64[kNumQueueVariantsF64][kNumQueueSources];
// Chunks are whole multiples of this many sources (every variant's tile
// size divides it).
constexpr int kQueueQuantum = 256;
// Largest number of jobs one launch may carry (the kernel keeps their unit
// offsets in shared memory).
constexpr int kQueueMaxJobs = 256;
// Source chunking of a job with n_src sources in a system of n_particles
// target particles: about 8192 units of 128 targets over the system, at
// most kMaxSplits chunks. A function of the sizes alone, so a product is
// split the same way whatever launch carries it.
void queue_chunking(int n_src, int n_particles, int *chunk, int *n_chunks);
// Launch the queue kernel of (precision, variant, sources) over the jobs
// (device array `jobs`; `jobs_host` is the same array on the host, used to
// size the grid). counters: [2] zeroed unsigned. ev (optional): events
// recorded around the launch.
cudaError_t launch_queue(int fp32, int variant, int sources, const QueueJob *jobs,
                         const QueueJob *jobs_host, int n_jobs, unsigned *counters,
                         cudaStream_t st, cudaEvent_t *ev = nullptr);
// Work units of the jobs for a variant's target block (BLOCK * TPT targets).
long long queue_units(const QueueJob *jobs_host, int n_jobs, int block_targets);
// The products a solver launches through the queue: M_ss, M_bs, both at once
// (segment sources, two jobs), M_sb (accumulating), M_bb, and the grand
// mobility (all sources, both target kinds: two jobs).
enum QueueKind { QK_MSS = 0, QK_MBS = 1, QK_SEGSRC = 2, QK_MSB = 3, QK_MBB = 4, QK_GRAND = 5 };
constexpr int kNumQueueKinds = 6;

// Tuning of one launch: variant and the number of full waves (resident CTAs
// on every SM) the source splitting aims for.
struct TileTuning {
  int variant;
  int waves;
};
int combo_of(int vd, int fda, int fdb);

int num_sms();
void count_launch();
void count_launch_n(long long n);  // n may be negative (launches recorded into a graph)
size_t record_bytes(int fp32, int fd);

cudaError_t launch_origin(const double *xa, int na, const double *xb, int nb, double *out,
                          unsigned *counter, cudaStream_t st);
size_t origin_elems();  // doubles of the origin buffer: [4] result + partials
cudaError_t launch_pack(int fp32, int fd, void *rec, const double *x, const double *f, int n,
                        const double *origin, cudaStream_t st);
// FP32x2 records (positions negated, every value duplicated), 80 B per
// segment and 48 B per blob.
cudaError_t launch_pack_x2(int fd, void *rec, const double *x, const double *f, int n,
                           const double *origin, cudaStream_t st);
// vd: 6 (segment targets) or 3 (blob targets); fda/fdb: 6 (segment sources),
// 3 (blob sources), fdb = 0 for a single source set. mode: OUT_ASSIGN or
// OUT_ACCUMULATE. scratch must hold kMaxSplits * n_tgt * vd doubles for
// split launches (the launcher falls back to one split when it is smaller).
// ev (optional): a pair of events recorded around the tile kernel itself
// (not the pack or reduce kernels), for the dominant-kernel timing hook.
cudaError_t launch_tile(const TileArgs &a, int vd, int fda, int fdb, TileTuning tune,
                        double *scratch, size_t scratch_elems, int mode, cudaStream_t st,
                        cudaEvent_t *ev = nullptr);
cudaError_t launch_barrier(const BarrierArgs &a, cudaStream_t st);
// Bytes of BarrierArgs::grid for these sizes.
size_t barrier_grid_bytes(int num_segs, int num_blobs);
// The weakly coupled filaments' segment product (weak.cu): filament means
// Z and total forces Ft (3 nfil each, written), then v_segs (6 Ns).
cudaError_t launch_msf(const double *x_segs, const double *f_segs, int nfil, int nseg,
                       double a_seg, double mu, double *Z, double *Ft, double *v_segs,
                       cudaStream_t st);
// out = M_bb f_blobs in float-float arithmetic (rpy_ff.cu): packs the source
// records into rec (ff_record_bytes() per blob), then the pair kernel and,
// with source splits, the split reduction (scratch as for launch_tile). ev
// (optional): events around the pair kernel.
size_t ff_record_bytes();
cudaError_t launch_bb_ff(const double *x_blobs, const double *f_blobs, int nb,
                         const double *origin, double a_blob, double scale, void *rec, double *out,
                         double *scratch, size_t scratch_elems, cudaStream_t st,
                         cudaEvent_t *ev = nullptr);
// out[i] (= or += with accumulate) sum over splits s, in order, of
// partial[s * n_elems + i].
cudaError_t launch_reduce_partials(double *out, const double *partial, int n_elems, int splits,
                                   int accumulate, cudaStream_t st);

}  // namespace tfs
