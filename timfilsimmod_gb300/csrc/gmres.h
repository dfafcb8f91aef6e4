// gmres.h -- device structures and launchers of the free-body solve
// (gmres.cu); internal to libtfs_gb300.so.
#pragma once

#include <cuda_runtime.h>

namespace tfs {

// Scalars of one solve, in device memory.
struct GmresScalars {
  double norm_rhs;
  double rel;    // |beta_k| / ||rhs|| of the last step
  double qnorm;  // ||w|| of the last Arnoldi step
  int iter;      // Arnoldi step being built (k)
  int done;      // 1: finished; later kernels of the sequence return at once
  int iters;     // iterations taken (0: warm start or zero right-hand side)
  int status;    // 0 ok, 1 non-finite residual
  int flag;      // warm-start test: 1 accepted, 2 discarded, 3 zero right-hand side
};

// Body pose: position and rotation matrix (column-major).
struct BodyPose {
  double x[3];
  double R[9];
};

struct GmresArgs {
  int n, nb, max_iter;
  double tol;
  double mu, a_blob;
  int fp32;                 // which record format the M_bb product reads
  const double *x_blobs;    // 3 nb
  const double *diff;       // 3 nb: R ref_m
  const double *origin;     // FP32 centring origin
  void *rec64, *rec32, *rec32x2;  // blob source records written for M_bb
  const double *mats;       // 72: rotated body mobility (36), rotated KTKinv (36)
  const double *rhs;        // n
  double *soln, *Q, *H, *beta, *cs, *sn, *y, *z, *tmp;
  double *v;                // 3 nb: M_bb output
  double *f_blobs, *v_bodies;  // warm start in, solution out
  GmresScalars *st;
  // multi-CTA work split: G CTAs of blobs_per_cta blobs (the last CTA also
  // owns the six body rows); per-CTA partial sums and last-CTA counters
  int G, blobs_per_cta;
  double *part;             // G * part_stride
  int part_stride;          // max_iter + 1
  double *part6;            // 6 * G
  unsigned *counters;       // 8, zero between kernels
  double *h1, *h2;          // max_iter + 1 each: the two Gram-Schmidt passes
};

// Persistent (cooperative) inner GMRES with an FP32 M_bb product
// (gmres_persistent.cu): launch shape and arguments.
constexpr int kMaxPgBlobsPerCta = 128;                 // rows per CTA <= 384
constexpr int kPgServiceBlobsPerCta = 64;              // a shared launch's CTAs per swimmer
constexpr int kMaxPgCtas = 256;                        // one CTA per SM
constexpr unsigned long long kPgTimeoutNs = 2000000000ull;  // one barrier wait
struct PgShape {
  int P;                  // CTAs (all resident: cooperative launch)
  int G, blobs_per_cta;   // CTAs owning blob slices, blobs per slice
  int TB, tbs;            // M_bb target blocks and their size
  int S, chunk;           // M_bb source splits and their size
  int Kr, Kr64;           // Krylov columns resident in shared memory (FP32, FP64 vectors)
  size_t dyn_smem;        // dynamic shared memory per CTA (bytes, FP32 vectors)
  size_t dyn_smem64;      // the same with FP64 vectors
};
struct PgArgs {
  GmresArgs g;            // vectors, body data, tolerance; g.G / g.blobs_per_cta = slices
  float *x32;             // 3 nb: blob positions minus the origin, FP32
  float *rec;             // 8 nb: FP32 blob records of the current z
  float2 *mpart;          // S * 3 nb: split partial products of M_bb, (hi, lo)
  // per-CTA partials, FP64-sized buffers holding values of the vector type:
  double *p6, *ps;        // partial 6-vectors and sums of squares
  double *pd1, *pd2;      // Gram-Schmidt partial dots ((max_iter + 2) * G each)
  double *aux;            // control words (3), then h1, h2, y (vector type) published by CTAs
  unsigned *bar;          // 4: barrier count, generation, abort
  int P, TB, tbs, S, chunk, Kr;  // P: the CTAs of this solve
  int rank;               // this CTA's index among them (set on the device)
  int zero_start;         // 1: the warm start is zero (A x0 = 0, r0 = rhs; its M_bb skipped)
  int vec64;              // 1: FP64 Arnoldi vectors (else FP32); Kr and dyn_smem match
  unsigned bar_extra;     // arrivals each barrier waits for beyond the P CTAs: 0, or 1
                          // under tfs_inject_barrier_stall (every wait then runs out)
  size_t dyn_smem;
  float a;                // blob radius
  float pc_asum2, pc_s, pc_s3;  // FP32 pair constants: (2a)^2, 2a^2/3, -2a^2
  double scale;           // 1 / (8 pi mu)
  double minv;            // 6 pi mu a (the preconditioner's blob block)
};
// Launch shape for nb blobs on `sms` SMs; 0 when the kernel cannot be used
// (no occupancy, or more than kMaxPgBlobsPerCta blobs per CTA).
int pg_grid(int nb, int sms, int max_iter, PgShape *shape);
// Buffer sizes (elements) of one shape.
inline size_t pg_p6_elems(const PgShape &s) { return 6 * 6 * (size_t)s.G; }
inline size_t pg_ps_elems(const PgShape &s) { return 3 * (size_t)s.G; }
inline size_t pg_pd_elems(const PgShape &s) { return 352 * (size_t)s.G; }
constexpr size_t kPgAuxElems = 3 + 3 * 352;
// One cooperative launch of `ctas` CTAs running the solves in gp[] (device
// array): CTA c works for solve cmap[c].x as its CTA cmap[c].y. Every solve's
// barrier words must be zero, and every solve's vec64 equal to vec64.
cudaError_t launch_gmres_persistent(const PgArgs *gp, const int2 *cmap, int ctas, size_t dyn_smem,
                                    int vec64, cudaStream_t st);

// The phase trace of the persistent GMRES (builds with -DTFS_PG_TRACE):
// [2 CTAs][steps][8 phases] globaltimer stamps into out (capacity elements);
// 0, or -1 (capacity too small), -2 (copy failed), -3 (not a trace build).
int pg_trace_read(unsigned long long *out, int capacity, int *steps);

// CTAs and blobs per CTA of the GMRES kernels for nb blobs on `sms` SMs.
int gmres_grid(int nb, int sms, int *blobs_per_cta);
cudaError_t launch_gmres_finish(const GmresArgs &a, cudaStream_t st);

cudaError_t launch_gmres_start(const GmresArgs &a, cudaStream_t st);
cudaError_t launch_gmres_residual(const GmresArgs &a, cudaStream_t st);
cudaError_t launch_gmres_precond(const GmresArgs &a, cudaStream_t st);
cudaError_t launch_gmres_arnoldi(const GmresArgs &a, cudaStream_t st);
cudaError_t launch_refine_residual(const GmresArgs &a, const double *x, double *r, double *dx,
                                   int outer, cudaStream_t st);
cudaError_t launch_axpy(double *x, const double *d, int n, cudaStream_t st);
cudaError_t launch_blob_positions(double *x_blobs, double *diff, const double *refs, int nb,
                                  const BodyPose &pose, cudaStream_t st);
cudaError_t launch_rhs(const GmresArgs &a, const double *frep, const double *v_blobs,
                       double *swimmer_f, double *rhs, cudaStream_t st);
cudaError_t launch_unit_rhs(double *rhs, int n, int j, cudaStream_t st);

}  // namespace tfs
