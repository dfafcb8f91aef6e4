// gmres.h -- device structures and launchers of the free-body solve
// (gmres.cu); internal to libtfs_gb300.so.
#pragma once

#include <cuda_runtime.h>

namespace tfs {

// Scalars of one solve, in device memory.
struct GmresScalars {
  double norm_rhs;
  double rel;    // |beta_k| / ||rhs|| of the last step
  int iter;      // Arnoldi step being built (k)
  int done;      // 1: finished; later kernels of the sequence return at once
  int iters;     // iterations taken (0: warm start or zero right-hand side)
  int status;    // 0 ok, 1 non-finite residual
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
  int w_in_smem;            // Arnoldi keeps the new basis vector in shared memory
};

bool gmres_w_fits_smem(int n);

cudaError_t launch_gmres_start(const GmresArgs &a, cudaStream_t st);
cudaError_t launch_gmres_residual(const GmresArgs &a, cudaStream_t st);
cudaError_t launch_gmres_precond(const GmresArgs &a, cudaStream_t st);
cudaError_t launch_gmres_arnoldi(const GmresArgs &a, cudaStream_t st);
cudaError_t launch_refine_residual(const GmresArgs &a, const double *x, double *r, double *dx,
                                   int outer, cudaStream_t st);
cudaError_t launch_axpy(double *x, const double *d, int n, cudaStream_t st);
cudaError_t launch_blob_positions(double *x_blobs, double *diff, const double *refs, int nb,
                                  const BodyPose &pose, cudaStream_t st);
cudaError_t launch_rhs(const double *frep, const double *diff, const double *v_blobs, int nb,
                       double *swimmer_f, double *rhs, cudaStream_t st);
cudaError_t launch_unit_rhs(double *rhs, int n, int j, cudaStream_t st);
cudaError_t launch_store_body_column(double *body_mob, const double *v_bodies, int j,
                                     cudaStream_t st);

}  // namespace tfs
