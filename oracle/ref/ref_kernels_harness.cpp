// ref_kernels_harness.cpp -- C entry points that run the reference's own RPY
// and barrier kernels (src/cilia/cuda_functions.cu, compiled unchanged under
// cuda_emu.hpp) on the CPU.
//
// TEST INFRASTRUCTURE ONLY. Built by oracle/Makefile into oracle/_ref/ when
// the reference tree is present; used to pin the C restatement in
// oracle/tfs_oracle.c and to generate the committed golden vectors.
//
// Launch shapes follow rpy_mobility_solver.cu:258-328 (single device:
// start = 0, count = all) and :207-245 for barrier_forces.
#include <algorithm>

#include "cuda_emu.hpp"
#include "cuda_functions.hpp"

extern int NSWIM_d, NSEG_d, NFIL_d, NBLOB_d, NTOTAL_d, END_FORCE_MAGNITUDE_d;

static int blocks_for(int n) { return (n + THREADS_PER_BLOCK - 1) / THREADS_PER_BLOCK; }

extern "C" {

// cuda_functions.cu:1533-1544 (sync_var), run as a 1-thread kernel.
void ref_sync_var(int nswim, int nseg, int nfil, int nblob, int end_force_magnitude,
                  double seg_sep) {
  emu_launch(1, 1, [&] { sync_var(nswim, nseg, nfil, nblob, end_force_magnitude, seg_sep); });
}

double ref_rseg(void) { return RSEG; }
double ref_rblob(void) { return RBLOB; }
double ref_mu(void) { return MU; }

void ref_mss(double *v_segs, const double *f_segs, const double *x_segs, int num_segs) {
  emu_launch(blocks_for(num_segs), THREADS_PER_BLOCK,
             [&] { Mss_mult(v_segs, f_segs, x_segs, 0, num_segs); });
}

void ref_msb(double *v_segs, const double *f_blobs, const double *x_segs, const double *x_blobs,
             int num_segs) {
  emu_launch(blocks_for(num_segs), THREADS_PER_BLOCK,
             [&] { Msb_mult(v_segs, f_blobs, x_segs, x_blobs, 0, num_segs); });
}

void ref_mbb(double *v_blobs, const double *f_blobs, const double *x_blobs, int num_blobs) {
  emu_launch(blocks_for(num_blobs), THREADS_PER_BLOCK,
             [&] { Mbb_mult(v_blobs, f_blobs, x_blobs, 0, num_blobs); });
}

void ref_mbs(double *v_blobs, const double *f_segs, const double *x_blobs, const double *x_segs,
             int num_blobs) {
  emu_launch(blocks_for(num_blobs), THREADS_PER_BLOCK,
             [&] { Mbs_mult(v_blobs, f_segs, x_blobs, x_segs, 0, num_blobs); });
}

void ref_barrier_forces(double *f_segs, double *f_blobs_repulsion, const double *x_segs,
                        const double *x_blobs, int num_segs, int num_blobs) {
  emu_launch(blocks_for(std::max(num_segs, num_blobs)), THREADS_PER_BLOCK, [&] {
    barrier_forces(f_segs, f_blobs_repulsion, x_segs, x_blobs, 0, num_segs, 0, num_blobs);
  });
}

}  // extern "C"
