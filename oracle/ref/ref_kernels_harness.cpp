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
#include <vector>

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

// The weakly coupled filaments' segment product, as
// weakly_coupled_filaments_rpy_mobility_solver.cu:50-107 runs it: filament
// means (reset_mean_fil_posns, write_mean_fil_posns), total forces
// (reset_mean_fil_force_and_moment, find_total_fil_force_and_first_moment),
// then Msf_mult over every segment. The first-moment array is the
// reference's one-element placeholder (its moment code is commented out).
void ref_msf(double *v_segs, const double *f_segs, const double *x_segs, int num_segs,
             int num_fils) {
  std::vector<double> Z(3 * (size_t)num_fils), F(3 * (size_t)num_fils), S(1);
  emu_launch(blocks_for(3 * num_segs), THREADS_PER_BLOCK, [&] { reset_mean_fil_posns(Z.data()); });
  emu_launch(blocks_for(num_segs), THREADS_PER_BLOCK,
             [&] { write_mean_fil_posns(Z.data(), x_segs); });
  emu_launch(blocks_for(3 * num_segs), THREADS_PER_BLOCK,
             [&] { reset_mean_fil_force_and_moment(F.data(), S.data()); });
  emu_launch(blocks_for(num_segs), THREADS_PER_BLOCK, [&] {
    find_total_fil_force_and_first_moment(F.data(), S.data(), f_segs, x_segs, Z.data());
  });
  emu_launch(blocks_for(num_segs), THREADS_PER_BLOCK, [&] {
    Msf_mult(v_segs, f_segs, F.data(), S.data(), x_segs, Z.data(), 0, num_segs);
  });
}

void ref_barrier_forces(double *f_segs, double *f_blobs_repulsion, const double *x_segs,
                        const double *x_blobs, int num_segs, int num_blobs) {
  emu_launch(blocks_for(std::max(num_segs, num_blobs)), THREADS_PER_BLOCK, [&] {
    barrier_forces(f_segs, f_blobs_repulsion, x_segs, x_blobs, 0, num_segs, 0, num_blobs);
  });
}

}  // extern "C"
