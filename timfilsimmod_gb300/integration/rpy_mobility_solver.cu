// rpy_mobility_solver.cu -- replacement for the reference's
// src/cilia/mobility/rpy_mobility_solver.cu. It defines the class the
// reference's unchanged rpy_mobility_solver.hpp declares, with every one of
// the 17 device hooks of mobility_solver.hpp:26-46 forwarded to the C ABI of
// libtfs_gb300.so (include/tfs_gb300.h). The reference's host arrays stay
// where they are -- pinned, of type Real, owned here as in the reference
// (rpy_mobility_solver.cu:54-71) -- and the library copies them in and out;
// filaments and swimmers keep writing into them in place.
//
// Build: in the reference's makefile, compile this file instead of its own
// rpy_mobility_solver.cu, add -I<repo>/include -I<repo>/timfilsimmod_gb300/integration
// and link -L<repo>/timfilsimmod_gb300 -ltfs_gb300. Works with Real = double
// or float (the float arrays go through the library's *_f32 entry points,
// converted on the device).
#include <cuda_runtime.h>

#include "rpy_mobility_solver.hpp"
#include "tfs_shim.hpp"

tfs_solver *g_tfs_solver = nullptr;

rpy_mobility_solver::rpy_mobility_solver() {}
rpy_mobility_solver::~rpy_mobility_solver() {}

void rpy_mobility_solver::allocate_host_memory() {
  num_gpus = 1;  // one GB300; the library keeps every target on one device
  const size_t ns = (size_t)NSWIM * NFIL * NSEG, nb = (size_t)NSWIM * NBLOB;
  cudaHostAlloc(&v_segs_host, 6 * ns * sizeof(Real), cudaHostAllocPortable);
  cudaHostAlloc(&v_blobs_host, 3 * nb * sizeof(Real), cudaHostAllocPortable);
  cudaHostAlloc(&x_segs_host, 3 * ns * sizeof(Real), cudaHostAllocPortable);
  cudaHostAlloc(&x_blobs_host, 3 * nb * sizeof(Real), cudaHostAllocPortable);
  cudaHostAlloc(&f_segs_host, 6 * ns * sizeof(Real), cudaHostAllocPortable);
  cudaHostAlloc(&f_blobs_host, 3 * nb * sizeof(Real), cudaHostAllocPortable);
  cudaHostAlloc(&f_blobs_repulsion_host, 3 * nb * sizeof(Real), cudaHostAllocPortable);
}

void rpy_mobility_solver::allocate_device_memory() {
  tfs_config cfg;
  tfs_check(tfs_config_default(&cfg, NSWIM, NFIL, NSEG, NBLOB));
  cfg.mu = MU;
  cfg.a_seg = RSEG;
  cfg.a_blob = RBLOB;
  cfg.end_force_magnitude = (int)END_FORCE_MAGNITUDE;  // the device's int copy (sync_var)
#if PRESCRIBED_CILIA  // prescribed filaments have no barrier forces (cuda_functions.cu:1242)
  cfg.repulsive_force_factor = 0.0;
#else
  cfg.repulsive_force_factor = REPULSIVE_FORCE_FACTOR;
#endif
  cfg.free_body = PRESCRIBED_BODY_VELOCITIES ? 0 : 1;
  cfg.precision = TFS_FP64;  // TFS_FP32C: FP32 pair sums, FP64-refined solves
  tfs_check(tfs_solver_create(&cfg, &g_tfs_solver));
}

void rpy_mobility_solver::free_host_memory() {
  cudaFreeHost(v_segs_host);
  cudaFreeHost(v_blobs_host);
  cudaFreeHost(x_segs_host);
  cudaFreeHost(x_blobs_host);
  cudaFreeHost(f_segs_host);
  cudaFreeHost(f_blobs_host);
  cudaFreeHost(f_blobs_repulsion_host);
}

void rpy_mobility_solver::free_device_memory() {
  tfs_solver_destroy(g_tfs_solver);
  g_tfs_solver = nullptr;
}

void rpy_mobility_solver::copy_segment_positions_to_device() {
  tfs_check(tfs_shim::seg_pos_in(g_tfs_solver, x_segs_host));
}
void rpy_mobility_solver::copy_segment_forces_to_device() {
  tfs_check(tfs_shim::seg_force_in(g_tfs_solver, f_segs_host));
}
void rpy_mobility_solver::copy_blob_positions_to_device() {
  tfs_check(tfs_shim::blob_pos_in(g_tfs_solver, x_blobs_host));
}
void rpy_mobility_solver::copy_blob_forces_to_device() {
  tfs_check(tfs_shim::blob_force_in(g_tfs_solver, f_blobs_host));
}
void rpy_mobility_solver::copy_interparticle_blob_forces_to_host() {
  tfs_check(tfs_shim::blob_rep_out(g_tfs_solver, f_blobs_repulsion_host));
}
void rpy_mobility_solver::copy_blob_velocities_to_host() {
  tfs_check(tfs_shim::blob_vel_out(g_tfs_solver, v_blobs_host));
}
void rpy_mobility_solver::copy_segment_velocities_to_host() {
  tfs_check(tfs_shim::seg_vel_out(g_tfs_solver, v_segs_host));
}
void rpy_mobility_solver::apply_interparticle_forces() {
  tfs_check(tfs_apply_interparticle_forces(g_tfs_solver));
}
void rpy_mobility_solver::wait_for_device() { tfs_check(tfs_wait_for_device(g_tfs_solver)); }
void rpy_mobility_solver::evaluate_segment_segment_mobility() {
  tfs_check(tfs_evaluate_segment_segment_mobility(g_tfs_solver));
}
void rpy_mobility_solver::evaluate_segment_blob_mobility() {
  tfs_check(tfs_evaluate_segment_blob_mobility(g_tfs_solver));
}
void rpy_mobility_solver::evaluate_blob_blob_mobility() {
  tfs_check(tfs_evaluate_blob_blob_mobility(g_tfs_solver));
}
void rpy_mobility_solver::evaluate_blob_segment_mobility() {
  tfs_check(tfs_evaluate_blob_segment_mobility(g_tfs_solver));
}
// v_segs = Mss f_segs + Msb f_blobs, v_blobs = Mbs f_segs, both copied to
// the host (the reference's evaluate_full_mobility, rpy_mobility_solver.cu:330-337:
// its Mbb result is overwritten by Mbs)
void rpy_mobility_solver::evaluate_full_mobility() {
  evaluate_segment_segment_mobility();
  evaluate_segment_blob_mobility();
  copy_segment_velocities_to_host();
  evaluate_blob_blob_mobility();
  evaluate_blob_segment_mobility();
  copy_blob_velocities_to_host();
}
