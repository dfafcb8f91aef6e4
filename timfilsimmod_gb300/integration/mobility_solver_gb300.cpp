// mobility_solver_gb300.cpp -- the device-resident solve for the reference's
// mobility_solver (stage 2 of the binding; rpy_mobility_solver.cu in this
// directory is stage 1). These two members replace the same-named
// definitions in the reference's src/cilia/mobility/mobility_solver.cpp
// (delete them there, or compile this file in their place): the free-body
// compute_velocities (mobility_solver.cpp:2574-2659, with
// read_positions_and_forces :176-236, assemble_rhs :439-570 and
// solve_linear_system :2092-2570 folded into one library call), and
// make_body_reference_matrices (:2950-3047). Everything else of
// mobility_solver.cpp -- compute_errors, write_data, initialise -- stays the
// reference's. Compiled against the reference's unchanged headers, with Real
// double or float.
//
// The library solves one swimmer per solver (the reference's NSWIM = 1 runs).
#include <algorithm>
#include <vector>

#include "mobility_solver.hpp"
#include "swimmer.hpp"
#include "tfs_shim.hpp"

#if !USE_BROYDEN_FOR_EVERYTHING

void mobility_solver::compute_velocities(std::vector<swimmer> &swimmers, int &num_gmres_iterations,
                                         const int nt) {
  (void)nt;
  swimmer &sw = swimmers[0];
  // the body pose places the blobs on the device (rigid_body::blob_positions)
  const double x[3] = {sw.body.x[0], sw.body.x[1], sw.body.x[2]};
  const double q[4] = {sw.body.q.scalar_part, sw.body.q.vector_part[0], sw.body.q.vector_part[1],
                       sw.body.q.vector_part[2]};
  tfs_check(tfs_set_body_pose(g_tfs_solver, x, q));
  copy_segment_positions_to_device();
  copy_segment_forces_to_device();
  // barrier forces, M_ss and M_bs, the right-hand side, GMRES for the blob
  // forces and body velocity, then M_sb of the solved blob forces; the
  // swimmer's total force gains the blob repulsion, as the reference adds it
  double f[6];
  for (int k = 0; k < 6; ++k) f[k] = sw.f(k);
  tfs_check(tfs_compute_velocities(g_tfs_solver, f, &num_gmres_iterations));
  for (int k = 0; k < 6; ++k) sw.f(k) = (Real)f[k];
  double v[6];
  tfs_check(tfs_get_body_velocities(g_tfs_solver, v));
  for (int k = 0; k < 6; ++k) v_bodies(k) = (Real)v[k];
  tfs_check(tfs_shim::blob_solved_out(g_tfs_solver, f_blobs_host));
  copy_segment_velocities_to_host();
  wait_for_device();
}

void mobility_solver::make_body_reference_matrices(std::vector<swimmer> &swimmers) {
  const std::vector<Real> &refs = swimmers[0].body.blob_references;
  const std::vector<double> refs64(refs.begin(), refs.end());
  tfs_check(tfs_set_blob_references(g_tfs_solver, refs64.data()));
  tfs_check(tfs_set_linear_solver(g_tfs_solver, LINEAR_SYSTEM_TOL,
                                  std::min(3 * NBLOB + 6, (int)MAX_LINEAR_SYSTEM_ITER)));
  tfs_check(tfs_make_body_reference_matrices(g_tfs_solver));
  double bm[36], kt[36];  // column-major, as the reference's matrix
  tfs_check(tfs_get_body_reference_matrices(g_tfs_solver, bm, kt));
  for (int k = 0; k < 36; ++k) {
    body_mobility_reference(k) = (Real)bm[k];
    KTKinv_reference(k) = (Real)kt[k];
  }
}

#endif
