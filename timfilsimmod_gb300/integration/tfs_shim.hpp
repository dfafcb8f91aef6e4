// tfs_shim.hpp -- shared by the replacement translation units that bind the
// reference's mobility solver and flow-field classes to libtfs_gb300.so
// (rpy_mobility_solver.cu, mobility_solver_gb300.cpp,
// flow_field_evaluator_gb300.cpp in this directory).
//
// The reference's floating type `Real` is double or float (config.hpp:36-53,
// FIL_USE_DOUBLE_PRECISION); its pinned host arrays are Real
// (rpy_mobility_solver.cu:54-71). The overloads below pick the library's
// float64 or float32 copy entry point from the array type at compile time,
// so the same shim source serves both builds.
#pragma once

#include <cstdio>
#include <cstdlib>

#include "tfs_gb300.h"

// The library's solver behind the reference's rpy_mobility_solver (one per
// process, as the reference's single `mobility` object).
extern tfs_solver *g_tfs_solver;

// The reference signals no errors through its hooks (all void); a failing
// library call ends the run with the library's message, as the reference
// ends on a missing file (std::exit(-1)).
inline void tfs_check(int rc) {
  if (rc != TFS_OK) {
    std::fprintf(stderr, "libtfs_gb300: %s\n", tfs_last_error());
    std::exit(-1);
  }
}

namespace tfs_shim {
inline int seg_pos_in(tfs_solver *s, const double *p) { return tfs_copy_segment_positions_to_device(s, p); }
inline int seg_pos_in(tfs_solver *s, const float *p) { return tfs_copy_segment_positions_to_device_f32(s, p); }
inline int seg_force_in(tfs_solver *s, const double *p) { return tfs_copy_segment_forces_to_device(s, p); }
inline int seg_force_in(tfs_solver *s, const float *p) { return tfs_copy_segment_forces_to_device_f32(s, p); }
inline int blob_pos_in(tfs_solver *s, const double *p) { return tfs_copy_blob_positions_to_device(s, p); }
inline int blob_pos_in(tfs_solver *s, const float *p) { return tfs_copy_blob_positions_to_device_f32(s, p); }
inline int blob_force_in(tfs_solver *s, const double *p) { return tfs_copy_blob_forces_to_device(s, p); }
inline int blob_force_in(tfs_solver *s, const float *p) { return tfs_copy_blob_forces_to_device_f32(s, p); }
inline int blob_rep_out(tfs_solver *s, double *p) { return tfs_copy_interparticle_blob_forces_to_host(s, p); }
inline int blob_rep_out(tfs_solver *s, float *p) { return tfs_copy_interparticle_blob_forces_to_host_f32(s, p); }
inline int blob_vel_out(tfs_solver *s, double *p) { return tfs_copy_blob_velocities_to_host(s, p); }
inline int blob_vel_out(tfs_solver *s, float *p) { return tfs_copy_blob_velocities_to_host_f32(s, p); }
inline int seg_vel_out(tfs_solver *s, double *p) { return tfs_copy_segment_velocities_to_host(s, p); }
inline int seg_vel_out(tfs_solver *s, float *p) { return tfs_copy_segment_velocities_to_host_f32(s, p); }
inline int blob_solved_out(tfs_solver *s, double *p) { return tfs_copy_blob_forces_to_host(s, p); }
inline int blob_solved_out(tfs_solver *s, float *p) { return tfs_copy_blob_forces_to_host_f32(s, p); }
}  // namespace tfs_shim
