// weakly_coupled_gb300.cu -- replacement for the reference's
// src/cilia/mobility/weakly_coupled_filaments_rpy_mobility_solver.cu
// (the mobility object when MOBILITY_TYPE is 2). The class its unchanged
// header declares overrides five hooks of rpy_mobility_solver; here they
// forward to libtfs_gb300.so like the base class's in rpy_mobility_solver.cu.
// The filament means and total forces the reference computes on upload
// (:50-89) are computed inside tfs_evaluate_weakly_coupled_segment_mobility
// from the device arrays, so the uploads are the plain copies; the
// per-filament device arrays of the header are not used.
#include "weakly_coupled_filaments_rpy_mobility_solver.hpp"
#include "tfs_shim.hpp"

weakly_coupled_filaments_rpy_mobility_solver::weakly_coupled_filaments_rpy_mobility_solver()
    : f_fils_device(nullptr), s_fils_device(nullptr), x_fils_device(nullptr) {}
weakly_coupled_filaments_rpy_mobility_solver::~weakly_coupled_filaments_rpy_mobility_solver() {}

void weakly_coupled_filaments_rpy_mobility_solver::allocate_device_memory() {
  rpy_mobility_solver::allocate_device_memory();
}

void weakly_coupled_filaments_rpy_mobility_solver::free_device_memory() {
  rpy_mobility_solver::free_device_memory();
}

void weakly_coupled_filaments_rpy_mobility_solver::copy_segment_positions_to_device() {
  rpy_mobility_solver::copy_segment_positions_to_device();
}

void weakly_coupled_filaments_rpy_mobility_solver::copy_segment_forces_to_device() {
  rpy_mobility_solver::copy_segment_forces_to_device();
}

// Msf_mult (cuda_functions.cu:1129-1229): RPY within each filament, the
// Stokeslet of every other filament's total force at its mean position
void weakly_coupled_filaments_rpy_mobility_solver::evaluate_segment_segment_mobility() {
  tfs_check(tfs_evaluate_weakly_coupled_segment_mobility(g_tfs_solver));
}
