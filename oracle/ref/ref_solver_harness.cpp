// ref_solver_harness.cpp -- runs the reference's own mobility solve
// (src/cilia/mobility/mobility_solver.cpp: compute_velocities,
// assemble_rhs, solve_linear_system, apply_preconditioner_new,
// system_matrix_mult_new, make_body_reference_matrices) on the CPU.
//
// TEST INFRASTRUCTURE ONLY. Built by oracle/Makefile into oracle/_ref/ from
// the reference sources in place, against a CPU stand-in for
// rpy_mobility_solver whose hooks call the reference's own kernels (run by
// the CUDA emulation in ref_kernels_harness.cpp) on separate "device"
// buffers, so the reference's host/device copy semantics are kept (e.g.
// barrier forces reach only the device copy of the segment forces).
//
// Also provided here because the reference links them from elsewhere:
//   - the run-time globals of globals.cu (that file does not compile with
//     CILIA_TYPE 0, where DT is a macro);
//   - a LAPACK stand-in (dgetrf_/dgetri_/dgemm_: textbook LU with partial
//     pivoting, inverse from the LU factors, naive GEMM), since no LAPACK is
//     installed; it only serves matrix::invert and matrix products;
//   - stubs for the seeding functions (seeding.cu needs a GPU), which the
//     harness never calls: geometry is injected directly.
#include <cmath>
#include <fstream>
#include <iomanip>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "mobility/mobility_solver.hpp"
#include "swimmer.hpp"

// ---------------------------------------------------------------------------
// globals (globals.cu / config.hpp externs)
int NSWIM = 1, NSEG = 1, NFIL = 1, NBLOB = 1;
Real AR = 1.0, AXIS_DIR_BODY_LENGTH = 1.0, TORSIONAL_SPRING_MAGNITUDE_FACTOR = 2.0,
     GEN_FORCE_MAGNITUDE_FACTOR = 1.0;
int NTOTAL = 0;
Real END_FORCE_MAGNITUDE = 0.0, SEG_SEP = 2.2, DL = 2.2, SIM_LENGTH = 1.0, PERIOD = 1.0;
int TOTAL_TIME_STEPS = 1;
std::string SIMULATION_DIR = "/tmp/", SIMULATION_FILE = "tfs_ref";
std::string SIMULATION_NAME = "/tmp/tfs_ref", SIMULATION_CONFIG_NAME, SIMULATION_BACKUP_NAME,
            SIMULATION_BODY_STATE_NAME, SIMULATION_SEG_STATE_NAME, SIMULATION_BODY_VEL_NAME,
            SIMULATION_SEG_VEL_NAME, SIMULATION_BLOB_FORCES_NAME, SIMULATION_SEG_FORCES_NAME,
            SIMULATION_TIME_NAME, SIMULATION_TETHERLAM_NAME, SIMULATION_TRUESTATE_NAME,
            SIMULATION_READPHASE_NAME, SIMULATION_READANGLE_NAME;

// ---------------------------------------------------------------------------
// LAPACK stand-in (column-major, Fortran calling convention)
extern "C" {

void dgetrf_(int *m, int *n, double *a, int *lda, int *ipiv, int *info) {
  const int M = *m, N = *n, L = *lda;
  *info = 0;
  for (int k = 0; k < std::min(M, N); ++k) {
    int p = k;
    double best = std::fabs(a[k + k * L]);
    for (int i = k + 1; i < M; ++i)
      if (std::fabs(a[i + k * L]) > best) {
        best = std::fabs(a[i + k * L]);
        p = i;
      }
    ipiv[k] = p + 1;
    if (a[p + k * L] == 0.0) {
      if (*info == 0) *info = k + 1;
      continue;
    }
    if (p != k)
      for (int j = 0; j < N; ++j) std::swap(a[k + j * L], a[p + j * L]);
    for (int i = k + 1; i < M; ++i) a[i + k * L] /= a[k + k * L];
    for (int j = k + 1; j < N; ++j)
      for (int i = k + 1; i < M; ++i) a[i + j * L] -= a[i + k * L] * a[k + j * L];
  }
}

void dgetri_(int *n, double *a, int *lda, int *ipiv, double *work, int *lwork, int *info) {
  const int N = *n, L = *lda;
  *info = 0;
  if (*lwork == -1) {  // workspace query
    work[0] = N;
    return;
  }
  std::vector<double> inv((size_t)N * N, 0.0);
  for (int c = 0; c < N; ++c) {
    std::vector<double> b(N, 0.0);
    b[c] = 1.0;
    // solve A x = e_c with P A = L U: apply the row swaps to b in order
    for (int k = 0; k < N; ++k) std::swap(b[k], b[ipiv[k] - 1]);
    for (int i = 0; i < N; ++i)
      for (int k = 0; k < i; ++k) b[i] -= a[i + k * L] * b[k];
    for (int i = N - 1; i >= 0; --i) {
      for (int k = i + 1; k < N; ++k) b[i] -= a[i + k * L] * b[k];
      b[i] /= a[i + i * L];
    }
    for (int i = 0; i < N; ++i) inv[i + (size_t)c * N] = b[i];
  }
  for (int j = 0; j < N; ++j)
    for (int i = 0; i < N; ++i) a[i + j * L] = inv[i + (size_t)j * N];
}

void dgemm_(char *ta, char *tb, int *m, int *n, int *k, double *alpha, const double *A, int *lda,
            const double *B, int *ldb, double *beta, double *C, int *ldc) {
  const bool tA = (*ta == 'T' || *ta == 't'), tB = (*tb == 'T' || *tb == 't');
  for (int j = 0; j < *n; ++j)
    for (int i = 0; i < *m; ++i) {
      double s = 0.0;
      for (int p = 0; p < *k; ++p) {
        const double av = tA ? A[p + i * *lda] : A[i + p * *lda];
        const double bv = tB ? B[j + p * *ldb] : B[p + j * *ldb];
        s += av * bv;
      }
      C[i + j * *ldc] = *alpha * s + (*beta == 0.0 ? 0.0 : *beta * C[i + j * *ldc]);
    }
}

// reference kernels (ref_kernels_harness.cpp)
void ref_sync_var(int nswim, int nseg, int nfil, int nblob, int end_force_magnitude,
                  double seg_sep);
void ref_mss(double *, const double *, const double *, int);
void ref_msb(double *, const double *, const double *, const double *, int);
void ref_mbb(double *, const double *, const double *, int);
void ref_mbs(double *, const double *, const double *, const double *, int);
void ref_msf(double *, const double *, const double *, int, int);
void ref_barrier_forces(double *, double *, const double *, const double *, int, int);
}

// The C restatement of the same kernels (tfs_oracle.c, pinned to these to
// ~5e-16 by tests/test_oracle.py), multi-threaded: the implicit-step runs
// switch to it with ref_use_port_kernels, because the emulated kernels (one
// host thread per CUDA thread) take minutes per Broyden iteration.
#include "../tfs_oracle.h"
static int g_use_port = 0;
static orc_params g_port_params = {1.0, 1.0, 1.0};
extern "C" void ref_use_port_kernels(int threads) {
  g_use_port = threads > 0;
  if (threads > 0) orc_set_threads(threads);
}

void seed_blobs(Real *const, Real *const, Real *const, Real *const) { std::abort(); }
void seed_filaments(Real *const, Real *const, Real *const, Real *const) { std::abort(); }
void check_seeding(Real *const, Real *const, Real *const, Real *const) { std::abort(); }

// ---------------------------------------------------------------------------
// CPU stand-in for rpy_mobility_solver (one "GPU"): the 17 hooks of
// mobility_solver.hpp:26-46 with host buffers for the device arrays.
class emu_rpy_mobility_solver : public mobility_solver {
 public:
  std::vector<Real> xs_d, fs_d, vs_d, xb_d, fb_d, vb_d, frep_d;
  int ns() const { return NSWIM * NFIL * NSEG; }
  int nb() const { return NSWIM * NBLOB; }

  void free_host_memory() override {
    delete[] v_segs_host; delete[] v_blobs_host; delete[] x_segs_host; delete[] x_blobs_host;
    delete[] f_segs_host; delete[] f_blobs_host; delete[] f_blobs_repulsion_host;
  }
  void free_device_memory() override {}
  void allocate_host_memory() override {
    v_segs_host = new Real[6 * ns()](); x_segs_host = new Real[3 * ns()]();
    f_segs_host = new Real[6 * ns()](); v_blobs_host = new Real[3 * nb()]();
    x_blobs_host = new Real[3 * nb()](); f_blobs_host = new Real[3 * nb()]();
    f_blobs_repulsion_host = new Real[3 * nb()]();
  }
  void allocate_device_memory() override {
    xs_d.assign(3 * ns(), 0); fs_d.assign(6 * ns(), 0); vs_d.assign(6 * ns(), 0);
    xb_d.assign(3 * nb(), 0); fb_d.assign(3 * nb(), 0); vb_d.assign(3 * nb(), 0);
    frep_d.assign(3 * nb(), 0);
  }
  void copy_segment_positions_to_device() override { std::memcpy(xs_d.data(), x_segs_host, 8 * xs_d.size()); }
  void copy_segment_forces_to_device() override { std::memcpy(fs_d.data(), f_segs_host, 8 * fs_d.size()); }
  void copy_blob_positions_to_device() override { std::memcpy(xb_d.data(), x_blobs_host, 8 * xb_d.size()); }
  void copy_blob_forces_to_device() override { std::memcpy(fb_d.data(), f_blobs_host, 8 * fb_d.size()); }
  void copy_interparticle_blob_forces_to_host() override { std::memcpy(f_blobs_repulsion_host, frep_d.data(), 8 * frep_d.size()); }
  void copy_blob_velocities_to_host() override { std::memcpy(v_blobs_host, vb_d.data(), 8 * vb_d.size()); }
  void copy_segment_velocities_to_host() override { std::memcpy(v_segs_host, vs_d.data(), 8 * vs_d.size()); }
  void apply_interparticle_forces() override {
#if !PRESCRIBED_CILIA  // the prescribed-cilia configurations never call it
    if (g_use_port)
      orc_barrier_forces(&g_port_params, fs_d.data(), frep_d.data(), xs_d.data(), xb_d.data(), ns(),
                         nb(), NSEG, (int)END_FORCE_MAGNITUDE, REPULSIVE_FORCE_FACTOR, 1);
    else
      ref_barrier_forces(fs_d.data(), frep_d.data(), xs_d.data(), xb_d.data(), ns(), nb());
#endif
  }
  void wait_for_device() override {}
  void evaluate_segment_segment_mobility() override {
#if WEAKLY_COUPLED_FILAMENTS_RPY_MOBILITY
    // weakly_coupled_filaments_rpy_mobility_solver.cu:50-107: filament means
    // and total forces, then Msf_mult (all by the reference's kernels)
    ref_msf(vs_d.data(), fs_d.data(), xs_d.data(), ns(), NSWIM * NFIL);
#else
    if (g_use_port) orc_mss(&g_port_params, vs_d.data(), fs_d.data(), xs_d.data(), ns());
    else ref_mss(vs_d.data(), fs_d.data(), xs_d.data(), ns());
#endif
  }
  void evaluate_segment_blob_mobility() override {
    if (g_use_port) orc_msb(&g_port_params, vs_d.data(), fb_d.data(), xs_d.data(), xb_d.data(), ns(), nb());
    else ref_msb(vs_d.data(), fb_d.data(), xs_d.data(), xb_d.data(), ns());
  }
  void evaluate_blob_blob_mobility() override {
    if (g_use_port) orc_mbb(&g_port_params, vb_d.data(), fb_d.data(), xb_d.data(), nb());
    else ref_mbb(vb_d.data(), fb_d.data(), xb_d.data(), nb());
  }
  void evaluate_blob_segment_mobility() override {
    if (g_use_port) orc_mbs(&g_port_params, vb_d.data(), fs_d.data(), xb_d.data(), xs_d.data(), nb(), ns());
    else ref_mbs(vb_d.data(), fs_d.data(), xb_d.data(), xs_d.data(), nb());
  }
  void evaluate_full_mobility() override {
    evaluate_segment_segment_mobility(); evaluate_segment_blob_mobility();
    copy_segment_velocities_to_host(); evaluate_blob_blob_mobility();
    evaluate_blob_segment_mobility(); copy_blob_velocities_to_host();
  }
};

static emu_rpy_mobility_solver *g_solver = nullptr;
static std::vector<swimmer> *g_swimmers = nullptr;

extern "C" {

// One swimmer: NFIL x NSEG segments, NBLOB blobs with body-frame references
// blob_refs[3*NBLOB], body position x[3] and orientation q = (q0, q1, q2, q3).
// end_force_magnitude is the Real END_FORCE_MAGNITUDE; the device copy used by
// the barrier kernel is its int truncation, as sync_var makes it.
int ref_solver_setup(int nfil, int nseg, int nblob, double end_force_magnitude, double seg_sep,
                     const double *blob_refs, const double *body_x, const double *body_q) {
  NSWIM = 1; NFIL = nfil; NSEG = nseg; NBLOB = nblob;
  SEG_SEP = seg_sep; DL = seg_sep;
  END_FORCE_MAGNITUDE = end_force_magnitude;
  NTOTAL = NSWIM * (NFIL * NSEG + NBLOB);
  ref_sync_var(NSWIM, NSEG, NFIL, NBLOB, (int)END_FORCE_MAGNITUDE, SEG_SEP);
  delete g_swimmers;
  if (g_solver) { g_solver->finalise(); delete g_solver; }
  g_solver = new emu_rpy_mobility_solver();
  g_solver->initialise();
  g_swimmers = new std::vector<swimmer>(1);
  swimmer &s = (*g_swimmers)[0];
  s.f = matrix(6, 1);
  s.f.zero();
  s.body.blob_references.assign(blob_refs, blob_refs + 3 * nblob);
  for (int k = 0; k < 3; ++k) s.body.x[k] = body_x[k];
  s.body.q = quaternion(body_q[0], body_q[1], body_q[2], body_q[3]);
  return 0;
}

// make_body_reference_matrices (mobility_solver.cpp:2950-3047) on the current
// segment positions/forces; returns body_mobility_reference and
// KTKinv_reference (6x6, column-major as matrix stores them).
void ref_make_body_reference_matrices(const double *x_segs, const double *f_segs,
                                      double *body_mobility, double *ktkinv) {
  std::memcpy(g_solver->x_segs_host, x_segs, 8 * 3 * g_solver->ns());
  std::memcpy(g_solver->f_segs_host, f_segs, 8 * 6 * g_solver->ns());
  g_solver->make_body_reference_matrices(*g_swimmers);
  for (int k = 0; k < 36; ++k) {
    body_mobility[k] = g_solver->body_mobility_reference.data[k];
    ktkinv[k] = g_solver->KTKinv_reference.data[k];
  }
}

// compute_velocities (mobility_solver.cpp:2574-2659, free-body branch) with the
// swimmer's total force/torque swimmer_f[6] (what swimmer::forces_and_torques
// leaves in swimmer.f). Returns the GMRES iteration count.
int ref_compute_velocities(const double *x_segs, const double *f_segs, const double *swimmer_f,
                           int nt, double *v_segs, double *v_blobs, double *f_blobs,
                           double *v_bodies, double *swimmer_f_out) {
  std::memcpy(g_solver->x_segs_host, x_segs, 8 * 3 * g_solver->ns());
  std::memcpy(g_solver->f_segs_host, f_segs, 8 * 6 * g_solver->ns());
  swimmer &s = (*g_swimmers)[0];
  for (int k = 0; k < 6; ++k) s.f(k) = swimmer_f[k];
  int iters = 0;
  g_solver->compute_velocities(*g_swimmers, iters, nt);
  std::memcpy(v_segs, g_solver->v_segs_host, 8 * 6 * g_solver->ns());
  std::memcpy(v_blobs, g_solver->v_blobs_host, 8 * 3 * g_solver->nb());
  std::memcpy(f_blobs, g_solver->f_blobs_host, 8 * 3 * g_solver->nb());
  for (int k = 0; k < 6; ++k) {
    v_bodies[k] = g_solver->v_bodies(k);
    swimmer_f_out[k] = s.f(k);
  }
  return iters;
}

// The GMRES warm-start state (f_blobs_host, v_bodies), settable for tests.
void ref_set_warm_start(const double *f_blobs, const double *v_bodies) {
  std::memcpy(g_solver->f_blobs_host, f_blobs, 8 * 3 * g_solver->nb());
  for (int k = 0; k < 6; ++k) g_solver->v_bodies(k) = v_bodies[k];
}

// Move/rotate the body (rigid_body::x, q).
void ref_set_body(const double *body_x, const double *body_q) {
  swimmer &s = (*g_swimmers)[0];
  for (int k = 0; k < 3; ++k) s.body.x[k] = body_x[k];
  s.body.q = quaternion(body_q[0], body_q[1], body_q[2], body_q[3]);
}

double ref_linear_system_tol(void) { return LINEAR_SYSTEM_TOL; }
int ref_max_linear_system_iter(void) { return MAX_LINEAR_SYSTEM_ITER; }

}  // extern "C"

#if INSTABILITY_CILIA
// ---------------------------------------------------------------------------
// Implicit time steps (src/cilia/cilia_sim_main.cu:355-527) of one free
// swimmer with elastic filaments, driven stage by stage so that tests can
// compare every stage: initial guess, forces, compute_velocities,
// compute_errors, the approximate Jacobian, Broyden updates, end of step.
#include "broyden_solver.hpp"

static broyden_solver *g_broyden = nullptr;

extern "C" {

// Geometry: blob references (body frame, blob_refs[3*NBLOB]), filament base
// offsets (body frame, fil_refs[3*NFIL], as swimmer::initial_setup leaves
// filament_references: already including the (RBLOB + DL/2) normal offset),
// filament directions fil_dirs[3*NFIL], body position/orientation, and the
// body length AXIS_DIR_BODY_LENGTH = 2R used by the sphere correction of
// swimmer::prepare_jacobian_inv.
int ref_step_setup(int nfil, int nseg, int nblob, double end_force_magnitude, double seg_sep,
                   double axis_dir_body_length, const double *blob_refs, const double *fil_refs,
                   const double *fil_dirs, const double *body_x, const double *body_q) {
  NSWIM = 1; NFIL = nfil; NSEG = nseg; NBLOB = nblob;
  SEG_SEP = seg_sep; DL = seg_sep;
  AXIS_DIR_BODY_LENGTH = axis_dir_body_length;
  END_FORCE_MAGNITUDE = end_force_magnitude;
  NTOTAL = NSWIM * (NFIL * NSEG + NBLOB);
  ref_sync_var(NSWIM, NSEG, NFIL, NBLOB, (int)END_FORCE_MAGNITUDE, SEG_SEP);
  delete g_swimmers;
  delete g_broyden;
  if (g_solver) { g_solver->finalise(); delete g_solver; }
  g_solver = new emu_rpy_mobility_solver();
  g_solver->initialise();
  g_broyden = new broyden_solver();
  g_swimmers = new std::vector<swimmer>(1);
  swimmer &s = (*g_swimmers)[0];
  s.f = matrix(6, 1);
  s.f.zero();
  s.schur_mat_inv = matrix(6, 6);
  s.jacobian_B_blocks = std::vector<matrix>(NFIL);
  rigid_body &b = s.body;
  b.blob_references.assign(blob_refs, blob_refs + 3 * nblob);
  b.Q_init = matrix(3, 3);
  for (int k = 0; k < 3; ++k) {
    b.x[k] = b.xm1[k] = b.xm2[k] = body_x[k];
    b.u[k] = b.um1[k] = 0.0;
  }
  b.q = quaternion(body_q[0], body_q[1], body_q[2], body_q[3]);
  b.qm1 = b.q;
  s.filament_references.assign(fil_refs, fil_refs + 3 * nfil);
  s.normal_refs.assign(fil_dirs, fil_dirs + 3 * nfil);
  s.filaments = std::vector<filament>(NFIL);
  const Real strain_twist[3] = {0.0, 0.0, 0.0};
  for (int i = 0; i < NFIL; ++i) {
    const Real pos[3] = {b.x[0] + fil_refs[3 * i], b.x[1] + fil_refs[3 * i + 1],
                         b.x[2] + fil_refs[3 * i + 2]};
    s.filaments[i].initial_setup(pos, &fil_dirs[3 * i], strain_twist, nullptr,
                                 &g_solver->x_segs_host[3 * i * NSEG],
                                 &g_solver->f_segs_host[6 * i * NSEG], i);
  }
  return 0;
}

void ref_step_make_body_reference_matrices(double *body_mobility, double *ktkinv) {
  g_solver->make_body_reference_matrices(*g_swimmers);
  (*g_swimmers)[0].body_mobility_reference = g_solver->body_mobility_reference;
  for (int k = 0; k < 36; ++k) {
    body_mobility[k] = g_solver->body_mobility_reference.data[k];
    ktkinv[k] = g_solver->KTKinv_reference.data[k];
  }
}

void ref_step_initial_guess(int nt) { (*g_swimmers)[0].initial_guess(nt); }

// forces_and_torques; returns the host segment forces and the swimmer force.
void ref_step_forces(int nt, double *f_segs, double *swimmer_f) {
  swimmer &s = (*g_swimmers)[0];
  s.forces_and_torques(nt, 0);
  std::memcpy(f_segs, g_solver->f_segs_host, 8 * 6 * g_solver->ns());
  for (int k = 0; k < 6; ++k) swimmer_f[k] = s.f(k);
}

// compute_velocities on the current state; returns GMRES iterations.
int ref_step_compute_velocities(int nt, double *v_segs, double *v_bodies, double *f_blobs) {
  int iters = 0;
  g_solver->compute_velocities(*g_swimmers, iters, nt);
  std::memcpy(v_segs, g_solver->v_segs_host, 8 * 6 * g_solver->ns());
  std::memcpy(f_blobs, g_solver->f_blobs_host, 8 * 3 * g_solver->nb());
  for (int k = 0; k < 6; ++k) v_bodies[k] = g_solver->v_bodies(k);
  return iters;
}

// compute_errors into broyden.error (which = 0) or broyden.new_error (1).
int ref_step_compute_errors(int nt, int which, double *error) {
  matrix &e = which ? g_broyden->new_error : g_broyden->error;
  const bool big = g_solver->compute_errors(e, *g_swimmers, nt);
  std::memcpy(error, e.data.data(), 8 * e.data.size());
  return big ? 1 : 0;
}

void ref_step_prepare_jacobian_inv(int nt, double *schur_inv) {
  swimmer &s = (*g_swimmers)[0];
  s.prepare_jacobian_inv(nt);
  for (int k = 0; k < 36; ++k) schur_inv[k] = s.schur_mat_inv.data[k];
}

// Filament i's inverse approximate Jacobian (6 NSEG x 6 NSEG, column-major).
void ref_step_inverse_jacobian(int i, double *out) {
  const matrix &J = (*g_swimmers)[0].filaments[i].inverse_jacobian;
  std::memcpy(out, J.data.data(), 8 * J.data.size());
}

// swimmer.jacobian_inv_mult(in) (the approximate inverse Jacobian product).
void ref_step_jacobian_inv_mult(int nt, const double *in, double *out) {
  const int nbroy = 6 * (NFIL * NSEG + 1);
  matrix m(nbroy, 1);
  std::memcpy(m.data.data(), in, 8 * nbroy);
  const matrix r = (*g_swimmers)[0].jacobian_inv_mult(m, nt);
  std::memcpy(out, r.data.data(), 8 * nbroy);
}

void ref_step_broyden_reset(void) { g_broyden->iter = 0; }

void ref_step_find_update(int nt, double *update) {
  g_broyden->find_update(*g_swimmers, nt);
  std::memcpy(update, g_broyden->update.data.data(), 8 * g_broyden->update.data.size());
}

// swimmer.update(broyden.update) then forces_and_torques (the loop body).
void ref_step_apply_update(int nt) {
  swimmer &s = (*g_swimmers)[0];
  s.update(&g_broyden->update.data[0]);
  s.forces_and_torques(nt, 0);
}

void ref_step_end_of_iter(int nt, int error_is_too_large) {
  g_broyden->end_of_iter(*g_swimmers, nt, 0, error_is_too_large != 0);
}

// One whole time step (the loop of cilia_sim_main.cu:355-527); returns the
// Broyden iteration count (-1 if Broyden diverged), total GMRES iterations in
// *gmres_iters.
int ref_step_run(int nt, int *gmres_iters) {
  swimmer &s = (*g_swimmers)[0];
  s.initial_guess(nt);
  s.forces_and_torques(nt, 0);
  int it = 0, total = 0;
  g_solver->compute_velocities(*g_swimmers, it, nt);
  total += it;
  bool big = g_solver->compute_errors(g_broyden->error, *g_swimmers, nt);
  if (big) s.prepare_jacobian_inv(nt);
  g_broyden->iter = 0;
  while (big && g_broyden->iter < MAX_BROYDEN_ITER) {
    g_broyden->find_update(*g_swimmers, nt);
    s.update(&g_broyden->update.data[0]);
    s.forces_and_torques(nt, 0);
    g_solver->compute_velocities(*g_swimmers, it, nt);
    total += it;
    big = g_solver->compute_errors(g_broyden->new_error, *g_swimmers, nt);
    if (!g_broyden->new_error.is_finite()) return -1;
    g_broyden->end_of_iter(*g_swimmers, nt, 0, big);
  }
  s.end_of_step(nt);
  if (gmres_iters) *gmres_iters = total;
  return g_broyden->iter;
}

// State: segment positions x[3 Ns], quaternions q[4 Ns] (scalar first),
// Lie algebra u[3 Ns]; per filament lambda[3 (NSEG-1)], tether[3], clamp[3];
// body x[3], q[4], u[3].
void ref_step_state(double *x, double *q, double *u, double *lambda, double *tether,
                    double *clamp, double *body_x, double *body_q, double *body_u) {
  swimmer &s = (*g_swimmers)[0];
  for (int i = 0; i < NFIL; ++i) {
    filament &fl = s.filaments[i];
    for (int j = 0; j < NSEG; ++j) {
      const segment &sg = fl.segments[j];
      const int id = i * NSEG + j;
      for (int k = 0; k < 3; ++k) { x[3 * id + k] = sg.x[k]; u[3 * id + k] = sg.u[k]; }
      q[4 * id] = sg.q.scalar_part;
      for (int k = 0; k < 3; ++k) q[4 * id + 1 + k] = sg.q.vector_part[k];
    }
    for (int k = 0; k < 3 * (NSEG - 1); ++k) lambda[3 * (NSEG - 1) * i + k] = fl.lambda[k];
    for (int k = 0; k < 3; ++k) { tether[3 * i + k] = fl.tether_lambda[k]; clamp[3 * i + k] = fl.clamp_lambda[k]; }
  }
  for (int k = 0; k < 3; ++k) { body_x[k] = s.body.x[k]; body_u[k] = s.body.u[k]; }
  body_q[0] = s.body.q.scalar_part;
  for (int k = 0; k < 3; ++k) body_q[1 + k] = s.body.q.vector_part[k];
}

// The reference's own writers at a plot step after step nt, in the order
// its main loop calls them (cilia_sim_main.cu:563-600): swimmer::write_data
// into <prefix>_seg_states.dat, _body_states.dat, _tether_force.dat (step
// nt+1), mobility_solver::write_data into the velocity and force files (step
// nt), swimmer::write_backup into <prefix>.backup. File names as
// cilia_sim_main.cu:94-102 derives them.
void ref_step_write_files(const char *prefix, int nt) {
  swimmer &s = (*g_swimmers)[0];
  SIMULATION_NAME = prefix;
  SIMULATION_BACKUP_NAME = SIMULATION_NAME + ".backup";
  SIMULATION_BODY_STATE_NAME = SIMULATION_NAME + "_body_states.dat";
  SIMULATION_SEG_STATE_NAME = SIMULATION_NAME + "_seg_states.dat";
  SIMULATION_BODY_VEL_NAME = SIMULATION_NAME + "_body_vels.dat";
  SIMULATION_SEG_VEL_NAME = SIMULATION_NAME + "_seg_vels.dat";
  SIMULATION_BLOB_FORCES_NAME = SIMULATION_NAME + "_blob_forces.dat";
  SIMULATION_SEG_FORCES_NAME = SIMULATION_NAME + "_seg_forces.dat";
  SIMULATION_TETHERLAM_NAME = SIMULATION_NAME + "_tether_force.dat";
  const int save_step = nt + 1;
  std::ofstream seg(SIMULATION_SEG_STATE_NAME, std::ios::app);
  std::ofstream body(SIMULATION_BODY_STATE_NAME, std::ios::app);
  std::ofstream tether(SIMULATION_TETHERLAM_NAME, std::ios::app);
  for (std::ofstream *f : {&seg, &body, &tether}) *f << save_step << " " << std::scientific << std::setprecision(10);
  s.write_data(seg, body, tether);
  for (std::ofstream *f : {&seg, &body, &tether}) *f << std::endl;
  seg.close();
  body.close();
  tether.close();
  g_solver->write_data(nt, *g_swimmers);
  std::ofstream backup(SIMULATION_BACKUP_NAME);
  backup << save_step << " " << std::scientific << std::setprecision(10);
  s.write_backup(backup);
  backup << std::endl;
}

}  // extern "C"
#endif  // INSTABILITY_CILIA

#if PRESCRIBED_CILIA
// ---------------------------------------------------------------------------
// Prescribed-cilia mobility solve of one swimmer: compute_velocities under
// PRESCRIBED_CILIA (mobility_solver.cpp:2574-2596) with assemble_rhs
// (:282-437), solve_linear_system (:2092-2570), apply_preconditioner_new
// (:1040-1436) and system_matrix_mult_new (:1806-2026). The filaments'
// kinematics (segment positions, d x / d phase, d x / d angle, phases,
// natural frequencies, shape-rotation angles, prescribed phase rates) are
// set directly instead of by the shape-sequence code, and
// swimmer::make_precon_mat (swimmer.cpp:1154-1322) runs after them, as
// swimmer::initial_guess runs it.
#include <sys/stat.h>
#include <unistd.h>

// Under PRESCRIBED_CILIA the time step is a run-time global (globals.cu:21);
// it only scales the prescribed body velocities' time argument, which are
// zero (rigid_body.cpp:584-598). The solver's DISPLAYTIME blocks
// (config.hpp:531) synchronise the device before each timer read.
Real DT = 1.0;
cudaError_t cudaDeviceSynchronize(void) { return cudaSuccess; }

extern "C" {

// Which prescribed-cilia branches this build compiled: 1 prescribed body
// velocities, 2 dynamic phase evolution, 4 dynamic shape rotation, 8 weakly
// coupled filaments' mobility.
int ref_pres_flags(void) {
  return (PRESCRIBED_BODY_VELOCITIES ? 1 : 0) | (DYNAMIC_PHASE_EVOLUTION ? 2 : 0) |
         (DYNAMIC_SHAPE_ROTATION ? 4 : 0) | (WEAKLY_COUPLED_FILAMENTS_RPY_MOBILITY ? 8 : 0);
}

static void write_force_refs(const std::string &name, const double *v, int n) {
  std::ofstream f(name);
  f << n << std::scientific << std::setprecision(17);
  for (int i = 0; i < n; ++i) f << " " << v[i];
  f << std::endl;
}

// One swimmer of nfil x nseg prescribed filaments and nblob blobs. The
// generalised-force tables (dynamic phase / shape rotation) are written
// where mobility_solver::initialise reads them (filament.cpp:2036-2083: a
// path relative to the working directory, here a fresh directory made under
// scratch_dir and removed once they are read).
int ref_pres_setup(int nfil, int nseg, int nblob, double seg_sep, const double *blob_refs,
                   const double *body_x, const double *body_q, const double *phase_refs,
                   int n_phase_refs, const double *angle_refs, int n_angle_refs,
                   const char *scratch_dir) {
  NSWIM = 1; NFIL = nfil; NSEG = nseg; NBLOB = nblob;
  SEG_SEP = seg_sep; DL = seg_sep;
  NTOTAL = NSWIM * (NFIL * NSEG + NBLOB);
  ref_sync_var(NSWIM, NSEG, NFIL, NBLOB, 0, SEG_SEP);
  delete g_swimmers;
  g_swimmers = nullptr;
  if (g_solver) { g_solver->finalise(); delete g_solver; g_solver = nullptr; }
  std::string tmpl = std::string(scratch_dir) + "/tfs_pres_XXXXXX";
  std::vector<char> dir(tmpl.begin(), tmpl.end());
  dir.push_back('\0');
  char cwd[4096];
  if (mkdtemp(dir.data()) == nullptr || getcwd(cwd, sizeof cwd) == nullptr ||
      chdir(dir.data()) != 0)
    return -1;
  mkdir("data", 0755);
  mkdir("data/forcing", 0755);
#if DYNAMIC_PHASE_EVOLUTION
  write_force_refs(reference_phase_generalised_force_file_name(), phase_refs, n_phase_refs);
#endif
#if DYNAMIC_SHAPE_ROTATION
  write_force_refs(reference_angle_generalised_force_file_name(), angle_refs, n_angle_refs);
#endif
  g_solver = new emu_rpy_mobility_solver();
  g_solver->initialise();
  // the tables are read; remove them and the directory
#if DYNAMIC_PHASE_EVOLUTION
  unlink(reference_phase_generalised_force_file_name().c_str());
#endif
#if DYNAMIC_SHAPE_ROTATION
  unlink(reference_angle_generalised_force_file_name().c_str());
#endif
  rmdir("data/forcing");
  rmdir("data");
  if (chdir(cwd) != 0) return -1;
  rmdir(dir.data());
  g_swimmers = new std::vector<swimmer>(1);
  swimmer &s = (*g_swimmers)[0];
  s.f = matrix(6, 1);
  s.f.zero();
  s.KTMinvK_inv = matrix(6, 6);
  s.KTMinvK_inv.zero();
  rigid_body &b = s.body;
  b.blob_references.assign(blob_refs, blob_refs + 3 * nblob);
  for (int k = 0; k < 3; ++k) b.x[k] = body_x[k];
  b.q = quaternion(body_q[0], body_q[1], body_q[2], body_q[3]);
  b.qm1 = b.q;
  s.filaments = std::vector<filament>(NFIL);
  for (int i = 0; i < NFIL; ++i) {
    filament &fl = s.filaments[i];
    fl.segments = std::vector<segment>(NSEG);
    for (int j = 0; j < NSEG; ++j) fl.segments[j].x = &g_solver->x_segs_host[3 * (i * NSEG + j)];
    fl.vel_dir_phase.assign(3 * NSEG, 0.0);
    fl.phase = fl.phase_dot = fl.omega0 = 0.0;
#if DYNAMIC_SHAPE_ROTATION
    fl.vel_dir_angle.assign(3 * NSEG, 0.0);
    fl.shape_rotation_angle = fl.shape_rotation_angle_dot = 0.0;
#endif
  }
  return 0;
}

int ref_pres_system_size(void) { return g_solver->rhs.num_rows; }

// The kinematics of the current step (NULL for the arrays a build does not
// use), then read_positions_and_forces and make_precon_mat.
void ref_pres_set_kinematics(const double *x_segs, const double *vel_dir_phase,
                             const double *vel_dir_angle, const double *phase,
                             const double *omega0, const double *angle,
                             const double *phase_dot_prescribed) {
  swimmer &s = (*g_swimmers)[0];
  std::memcpy(g_solver->x_segs_host, x_segs, 8 * 3 * g_solver->ns());
  for (int i = 0; i < NFIL; ++i) {
    filament &fl = s.filaments[i];
    for (int k = 0; k < 3 * NSEG; ++k) fl.vel_dir_phase[k] = vel_dir_phase[3 * i * NSEG + k];
    fl.phase = phase[i];
    fl.omega0 = omega0[i];
#if DYNAMIC_SHAPE_ROTATION
    for (int k = 0; k < 3 * NSEG; ++k) fl.vel_dir_angle[k] = vel_dir_angle[3 * i * NSEG + k];
    fl.shape_rotation_angle = angle[i];
#endif
#if !DYNAMIC_PHASE_EVOLUTION
    fl.phase_dot = phase_dot_prescribed[i];
#endif
  }
  s.body.qm1 = s.body.q;
  s.make_precon_mat();
  g_solver->read_positions_and_forces(*g_swimmers);
}

// The unknown rates' current values (the warm start of the next solve).
void ref_pres_set_rates(const double *phase_dot, const double *angle_dot) {
  swimmer &s = (*g_swimmers)[0];
  for (int i = 0; i < NFIL; ++i) {
#if DYNAMIC_PHASE_EVOLUTION
    s.filaments[i].phase_dot = phase_dot[i];
#endif
#if DYNAMIC_SHAPE_ROTATION
    s.filaments[i].shape_rotation_angle_dot = angle_dot[i];
#endif
  }
}

// swimmer::KTMinvK_inv after make_precon_mat (6x6, column-major).
void ref_pres_ktminvk(double *out) {
  const matrix &M = (*g_swimmers)[0].KTMinvK_inv;
  for (int k = 0; k < 36; ++k) out[k] = M.data[k];
}

void ref_pres_rhs(int nt, double *rhs) {
  g_solver->assemble_rhs(*g_swimmers, nt);
  std::memcpy(rhs, g_solver->rhs.data.data(), 8 * g_solver->rhs.num_rows);
}

// which = 0: system_matrix_mult_new(in); 1: apply_preconditioner_new(in).
// (The product writes its input into the solver's force arrays, the warm
// start of the next solve, as it does in the reference.)
void ref_pres_apply(int which, const double *in, double *out) {
  const int n = g_solver->rhs.num_rows;
  matrix v(n, 1);
  std::memcpy(v.data.data(), in, 8 * n);
  const matrix r = which == 0 ? g_solver->system_matrix_mult_new(v, *g_swimmers)
                              : g_solver->apply_preconditioner_new(v, *g_swimmers);
  std::memcpy(out, r.data.data(), 8 * n);
}

// compute_velocities on the kinematics set last; the solution: segment
// forces (3 per segment), blob forces, body velocities, phase and angle
// rates. Returns the GMRES iterations.
int ref_pres_compute_velocities(int nt, double *f_segs, double *f_blobs, double *v_body,
                                double *phase_dot, double *angle_dot) {
  swimmer &s = (*g_swimmers)[0];
  int iters = 0;
  g_solver->compute_velocities(*g_swimmers, iters, nt);
  for (int n = 0; n < g_solver->ns(); ++n)
    for (int k = 0; k < 3; ++k) f_segs[3 * n + k] = g_solver->f_segs_host[6 * n + k];
  std::memcpy(f_blobs, g_solver->f_blobs_host, 8 * 3 * g_solver->nb());
  for (int k = 0; k < 6; ++k) v_body[k] = g_solver->v_bodies(k);
  for (int i = 0; i < NFIL; ++i) {
    phase_dot[i] = s.filaments[i].phase_dot;
#if DYNAMIC_SHAPE_ROTATION
    angle_dot[i] = s.filaments[i].shape_rotation_angle_dot;
#else
    angle_dot[i] = 0.0;
#endif
  }
  return iters;
}

}  // extern "C"
#endif  // PRESCRIBED_CILIA
