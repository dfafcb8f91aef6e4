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
void ref_barrier_forces(double *, double *, const double *, const double *, int, int);
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
    ref_barrier_forces(fs_d.data(), frep_d.data(), xs_d.data(), xb_d.data(), ns(), nb());
  }
  void wait_for_device() override {}
  void evaluate_segment_segment_mobility() override { ref_mss(vs_d.data(), fs_d.data(), xs_d.data(), ns()); }
  void evaluate_segment_blob_mobility() override {
    ref_msb(vs_d.data(), fb_d.data(), xs_d.data(), xb_d.data(), ns());
  }
  void evaluate_blob_blob_mobility() override { ref_mbb(vb_d.data(), fb_d.data(), xb_d.data(), nb()); }
  void evaluate_blob_segment_mobility() override {
    ref_mbs(vb_d.data(), fs_d.data(), xb_d.data(), xs_d.data(), nb());
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
