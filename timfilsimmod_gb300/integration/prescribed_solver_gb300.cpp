// prescribed_solver_gb300.cpp -- the device-resident prescribed-cilia solve
// for the reference's mobility_solver (CILIA_TYPE 3). This member replaces
// the PRESCRIBED_CILIA branch of compute_velocities in the reference's
// src/cilia/mobility/mobility_solver.cpp (:2574-2596: assemble_rhs
// :282-437 and solve_linear_system :2092-2570 with apply_preconditioner_new
// :1040-1436 and system_matrix_mult_new :1806-2026), one swimmer. The
// swimmer's make_precon_mat (swimmer.cpp:1154-1322) is recomputed inside the
// library from the same kinematics. Compiled against the reference's
// unchanged headers, Real double or float; the hooks of
// rpy_mobility_solver.cu in this directory provide g_tfs_solver.
#include <algorithm>
#include <vector>

#include "mobility_solver.hpp"
#include "swimmer.hpp"
#include "tfs_shim.hpp"

#if PRESCRIBED_CILIA && !USE_BROYDEN_FOR_EVERYTHING

namespace {
bool g_prescribed_ready = false;

std::vector<double> to64(const Real *p, size_t n) { return std::vector<double>(p, p + n); }
}  // namespace

void mobility_solver::compute_velocities(std::vector<swimmer> &swimmers, int &num_gmres_iterations,
                                         const int nt) {
  swimmer &sw = swimmers[0];
  const size_t nfil = NFIL, nseg = NSEG, ns = nfil * nseg, nb = NBLOB;
  if (!g_prescribed_ready) {
    // once: the configuration, the body geometry and the generalised-force
    // tables mobility_solver::initialise read (:28-116)
    tfs_prescribed_config pc;
    const int flags = (PRESCRIBED_BODY_VELOCITIES ? TFS_PRESCRIBED_BODY : 0) |
                      (DYNAMIC_PHASE_EVOLUTION ? TFS_DYNAMIC_PHASE : 0) |
                      (DYNAMIC_SHAPE_ROTATION ? TFS_DYNAMIC_ANGLE : 0) |
                      (WEAKLY_COUPLED_FILAMENTS_RPY_MOBILITY ? TFS_WEAKLY_COUPLED : 0);
    tfs_check(tfs_prescribed_config_default(&pc, flags, NSEG, DL));
    pc.gen_force_magnitude_factor = GEN_FORCE_MAGNITUDE_FACTOR;
    pc.torsional_spring_magnitude_factor = TORSIONAL_SPRING_MAGNITUDE_FACTOR;
    const std::vector<double> refs = to64(sw.body.blob_references.data(), 3 * nb);
    tfs_check(tfs_set_blob_references(g_tfs_solver, refs.data()));
    std::vector<double> tab_p, tab_a;
#if DYNAMIC_PHASE_EVOLUTION
    tab_p.assign(gen_phase_force_refs.begin(), gen_phase_force_refs.end());
#endif
#if DYNAMIC_SHAPE_ROTATION
    tab_a.assign(gen_angle_force_refs.begin(), gen_angle_force_refs.end());
#endif
    tfs_check(tfs_prescribed_setup(g_tfs_solver, &pc, tab_p.data(), (int)tab_p.size(),
                                   tab_a.data(), (int)tab_a.size()));
    tfs_check(tfs_set_linear_solver(g_tfs_solver, LINEAR_SYSTEM_TOL,
                                    std::min(3 * NBLOB + 6, (int)MAX_LINEAR_SYSTEM_ITER)));
    g_prescribed_ready = true;
  }
  // read_positions_and_forces (:176-236): the body pose places the blobs
  const double x[3] = {sw.body.x[0], sw.body.x[1], sw.body.x[2]};
  const double q[4] = {sw.body.q.scalar_part, sw.body.q.vector_part[0], sw.body.q.vector_part[1],
                       sw.body.q.vector_part[2]};
  tfs_check(tfs_set_body_pose(g_tfs_solver, x, q));
  copy_segment_positions_to_device();
  // the filaments' kinematics (filament.hpp:97-118) as flat arrays
  std::vector<double> kphi(3 * ns), kth, phase(nfil), omega0(nfil), angle, pdot(nfil);
#if DYNAMIC_SHAPE_ROTATION
  kth.resize(3 * ns);
  angle.resize(nfil);
#endif
  for (size_t m = 0; m < nfil; ++m) {
    const filament &fl = sw.filaments[m];
    for (size_t k = 0; k < 3 * nseg; ++k) kphi[3 * nseg * m + k] = fl.vel_dir_phase[k];
    phase[m] = fl.phase;
    omega0[m] = fl.omega0;
    pdot[m] = fl.phase_dot;
#if DYNAMIC_SHAPE_ROTATION
    for (size_t k = 0; k < 3 * nseg; ++k) kth[3 * nseg * m + k] = fl.vel_dir_angle[k];
    angle[m] = fl.shape_rotation_angle;
#endif
  }
  double vb[6] = {0, 0, 0, 0, 0, 0};
#if PRESCRIBED_BODY_VELOCITIES
  Real V[3], W[3];
  sw.body.prescribed_translational_velocity(V, DT * (nt + 1.0), 0);
  sw.body.prescribed_rotational_velocity(W, DT * (nt + 1.0), 0);
  for (int k = 0; k < 3; ++k) {
    vb[k] = V[k];
    vb[3 + k] = W[k];
    v_bodies(k) = V[k];
    v_bodies(3 + k) = W[k];
  }
#else
  (void)nt;
#endif
  tfs_prescribed_kinematics kin = {kphi.data(), kth.empty() ? nullptr : kth.data(), phase.data(),
                                   omega0.data(), angle.empty() ? nullptr : angle.data(),
                                   pdot.data(), vb};
  tfs_check(tfs_prescribed_compute_velocities(g_tfs_solver, &kin, &num_gmres_iterations));
  // the solution back where the reference leaves it: segment forces (the
  // first three of six per segment), blob forces, v_bodies, the filaments'
  // rates; and in rhs, which write_data reads (:2439-2456, :3051-3060)
  std::vector<double> fs(3 * ns), fb(3 * nb), pd(nfil), ad(nfil);
  double v6[6];
  tfs_check(tfs_prescribed_solution(g_tfs_solver, fs.data(), fb.data(), v6, pd.data(), ad.data()));
  for (size_t i = 0; i < ns; ++i)
    for (int k = 0; k < 3; ++k) f_segs_host[6 * i + k] = (Real)fs[3 * i + k];
  for (size_t j = 0; j < 3 * nb; ++j) f_blobs_host[j] = (Real)fb[j];
  size_t row = 0;
  for (size_t i = 0; i < 3 * ns; ++i) rhs(row++) = (Real)fs[i];
  for (size_t j = 0; j < 3 * nb; ++j) rhs(row++) = (Real)fb[j];
#if !PRESCRIBED_BODY_VELOCITIES
  for (int k = 0; k < 6; ++k) {
    v_bodies(k) = (Real)v6[k];
    rhs(row++) = (Real)v6[k];
  }
#endif
#if DYNAMIC_PHASE_EVOLUTION
  for (size_t m = 0; m < nfil; ++m) {
    sw.filaments[m].phase_dot = (Real)pd[m];
    rhs(row++) = (Real)pd[m];
  }
#endif
#if DYNAMIC_SHAPE_ROTATION
  for (size_t m = 0; m < nfil; ++m) {
    sw.filaments[m].shape_rotation_angle_dot = (Real)ad[m];
    rhs(row++) = (Real)ad[m];
  }
#endif
}

#endif
