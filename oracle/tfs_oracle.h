/* tfs_oracle.h -- CPU restatement of the reference's RPY mobility path.
 *
 * TEST INFRASTRUCTURE ONLY. This is the checker for the CUDA library: it is
 * loaded by tests/, by __graft_entry__.smoke() and by bench.py's CPU-baseline
 * leg, and never by the product library (timfilsimmod_gb300/), which has no
 * CPU fallback.
 *
 * Every routine restates the arithmetic of one reference routine in plain
 * FP64 C; the reference file:line each follows is given beside it. Layouts
 * are the reference's AoS host layouts (rpy_mobility_solver.cu:65-71):
 *   x_segs[3*Ns], f_segs[6*Ns] (fx,fy,fz,tx,ty,tz), v_segs[6*Ns]
 *   (vx,vy,vz,wx,wy,wz), x_blobs[3*Nb], f_blobs[3*Nb], v_blobs[3*Nb].
 *
 * Targets are independent, so loops over targets run under OpenMP when the
 * caller asks for threads; each target still sums its sources in index order
 * j = 0..N-1 (cuda_functions.cu:399-457), so results do not depend on the
 * thread count.
 */
#ifndef TFS_ORACLE_H
#define TFS_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_params {
  double mu;     /* fluid viscosity (config.hpp:254 MU) */
  double a_seg;  /* segment radius (config.hpp:256 RSEG) */
  double a_blob; /* blob radius (config.hpp:257 RBLOB) */
} orc_params;

/* Number of OpenMP threads the oracle loops use (<= 0: runtime default). */
void orc_set_threads(int n);
int orc_get_threads(void);

/* One RPY pair, cuda_functions.cu:205-356 (unbounded branch). Adds into
 * V[0..vd) the velocity of particle i (radius ai) due to the force (fd = 3)
 * or force and torque (fd = 6) F on particle j (radius aj). */
void orc_rpy_pair(int vd, int fd, double *V, const double *F, double xi, double yi, double zi,
                  double ai, double xj, double yj, double zj, double aj, double mu);

/* Mss_mult, cuda_functions.cu:362-474: v_segs = M_ss f_segs (assigns). */
/* Weakly coupled filaments' segment product (Msf_mult with its filament
 * means and total forces): v_segs[6 Ns] from x_segs[3 Ns], f_segs[6 Ns],
 * Ns = nfil * nseg. */
void orc_msf(const orc_params *p, double *v_segs, const double *f_segs, const double *x_segs,
             int nfil, int nseg);
void orc_mss(const orc_params *p, double *v_segs, const double *f_segs, const double *x_segs,
             int num_segs);
/* Msb_mult, cuda_functions.cu:551-636: v_segs += M_sb f_blobs (accumulates). */
void orc_msb(const orc_params *p, double *v_segs, const double *f_blobs, const double *x_segs,
             const double *x_blobs, int num_segs, int num_blobs);
/* Mbb_mult, cuda_functions.cu:476-549: v_blobs = M_bb f_blobs (assigns). */
void orc_mbb(const orc_params *p, double *v_blobs, const double *f_blobs, const double *x_blobs,
             int num_blobs);
/* Mbs_mult, cuda_functions.cu:638-757: v_blobs = M_bs f_segs (assigns, the
 * GMRES-solver form :745-751). */
void orc_mbs(const orc_params *p, double *v_blobs, const double *f_segs, const double *x_blobs,
             const double *x_segs, int num_blobs, int num_segs);

/* General block: v[vd*i..] (= or +=) sum_j M(vd<-fd)(x_tgt[i] - x_src[j]) f_src[j]
 * for targets x_tgt (radius a_tgt) and sources x_src/f_src (radius a_src),
 * sources in index order. The four blocks above are this with the target
 * and source sets of each; it also serves target subsets (CPU baseline). */
void orc_rpy_block(const orc_params *p, int vd, int fd, double *v, const double *x_tgt, int n_tgt,
                   double a_tgt, const double *x_src, const double *f_src, int n_src,
                   double a_src, int accumulate);

/* barrier_forces, cuda_functions.cu:1240-1436 (no plane wall).
 * Adds the short-range repulsion on every segment into f_segs[0..2] of each
 * segment, and, when free_body != 0, writes the repulsion on every blob into
 * f_blobs_repulsion (assigns). end_force_magnitude is an int: the reference
 * keeps its device copy in an int (globals.hpp:14), so the caller passes the
 * truncated value. nseg is the number of segments per filament. */
void orc_barrier_forces(const orc_params *p, double *f_segs, double *f_blobs_repulsion,
                        const double *x_segs, const double *x_blobs, int num_segs, int num_blobs,
                        int nseg, int end_force_magnitude, double repulsive_force_factor,
                        int free_body);

/* flow_velocities, flow_field_evaluator.cu:13-228: Stokeslet + rotlet of the
 * segments, Stokeslet of the blobs, Blakelet image when blobs_per_body == 0,
 * optional removal of the net-force Stokeslet at each body centre; scaled by
 * prefac (the reference passes 1/(8 pi mu), :549). segs_per_body and
 * blobs_per_body are per body; there are num_bodies bodies. */
void orc_flow_velocities(double *v_flow, const double *x_flow, int num_flow, const double *f_segs,
                         const double *x_segs, int segs_per_body, const double *f_blobs,
                         const double *x_blobs, int blobs_per_body, const double *x_bodies,
                         int num_bodies, double prefac, int remove_net_force);

/* --- free-body mobility solve (tfs_oracle_solve.c) --------------------- */
typedef struct orc_solver orc_solver;
/* One swimmer: nfil x nseg segments, nblob blobs with body-frame references
 * blob_refs[3*nblob]; tol = LINEAR_SYSTEM_TOL, max_iter =
 * MAX_LINEAR_SYSTEM_ITER (capped at the system size). Body at the origin
 * with identity orientation until orc_solver_set_body. */
orc_solver *orc_solver_create(const orc_params *p, int nfil, int nseg, int nblob,
                              const double *blob_refs, int end_force_magnitude,
                              double repulsive_force_factor, double tol, int max_iter);
void orc_solver_destroy(orc_solver *s);
/* body position x[3] and orientation quaternion q = (q0, q1, q2, q3) */
void orc_solver_set_body(orc_solver *s, const double *x, const double *q);
/* mobility_solver.cpp:2950-3047 (six solves; updates the warm start) */
void orc_solver_make_body_reference_matrices(orc_solver *s, const double *x_segs,
                                             const double *f_segs);
/* compute_velocities, free-body branch (mobility_solver.cpp:2574-2659):
 * swimmer_f[6] is the swimmer's total force/torque and gets the blob
 * repulsion added, as in read_positions_and_forces. Writes v_segs[6 Ns],
 * v_blobs[3 Nb] (= M_bs f_segs, the RHS source; may be NULL); returns the
 * GMRES iteration count. The solution (blob forces, body velocity) is the
 * solver state (orc_solver_state) and the next solve's warm start. */
int orc_solver_compute_velocities(orc_solver *s, const double *x_segs, const double *f_segs,
                                  double *swimmer_f, double *v_segs, double *v_blobs);
/* GMRES on the current rhs/positions (solve_linear_system). */
int orc_solver_gmres(orc_solver *s);
void orc_solver_state(const orc_solver *s, double *f_blobs, double *v_bodies, double *body_mob,
                      double *ktkinv);
void orc_solver_set_state(orc_solver *s, const double *f_blobs, const double *v_bodies,
                          const double *body_mob, const double *ktkinv);

#ifdef __cplusplus
}
#endif

#endif /* TFS_ORACLE_H */
