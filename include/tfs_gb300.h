/* tfs_gb300.h -- C ABI of libtfs_gb300.so, the GB300 (sm_103a) implementation
 * of the reference's RPY mobility path.
 *
 * The reference exposes this path as the C++ class `rpy_mobility_solver`
 * (src/cilia/mobility/rpy_mobility_solver.hpp:15-64), which implements the 17
 * pure-virtual device hooks of `mobility_solver`
 * (src/cilia/mobility/mobility_solver.hpp:26-46). Each hook has one entry
 * point here, taking an opaque solver handle; a replacement
 * rpy_mobility_solver.cu calls them one to one.
 * Host arrays keep the reference's AoS float64 layouts
 * (rpy_mobility_solver.cu:65-71):
 *   x_segs[3*Ns]  f_segs[6*Ns] (fx,fy,fz,tx,ty,tz)  v_segs[6*Ns] (vx,vy,vz,wx,wy,wz)
 *   x_blobs[3*Nb] f_blobs[3*Nb]                      v_blobs[3*Nb]
 *   f_blobs_repulsion[3*Nb]
 * with Ns = NSWIM*NFIL*NSEG and Nb = NSWIM*NBLOB.
 *
 * Every call returns 0 (TFS_OK) or a negative TFS_E* status; no exception or
 * abort crosses the ABI. tfs_last_error() gives a message for the calling
 * thread's most recent failure. Copies and kernels are asynchronous on the
 * solver's stream; tfs_wait_for_device() is the synchronisation point, as
 * `wait_for_device` is in the reference (rpy_mobility_solver.cu:247-256).
 * Host buffers passed to the copy calls must stay valid until then (pinned
 * memory gives asynchronous copies; pageable memory also works).
 */
#ifndef TFS_GB300_H
#define TFS_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TFS_OK 0
#define TFS_EINVAL (-1)   /* bad argument or size */
#define TFS_ENOMEM (-2)   /* device allocation failed */
#define TFS_ECUDA (-3)    /* CUDA runtime error (message has the CUDA text) */
#define TFS_ENOTCONV (-4) /* iterative solve hit its iteration cap */
#define TFS_ENAN (-5)     /* non-finite value in a solve */
#define TFS_ETIMEOUT (-6) /* bounded wait expired */
#define TFS_ESTATE (-7)   /* call out of order (e.g. data not set) */

/* Arithmetic of the pairwise sums. */
#define TFS_FP64 0        /* plain FP64 (the parity drop-in) */
#define TFS_FP32C 1       /* FP32 pairs, compensated (two-sum) accumulation */

typedef struct tfs_solver tfs_solver; /* opaque */

/* Sizes and physical constants. The reference takes these from config.hpp
 * macros and globals.ini (config.hpp:254-257, cilia_sim_main.cu:56-87);
 * here they are run-time values. */
typedef struct tfs_config {
  int nswim;                 /* swimmers (NSWIM) */
  int nfil;                  /* filaments per swimmer (NFIL) */
  int nseg;                  /* segments per filament (NSEG) */
  int nblob;                 /* blobs per swimmer (NBLOB) */
  double mu;                 /* viscosity (MU) */
  double a_seg;              /* segment radius (RSEG) */
  double a_blob;             /* blob radius (RBLOB) */
  int end_force_magnitude;   /* device copy of END_FORCE_MAGNITUDE: an int in the
                                reference (globals.hpp:14, sync_var) */
  double repulsive_force_factor; /* REPULSIVE_FORCE_FACTOR (config.hpp:404) */
  int free_body;             /* !PRESCRIBED_BODY_VELOCITIES: barrier forces on blobs */
  int precision;             /* TFS_FP64 or TFS_FP32C */
} tfs_config;

/* Fill *cfg with the reference's defaults for the elastic-filament, free-body
 * RPY configuration (MU = RSEG = RBLOB = 1, REPULSIVE_FORCE_FACTOR = 2,
 * free body, FP64) and the given sizes. */
int tfs_config_default(tfs_config *cfg, int nswim, int nfil, int nseg, int nblob);

/* allocate_host_memory + allocate_device_memory
 * (rpy_mobility_solver.cu:54-117). Uses the current CUDA device. Host arrays
 * stay owned by the caller. */
int tfs_solver_create(const tfs_config *cfg, tfs_solver **out);
/* free_host_memory + free_device_memory (rpy_mobility_solver.cu:14-52). */
int tfs_solver_destroy(tfs_solver *s);

/* Run the solver's work on `stream` (a cudaStream_t; NULL = the solver's own
 * non-blocking stream). */
int tfs_solver_set_stream(tfs_solver *s, void *stream);
/* Change the pairwise-sum arithmetic (TFS_FP64 / TFS_FP32C). */
int tfs_solver_set_precision(tfs_solver *s, int precision);

/* Device buffers of the solver (AoS float64), for callers that keep data
 * resident in HBM instead of going through the host copy hooks. */
typedef struct tfs_device_buffers {
  double *x_segs, *f_segs, *v_segs;
  double *x_blobs, *f_blobs, *v_blobs, *f_blobs_repulsion;
} tfs_device_buffers;
int tfs_solver_device_buffers(tfs_solver *s, tfs_device_buffers *out);
/* Tell the solver that positions in its device buffers were written directly
 * (the copy hooks do this themselves). */
int tfs_solver_positions_updated(tfs_solver *s);

/* --- the 17 hooks of mobility_solver.hpp:26-46 ------------------------- */
int tfs_copy_segment_positions_to_device(tfs_solver *s, const double *x_segs_host);   /* rpy_mobility_solver.cu:119-128 */
int tfs_copy_segment_forces_to_device(tfs_solver *s, const double *f_segs_host);      /* :130-139 */
int tfs_copy_blob_positions_to_device(tfs_solver *s, const double *x_blobs_host);     /* :141-150 */
int tfs_copy_blob_forces_to_device(tfs_solver *s, const double *f_blobs_host);        /* :152-161 */
int tfs_copy_interparticle_blob_forces_to_host(tfs_solver *s, double *f_blobs_repulsion_host); /* :163-175 */
int tfs_copy_blob_velocities_to_host(tfs_solver *s, double *v_blobs_host);           /* :177-189 */
int tfs_copy_segment_velocities_to_host(tfs_solver *s, double *v_segs_host);         /* :191-205 */
/* The same seven copies for host arrays of float, the reference's Real in its
 * shipped configuration (config.hpp:53, FIL_USE_DOUBLE_PRECISION false;
 * rpy_mobility_solver.cu:54-71 allocates Real host arrays): the floats cross
 * the bus as floats and are converted to or from the solver's float64
 * device arrays on the device, on the solver's stream (a float staging
 * buffer of the largest array is allocated on the first such call). */
int tfs_copy_segment_positions_to_device_f32(tfs_solver *s, const float *x_segs_host);
int tfs_copy_segment_forces_to_device_f32(tfs_solver *s, const float *f_segs_host);
int tfs_copy_blob_positions_to_device_f32(tfs_solver *s, const float *x_blobs_host);
int tfs_copy_blob_forces_to_device_f32(tfs_solver *s, const float *f_blobs_host);
int tfs_copy_interparticle_blob_forces_to_host_f32(tfs_solver *s, float *f_blobs_repulsion_host);
int tfs_copy_blob_velocities_to_host_f32(tfs_solver *s, float *v_blobs_host);
int tfs_copy_segment_velocities_to_host_f32(tfs_solver *s, float *v_segs_host);
/* barrier_forces: adds segment repulsion into the device f_segs and writes
 * the blob repulsion (free body) (rpy_mobility_solver.cu:207-245,
 * cuda_functions.cu:1240-1436). */
int tfs_apply_interparticle_forces(tfs_solver *s);
int tfs_wait_for_device(tfs_solver *s);                                              /* :247-256 */
int tfs_evaluate_segment_segment_mobility(tfs_solver *s); /* v_segs  = Mss f_segs  (:258-274, cuda_functions.cu:362-474) */
int tfs_evaluate_segment_blob_mobility(tfs_solver *s);    /* v_segs += Msb f_blobs (:276-292, :551-636) */
int tfs_evaluate_blob_blob_mobility(tfs_solver *s);       /* v_blobs = Mbb f_blobs (:294-310, :476-549) */
int tfs_evaluate_blob_segment_mobility(tfs_solver *s);    /* v_blobs = Mbs f_segs  (:312-328, :638-757) */
/* The weakly coupled filaments' segment-segment product of the reference's
 * weakly_coupled_filaments_rpy_mobility_solver (its position and force
 * uploads compute each filament's mean position and total force,
 * weakly_coupled_filaments_rpy_mobility_solver.cu:50-89; its
 * evaluate_segment_segment_mobility runs Msf_mult, cuda_functions.cu:
 * 1129-1229, free space): v_segs from x_segs and f_segs -- full RPY
 * (translation only) within a filament, the Stokeslet of every other
 * filament's total force at its mean position; rotational velocities zero.
 * FP64 whatever the solver's precision. The segments must form whole
 * filaments of nseg. */
int tfs_evaluate_weakly_coupled_segment_mobility(tfs_solver *s);
/* v_blobs = Mbb f_blobs in float-float arithmetic (each pair quantity an
 * unevaluated sum of two FP32 numbers, about 1e-13 relative), whatever the
 * solver's precision: the product FP32C refinement computes its residuals
 * with. No counterpart in the reference. */
int tfs_evaluate_blob_blob_mobility_ff(tfs_solver *s);
/* evaluate_full_mobility (rpy_mobility_solver.cu:330-337): Mss + Msb into
 * v_segs and Mbb, then Mbs into v_blobs -- the reference's sequence assigns
 * v_blobs twice, so v_blobs ends as Mbs f_segs; this entry reproduces that.
 * Segment and blob velocities are copied to the given host arrays when they
 * are non-NULL. */
int tfs_evaluate_full_mobility(tfs_solver *s, double *v_segs_host, double *v_blobs_host);

/* --- fused forms (no reference counterpart; same arithmetic) ------------ */
/* One launch per target kind: v_segs = Mss f_segs + Msb f_blobs and
 * v_blobs = Mbs f_segs + Mbb f_blobs, i.e. the whole grand mobility applied
 * to [f_segs; f_blobs]. */
int tfs_apply_grand_mobility(tfs_solver *s);

/* --- the free-body mobility solve (one swimmer per solver, nswim = 1) ---- */
/* The body's blob references in the body frame (rigid_body::blob_references,
 * rigid_body.cpp:325-365), 3*nblob values. Required before the calls below. */
int tfs_set_blob_references(tfs_solver *s, const double *blob_refs_host);
/* Body position x[3] and orientation quaternion q[4] = (q0, q1, q2, q3)
 * (rigid_body::x, q; q may be NULL to keep the orientation). Computes the blob
 * positions on the device (rigid_body::blob_positions, rigid_body.cpp:482-500). */
int tfs_set_body_pose(tfs_solver *s, const double *x, const double *q);
/* LINEAR_SYSTEM_TOL and MAX_LINEAR_SYSTEM_ITER (config.hpp:312-313); the
 * defaults are the reference's 1e-4 and min(350, 3 nblob + 6). */
int tfs_set_linear_solver(tfs_solver *s, double tol, int max_iter);
/* TFS_FP32C only: the linear solve is iterative refinement -- FP64 residuals
 * r = rhs - A x around inner GMRES solves with FP32 blob-blob products, each
 * to inner_tol relative to |r|, at most max_cycles cycles. */
int tfs_set_refinement(tfs_solver *s, double inner_tol, int max_cycles);
/* TFS_FP32C only: the Arnoldi vectors of the cooperative inner solves.
 * TFS_VECTORS_FP32 (the default): FP32 vectors; a refinement that stalls is
 * run again from the warm start with FP64 ones. TFS_VECTORS_FP64: FP64
 * vectors for every solve (a few percent fewer Arnoldi steps, each slower:
 * medium swimmer's implicit steps at DT 0.121, 15.5 against 14.1 ms). The
 * inner solves of tfs_make_body_reference_matrices take FP64 vectors in
 * either mode. */
#define TFS_VECTORS_FP32 0
#define TFS_VECTORS_FP64 1
int tfs_set_refinement_vectors(tfs_solver *s, int mode);
/* FP32C only: run each inner GMRES solve of the refinement as one
 * cooperative kernel (enable = 1, the default where the device supports
 * cooperative launch and the system has at most 64 blobs per SM pair of
 * CTAs) or as a sequence of kernels per Arnoldi step (enable = 0). Both
 * compute the same iteration; the cooperative kernel removes the launch
 * gaps between its phases. TFS_ESTATE if enable = 1 cannot be honoured. */
int tfs_set_persistent_gmres(tfs_solver *s, int enable);
/* Fault injection on the host, for tests of the bounded waits (no reference
 * counterpart): with on = 1 the grid barriers of this solver's cooperative
 * inner GMRES wait for one arrival more than the launch has CTAs, so every
 * wait runs out its bound (2 s); the kernel then ends with an error status
 * and the solve returns TFS_ETIMEOUT, leaving the device usable. on = 0
 * (the default) restores normal solves. */
int tfs_inject_barrier_stall(tfs_solver *s, int on);
/* make_body_reference_matrices (mobility_solver.cpp:2950-3047): (K^T K)^-1
 * from the blob references and the 6x6 body mobility from six solves with
 * rhs = -e_{n-1-j}, at the current pose. Leaves the last solution as the next
 * warm start, as the reference does. */
int tfs_make_body_reference_matrices(tfs_solver *s);
/* The two 6x6 matrices (column-major, body frame); either pointer may be NULL. */
int tfs_get_body_reference_matrices(tfs_solver *s, double *body_mobility, double *ktkinv);
int tfs_set_body_reference_matrices(tfs_solver *s, const double *body_mobility,
                                    const double *ktkinv);
/* compute_velocities, free-body branch (mobility_solver.cpp:2574-2659) on the
 * segment positions and forces already on the device: barrier forces, Mss and
 * Mbs, the right-hand side [-v_blobs; -F] with F = swimmer_f[6] (the swimmer's
 * total force and torque, swimmer::forces_and_torques) plus the blob
 * repulsion, the GMRES solve for blob forces and body velocity (warm-started
 * from the previous solution), and Msb with the solved blob forces. On return
 * swimmer_f holds F with the blob repulsion added, as the reference leaves
 * swimmer.f; segment velocities, blob forces and body velocity are on the
 * device (tfs_copy_segment_velocities_to_host, tfs_copy_blob_forces_to_host,
 * tfs_get_body_velocities). Synchronises the solver's stream. */
int tfs_compute_velocities(tfs_solver *s, double *swimmer_f, int *gmres_iters);
/* The linear solve alone (solve_linear_system, mobility_solver.cpp:2092-2570)
 * for a right-hand side rhs_host[3 nblob + 6]. */
int tfs_solve_linear_system(tfs_solver *s, const double *rhs_host, int *gmres_iters);
int tfs_get_body_velocities(tfs_solver *s, double *v_bodies);
/* Warm start of the next solve (the reference keeps v_bodies between solves). */
int tfs_set_body_velocities(tfs_solver *s, const double *v_bodies);
/* The solved blob forces (f_blobs_host after the reference's GMRES). */
int tfs_copy_blob_forces_to_host(tfs_solver *s, double *f_blobs_host);
int tfs_copy_blob_forces_to_host_f32(tfs_solver *s, float *f_blobs_host);
/* Iterations (summed over refinement cycles), refinement cycles and final
 * relative residual of the last solve. FP32C: the cooperative inner solves
 * keep their Arnoldi vectors in FP32 (FP64 during
 * tfs_make_body_reference_matrices, or under TFS_VECTORS_FP64). A refinement cycle that does not reduce
 * the FP64 residual ends the refinement; it is run again from the caller's
 * warm start with FP64 Arnoldi vectors, and if that stalls too the solve
 * finishes as plain FP64 GMRES from the warm start; cycles is then negative
 * (minus the cycles run before). */
int tfs_solve_info(tfs_solver *s, int *iters, int *cycles, double *rel_residual);
/* FP32C refinements of this solver rerun with FP64 Arnoldi vectors after a
 * stall (a count over the solver's life). */
int tfs_refinement_retries(tfs_solver *s, long long *retries);

/* --- prescribed-cilia solve ---------------------------------------------- */
/* The reference's mobility solve for filaments that follow a prescribed
 * sequence of shapes (CILIA_TYPE 3): compute_velocities under
 * PRESCRIBED_CILIA (mobility_solver.cpp:2574-2596) with assemble_rhs
 * (:282-437), solve_linear_system (:2092-2570), apply_preconditioner_new
 * (:1040-1436), system_matrix_mult_new (:1806-2026) and
 * swimmer::make_precon_mat (swimmer.cpp:1154-1322), for one swimmer, FP64.
 * Unknowns (reference order): segment forces (3 Ns), blob forces (3 Nb), body
 * velocity and angular velocity (6, free body), phase rates (nfil, dynamic
 * phase), shape-rotation rates (nfil, dynamic shape rotation). Segment
 * positions come through tfs_copy_segment_positions_to_device, the body
 * through tfs_set_blob_references and tfs_set_body_pose; the GMRES tolerance
 * through tfs_set_linear_solver (the iteration cap is the reference's
 * MAX_LINEAR_SYSTEM_ITER, min(350, unknowns)). After tfs_prescribed_setup the
 * four block hooks (tfs_evaluate_*_mobility) take the form of the reference's
 * kernels under PRESCRIBED_CILIA (cuda_functions.cu:362-757): 3x3 pairs on
 * the forces only (segment torques are not read), zero rotational segment
 * velocities, and blob <- segment adding to blob <- blob. */
#define TFS_PRESCRIBED_BODY 1 /* PRESCRIBED_BODY_VELOCITIES: the body moves as given */
#define TFS_DYNAMIC_PHASE 2   /* DYNAMIC_PHASE_EVOLUTION: phase rates are unknowns */
#define TFS_DYNAMIC_ANGLE 4   /* DYNAMIC_SHAPE_ROTATION: shape-rotation rates are unknowns */
#define TFS_WEAKLY_COUPLED 8  /* WEAKLY_COUPLED_FILAMENTS_RPY_MOBILITY: Msf_mult for the
                                 segment block (cuda_functions.cu:1129-1229) */
typedef struct tfs_prescribed_config {
  int flags;                                /* TFS_PRESCRIBED_BODY | ... */
  double gen_force_magnitude_factor;        /* GEN_FORCE_MAGNITUDE_FACTOR (globals) */
  double torsional_spring_magnitude_factor; /* TORSIONAL_SPRING_MAGNITUDE_FACTOR */
  double fil_length;                        /* FIL_LENGTH = DL (NSEG - 1), config.hpp:515-517 */
} tfs_prescribed_config;
/* Defaults: factors 1 and 2 (globals.ini), fil_length = dl (nseg - 1). */
int tfs_prescribed_config_default(tfs_prescribed_config *pc, int flags, int nseg, double dl);
/* Allocates the solve for the solver's sizes (nswim = 1; the blob references
 * must be set). The generalised-force tables over one period (the reference
 * reads them in mobility_solver::initialise, :28-116) are needed with the
 * dynamic phase / shape rotation flags. A free body takes both dynamic flags
 * or neither: the reference's free-body preconditioner indexes both. The
 * solution (warm start) starts at zero. */
int tfs_prescribed_setup(tfs_solver *s, const tfs_prescribed_config *pc,
                         const double *phase_force_refs, int n_phase_refs,
                         const double *angle_force_refs, int n_angle_refs);
/* The filaments' state for one solve (the fields of filament.hpp the solve
 * reads); arrays a configuration does not use may be NULL. */
typedef struct tfs_prescribed_kinematics {
  const double *vel_dir_phase;        /* 3 Ns: d x / d phase of every segment */
  const double *vel_dir_angle;        /* 3 Ns: d x / d angle (dynamic shape rotation) */
  const double *phase;                /* nfil (dynamic phase or shape rotation) */
  const double *omega0;               /* nfil natural frequencies (idem) */
  const double *shape_rotation_angle; /* nfil (dynamic shape rotation) */
  const double *phase_dot;            /* nfil prescribed rates (without dynamic phase) */
  const double *v_body;               /* 6: prescribed body velocities; NULL = zero, as
                                         rigid_body.cpp:584-598 */
} tfs_prescribed_kinematics;
/* Uploads the kinematics and computes the per-filament constants and (free
 * body) the inverse body block, swimmer.KTMinvK_inv, on the current segment
 * positions and body pose. Synchronises the solver's stream. */
int tfs_prescribed_set_kinematics(tfs_solver *s, const tfs_prescribed_kinematics *k);
/* assemble_rhs and the GMRES solve on the kinematics set last, warm started
 * from the previous solution. FP32C: inner solves on FP32 pair sums (FP64
 * Krylov vectors), each to max(1e-7, tol ||b|| / (2 ||r||)), refined on
 * float-float (equal radii, RPY) or FP64 residuals until the FP64 relative
 * residual meets the tolerance; tfs_solve_info reports the inner steps and
 * cycles. Synchronises the solver's stream. */
int tfs_prescribed_solve(tfs_solver *s, int *gmres_iters);
/* tfs_prescribed_set_kinematics, then tfs_prescribed_solve. */
int tfs_prescribed_compute_velocities(tfs_solver *s, const tfs_prescribed_kinematics *k,
                                      int *gmres_iters);
/* One piece on host vectors of tfs_prescribed_size entries: which = 0 the
 * operator A in, 1 the preconditioner P^-1 in, 2 the right-hand side (in
 * unused). */
int tfs_prescribed_apply(tfs_solver *s, int which, const double *in, double *out);
int tfs_prescribed_size(tfs_solver *s, int *n);
/* The inverse body block (6 x 6, column-major) of the kinematics set last. */
int tfs_prescribed_precon_matrix(tfs_solver *s, double *m36);
/* The solution of the last solve, which is also the next solve's warm start:
 * segment forces (3 Ns), blob forces (3 Nb), body velocities (6), phase and
 * angle rates (nfil each); NULL skips a part, absent parts read as zero. */
int tfs_prescribed_solution(tfs_solver *s, double *f_segs, double *f_blobs, double *v_body,
                            double *phase_dot, double *angle_dot);
int tfs_prescribed_set_solution(tfs_solver *s, const double *f_segs, const double *f_blobs,
                                const double *v_body, const double *phase_dot,
                                const double *angle_dot);

/* --- autotuning ---------------------------------------------------------- */
/* Products run as work-queue launches: one persistent grid whose CTAs take
 * (target block, source chunk) units of every product of the launch from a
 * device counter, with the source-split sums added in chunk order inside the
 * same launch. The launch variant (threads per CTA, targets per thread,
 * sources per tile, register cap) changes the speed, never the result: the
 * chunking depends on the system's sizes only.
 * Autotune times every queue variant for each product kind the solver has
 * (M_ss, M_bs, both at once, M_sb, M_bb, the grand mobility) and every
 * variant and source-split target of the tile kernel for the blob-blob
 * product of the kernel-sequence GMRES, on the current positions and forces,
 * and keeps the fastest of each. precision_mask: bit 0 = TFS_FP64, bit 1 =
 * TFS_FP32C. reps: timed launches per candidate. Overwrites the solver's
 * velocity buffers. Synchronises the solver's stream. */
int tfs_solver_autotune(tfs_solver *s, int precision_mask, int reps);
/* Pin the work-queue variant of one product kind: kind 0..5 = M_ss, M_bs,
 * M_ss with M_bs, M_sb, M_bb, grand mobility; variant in
 * [0, tfs_num_queue_variants(precision)). */
int tfs_solver_set_queue_variant(tfs_solver *s, int precision, int kind, int variant);
int tfs_num_queue_variants(int precision);
/* Pin the launch of one combination: combo 0..5 = seg<-seg, seg<-blob,
 * blob<-blob, blob<-seg, seg<-(seg,blob), blob<-(seg,blob); variant in
 * [0, tfs_num_tile_variants(precision)); waves in [1, 64] (the source split
 * aims for this many full waves of resident CTAs). */
int tfs_solver_set_tuning(tfs_solver *s, int precision, int combo, int variant, int waves);
int tfs_num_tile_variants(int precision);
/* The tuning table of the last autotune as JSON (NUL-terminated, truncated to
 * len); *needed (if non-NULL) gets the full size including the NUL. */
int tfs_solver_tuning_report(tfs_solver *s, char *buf, size_t len, size_t *needed);

/* --- implicit time step -------------------------------------------------- */
/* The reference's time step for one free swimmer with elastic filaments
 * (CILIA_TYPE 0: filaments tethered and clamped to the body, an end force
 * along the distal tangent), driven through this solver's mobility solve:
 * the loop body of src/cilia/cilia_sim_main.cu:355-527 -- initial guess
 * (swimmer::initial_guess, swimmer.cpp:433-467), internal forces
 * (filament::internal_forces_and_torques, filament.cpp:1467-1575;
 * swimmer::forces_and_torques, swimmer.cpp:469-533), compute_velocities, the
 * BDF residuals (mobility_solver::compute_errors, mobility_solver.cpp:2661-2946)
 * and Broyden's method (broyden_solver.cpp:21-129) with the approximate
 * inverse Jacobian (filament::invert_approx_jacobian, filament.cpp:1761-1894;
 * swimmer::prepare_jacobian_inv and jacobian_inv_mult, swimmer.cpp:535-1070).
 * Segments, filaments and the Broyden matrices live on the device; the
 * body's 6 degrees of freedom and its 6x6 Schur complement on the host.
 * The solver must have its blob references and body reference matrices set
 * (tfs_make_body_reference_matrices) before the first step. */
typedef struct tfs_stepper tfs_stepper; /* opaque */
typedef struct tfs_step_config {
  int nfil, nseg;              /* must match the solver's */
  double seg_sep;              /* DL (SEG_SEP, config.hpp:259) */
  double dt;                   /* DT */
  double tol;                  /* TOL of Broyden's method (config.hpp:302) */
  int max_broyden_iter;        /* MAX_BROYDEN_ITER (config.hpp:301) */
  double kb, kt;               /* bending and twisting moduli KB, KT */
  double end_force_magnitude;  /* END_FORCE_MAGNITUDE (the real value) */
  double jacobian_confidence;  /* JACOBIAN_CONFIDENCE_FACTOR (config.hpp:299) */
  double body_radius;          /* 0.5 AXIS_DIR_BODY_LENGTH of the spherical body */
  int perturb_first_step;      /* CILIA_IC_TYPE 0 perturbation at step 0 (filament.cpp:520-528) */
  double body_x[3];            /* initial body position */
  double body_q[4];            /* initial body orientation (scalar first) */
} tfs_step_config;
/* Defaults: DL 2.2, DT 36.3833/300, TOL 1e-4, 400 iterations, KB = KT = 1800,
 * END_FORCE_MAGNITUDE = 220 KB/(2.6 NSEG)^2, confidence 0.1, body radius 1,
 * perturbation on, body at the origin with identity orientation. */
int tfs_step_config_default(tfs_step_config *cfg, int nfil, int nseg);
/* Straight filaments along fil_dirs[3 nfil] from the bases X + R fil_refs
 * (fil_refs[3 nfil] in the body frame), at rest (filament::initial_setup,
 * filament.cpp:219-346). Segment positions live in the solver's x_segs. */
int tfs_stepper_create(tfs_solver *s, const tfs_step_config *cfg, const double *fil_refs,
                       const double *fil_dirs, tfs_stepper **out);
int tfs_stepper_destroy(tfs_stepper *st);
/* One whole step nt (0-based): returns TFS_OK when Broyden's method met TOL,
 * TFS_ENOTCONV when it stopped at max_broyden_iter (the state is advanced as
 * the reference leaves it), TFS_ENAN if the residual went non-finite. */
int tfs_stepper_step(tfs_stepper *st, int nt, int *broyden_iters, int *gmres_iters);
/* The stages of a step, in the order tfs_stepper_step runs them. */
int tfs_stepper_initial_guess(tfs_stepper *st, int nt);
/* Internal forces into f_segs; swimmer_f[6] (may be NULL) gets swimmer::f. */
int tfs_stepper_forces(tfs_stepper *st, int nt, double *swimmer_f);
int tfs_stepper_compute_velocities(tfs_stepper *st, int nt, int *gmres_iters);
/* Residuals into Broyden's error (which = 0) or new_error (which = 1);
 * err (may be NULL) gets a copy, 6 (NFIL NSEG + 1) values. */
int tfs_stepper_compute_errors(tfs_stepper *st, int nt, int which, double *err, int *too_large);
/* schur_inv (may be NULL): the inverted 6x6 Schur complement, column-major. */
int tfs_stepper_prepare_jacobian_inv(tfs_stepper *st, int nt, double *schur_inv);
/* Filament fil's inverse approximate Jacobian, (6 NSEG)^2 column-major. */
int tfs_stepper_inverse_jacobian(tfs_stepper *st, int fil, double *out);
int tfs_stepper_jacobian_inv_mult(tfs_stepper *st, int nt, const double *in, double *out);
int tfs_stepper_broyden_reset(tfs_stepper *st);
/* update (may be NULL) gets broyden.update. */
int tfs_stepper_find_update(tfs_stepper *st, int nt, double *update);
/* swimmer::update with the last update, then the internal forces. */
int tfs_stepper_apply_update(tfs_stepper *st, int nt);
int tfs_stepper_end_of_iter(tfs_stepper *st, int nt, int too_large);
/* Back to the straight start of tfs_stepper_create (state, histories,
 * Broyden memory, and the solver's warm start as it was at creation), with
 * each segment first turned by exp(seg_rotation[3 j..3 j+2]) when
 * seg_rotation (3 Ns values) is not NULL; positions then follow from the
 * robot arm (filament.cpp:625-647). The next step is step 0. */
int tfs_stepper_reset(tfs_stepper *st, const double *seg_rotation);
/* The state (any pointer may be NULL): x[3 Ns], q[4 Ns], u[3 Ns] per
 * segment; lambda[3 (NSEG-1) NFIL], tether[3 NFIL], clamp[3 NFIL]; the body's
 * x[3], q[4], u[3]. */
int tfs_stepper_state(tfs_stepper *st, double *x, double *q, double *u, double *lambda,
                      double *tether, double *clamp, double *body_x, double *body_q,
                      double *body_u);

/* --- the reference's data files for the step -------------------------- */
/* The backup record of the swimmer (swimmer::write_backup: per filament
 * 9 + 28 NSEG numbers, then 19 for the body; filament.cpp:1952-2037,
 * rigid_body.cpp:556-579) as doubles, its size, and restoring one (as the
 * reference reads a backup, filament.cpp:140-215: q^{n-1} = q; Broyden's
 * memory cleared; the solver's warm start as at creation). */
int tfs_stepper_backup_size(tfs_stepper *st, size_t *n);
int tfs_stepper_get_backup(tfs_stepper *st, double *values);
int tfs_stepper_set_backup(tfs_stepper *st, const double *values);
/* The reference's text files, formatted as its streams write them
 * (std::scientific, 10 digits): the backup "<save_step> <values...>"
 * (cilia_sim_main.cu:590-597), overwritten; reading one checks the count
 * and restores it (*save_step = the step to run next,
 * cilia_sim_main.cu:336-350). */
int tfs_stepper_write_backup(tfs_stepper *st, int save_step, const char *path);
int tfs_stepper_read_backup(tfs_stepper *st, const char *path, int *save_step);
/* A plot step after step nt (cilia_sim_main.cu:563-600): appends one record
 * to <prefix>_seg_states.dat, _body_states.dat, _tether_force.dat (step
 * nt+1) and, as mobility_solver::write_data (mobility_solver.cpp:3051-3173),
 * to _body_vels.dat, _blob_forces.dat, _seg_vels.dat, _seg_forces.dat (step
 * nt; segment forces before barrier forces, as the reference's host copy);
 * backup != 0 also writes <prefix>.backup. */
int tfs_stepper_write_files(tfs_stepper *st, int nt, const char *prefix, int backup);

/* --- many swimmers: batches and a request server ---------------------- */
/* No counterpart in the reference (one swimmer set per process). Each
 * swimmer is an instance -- its own tfs_solver and tfs_stepper on its own
 * stream -- and a pool of host worker threads runs the instances' step
 * pipelines so that their kernels overlap on the GPU. Instances share
 * no state on the device: a swimmer's result is the same alone (a batch of
 * one) and in a batch. The inner GMRES solves of FP32C instances can run
 * in shared cooperative launches of the persistent kernel (in the server,
 * and in a batch unless tfs_batch_share_inner_solves says otherwise): a solve
 * waiting for
 * the GPU is gathered with the others waiting (up to the SM count of CTAs),
 * each on a fixed number of CTAs chosen from its own blob count (about one
 * per 64 blobs), so its arithmetic does not depend on the others. FP32C
 * swimmers the persistent kernel cannot take, and FP64 swimmers, solve on
 * their own with the kernel sequence.
 * The pair products of every instance (M_ss with M_bs, M_sb, ...) run in
 * shared work-queue launches (in the server, and in a batch unless
 * tfs_batch_share_products says otherwise): products waiting while the
 * previous shared launch runs are gathered (those of one precision and
 * source set, up to 256 jobs) into one persistent launch whose CTAs take
 * the (target block, source chunk) units of all of them from one counter.
 * Each product keeps its own chunking, partial sums and ordered reduction,
 * so its result is the same, bit for bit, alone and shared. */
typedef struct tfs_batch tfs_batch;
int tfs_batch_create(int num_workers, tfs_batch **out);
int tfs_batch_destroy(tfs_batch *b);   /* does not destroy the instances */
/* Adds a swimmer (its stepper; the solver comes with it). */
int tfs_batch_add(tfs_batch *b, tfs_stepper *st, int *index);
int tfs_batch_size(tfs_batch *b, int *n);
/* Step nt of every swimmer. The per-swimmer arrays (any may be NULL) get
 * Broyden and GMRES iterations and the step's status; the return value is
 * TFS_OK or the first failing swimmer's status (the others still step). */
int tfs_batch_step(tfs_batch *b, int nt, int *broyden_iters, int *gmres_iters, int *status);
/* Which FP32C swimmers share launches: those whose solve takes at most
 * max_ctas CTAs there (one per 64 blobs); the others solve on their own with
 * the kernel sequence, as FP64 swimmers do. 0: none; < 0 (the default): all
 * (measured on 64 uneven swimmers: 1890 swimmer-steps/s sharing all, 1588
 * sharing none). */
int tfs_batch_share_inner_solves(tfs_batch *b, int max_ctas);
/* Inner solves run in shared launches so far, and those launches. */
int tfs_batch_shared_solves(tfs_batch *b, long long *launches, long long *solves);
/* Whether the batch's products share work-queue launches (default 1), and
 * the shared launches and the products they carried so far. */
int tfs_batch_share_products(tfs_batch *b, int enable);
int tfs_batch_shared_products(tfs_batch *b, long long *launches, long long *products);

/* A request: num_steps implicit steps (0 .. num_steps-1) of a swimmer
 * given by its geometry (blob references, filament bases and directions;
 * all arrays must stay valid until the request completes) from the
 * straight start, each segment turned by seg_rotation (3 Ns, may be NULL)
 * as in tfs_stepper_reset. Results: x_out[3 Ns] segment positions,
 * body_out[7] = body x, q and q_out[4 Ns] segment orientations (any may be
 * NULL). */
typedef struct tfs_request {
  int nfil, nseg, nblob;
  const double *blob_refs, *fil_refs, *fil_dirs;
  double body_radius;         /* 0: the server's step setting */
  const double *seg_rotation;
  int num_steps;
  double *x_out, *body_out;
  double *q_out;
} tfs_request;
typedef struct tfs_server_config {
  int num_workers;            /* requests in flight at once */
  size_t hbm_budget_bytes;    /* device memory for resident instances */
  int precision;              /* TFS_FP64 or TFS_FP32C */
  double linear_tol;          /* LINEAR_SYSTEM_TOL of every solve */
  tfs_step_config step;       /* step settings (nfil, nseg come from each request) */
  double max_bypass_ms;       /* age bound of admission past a waiting request (below) */
} tfs_server_config;
typedef struct tfs_server_counters {
  long long resident_instances, created, reused, evicted, queued, inflight;
  size_t bytes_in_use;
  long long bypassed;         /* requests admitted past an older waiting one */
} tfs_server_counters;
typedef struct tfs_server tfs_server;
/* Defaults: 16 workers, 160 GB, FP32C, linear tolerance 1e-8, the step
 * defaults of tfs_step_config_default, max_bypass_ms 1000. */
int tfs_server_config_default(tfs_server_config *cfg);
int tfs_server_create(const tfs_server_config *cfg, tfs_server **out);
/* Queues a request (arrival time = now); TFS_ENOMEM if its swimmer alone
 * exceeds the budget. Instances stay resident between requests, keyed by
 * geometry; a request can be admitted when an idle instance of its geometry
 * exists or a new one fits in the budget after evicting idle instances
 * (least recently used first). Requests are admitted in arrival order,
 * except that while the oldest waits for device memory held by running
 * requests, a later request that fits is admitted past it -- until the
 * oldest has waited max_bypass_ms; from then on nothing passes it. Memory is
 * accounted from each instance's estimated size at admission. */
int tfs_server_submit(tfs_server *sv, const tfs_request *r, long long *ticket);
/* The device bytes the server accounts for a request's instance. */
int tfs_server_request_bytes(const tfs_server *sv, const tfs_request *r, size_t *bytes);
/* *status: 1 while pending, else the request's TFS status (the ticket is
 * then released; a failed request's message becomes the calling thread's
 * tfs_last_error()). TFS_ENOTCONV: Broyden's method reached its cap at some
 * step; the run stopped there, as the reference's does, and x_out/body_out
 * hold that state. wait != 0 blocks until it completes. latency_ms:
 * arrival to completion. */
int tfs_server_poll(tfs_server *sv, long long ticket, int wait, int *status, double *latency_ms,
                    int *broyden_iters, int *gmres_iters);
int tfs_server_drain(tfs_server *sv);   /* until every submitted request completed */
int tfs_server_stats(tfs_server *sv, tfs_server_counters *out);
int tfs_server_shared_solves(tfs_server *sv, long long *launches, long long *solves);
int tfs_server_shared_products(tfs_server *sv, long long *launches, long long *products);
int tfs_server_destroy(tfs_server *sv); /* drains first */

/* --- flow-field evaluator ---------------------------------------------- */
/* Replaces the reference's flow_field_evaluator
 * (src/flow_field/flow_field_evaluator.hpp:8-61): the fluid velocity at
 * num_flow points due to the segment forces/torques and blob forces of a
 * saved state of num_bodies swimmers,
 *   v(x) = 1/(8 pi mu) [ sum_segs (Stokeslet + rotlet) + sum_blobs Stokeslet ]
 * (flow_velocities, flow_field_evaluator.cu:13-228; velocities, :546-579).
 * With blobs_per_body == 0 the segment Stokeslet becomes the Blakelet of a
 * no-slip wall at z = 0, as in the reference. precision TFS_FP64 (the
 * reference's arithmetic) or TFS_FP32C (FP32 pair terms about the mean body
 * centre, compensated sums, FP64 output). Arrays are AoS float64:
 * x_flow[3 num_flow] v_flow[3 num_flow], x_segs[3 Ns] f_segs[6 Ns],
 * x_blobs[3 Nb] f_blobs[3 Nb] (NULL when Nb = 0), x_bodies[3 num_bodies],
 * with Ns = num_bodies * segs_per_body and Nb = num_bodies * blobs_per_body.
 * A point on top of a source gives inf/NaN there, as in the reference. */
typedef struct tfs_flow tfs_flow;
int tfs_flow_create(int num_flow, int num_bodies, int segs_per_body, int blobs_per_body,
                    int precision, tfs_flow **out);
int tfs_flow_destroy(tfs_flow *f);
int tfs_flow_set_stream(tfs_flow *f, void *stream);
/* read_positions_and_forces (flow_field_evaluator.cu:401-544), from host
 * arrays; returns once they are on the device. */
int tfs_flow_copy_inputs_to_device(tfs_flow *f, const double *x_flow, const double *x_segs,
                                   const double *f_segs, const double *x_blobs,
                                   const double *f_blobs, const double *x_bodies);
/* velocities (flow_field_evaluator.cu:546-579); remove_net_force != 0
 * subtracts, for every source force, its Stokeslet placed at its body's
 * centre (REMOVE_NET_FORCE_STOKESLET). Asynchronous on the flow's stream. */
int tfs_flow_velocities(tfs_flow *f, double mu, int remove_net_force);
int tfs_flow_copy_velocities_to_host(tfs_flow *f, double *v_flow);
/* Launch variants of the flow kernel (threads per CTA x targets per thread)
 * for a precision; tfs_flow_set_variant picks one for the flow's precision.
 * tfs_flow_autotune times every variant on the inputs on the device (reps
 * evaluations each, after one warm-up) and keeps the fastest: *best gets
 * its index and *best_ms its time per evaluation (either may be NULL). */
int tfs_flow_num_variants(int precision);
int tfs_flow_set_variant(tfs_flow *f, int variant);
int tfs_flow_autotune(tfs_flow *f, double mu, int remove_net_force, int reps, int *best,
                      double *best_ms);
/* Device arrays x_flow[3 num_flow] and v_flow[3 num_flow] (either may be NULL). */
int tfs_flow_device_buffers(tfs_flow *f, double **x_flow, double **v_flow);
int tfs_flow_wait(tfs_flow *f);

/* --- without device allocation ------------------------------------------ */
/* No counterpart in the reference (its rpy_mobility_solver allocates its own
 * device arrays). For callers that cannot allocate device memory -- a driver
 * that reserves all device memory up front for its own pool, a real-time loop
 * that must not block on cudaMalloc, code running inside another framework's
 * stream capture: v_segs = M_ss f_segs in FP64 (the assign semantics of
 * tfs_evaluate_segment_segment_mobility, and its result to FP64 rounding:
 * the sources are split into different chunks, so the sums are added in a
 * different order and the two agree to ~1e-15, not bit for bit) on the caller's
 * device arrays x_segs[3n], f_segs[6n], v_segs[6n], on `stream` (a
 * cudaStream_t; NULL = the legacy default stream), asynchronously.
 * Working memory is one file-scope device array of fixed size that every GPU
 * loading this library holds until exit; it allows n <= TFS_NOALLOC_MAX_SEGS
 * (larger n returns TFS_EINVAL). The entry point calls no cudaMalloc, cudaFree
 * or other allocating routine. The first call on a device looks up the
 * array's device address there (cudaGetSymbolAddress) and keeps it for the
 * life of the process; make that first call outside any stream capture, and
 * do not reset the device (cudaDeviceReset) after it: the kept address would
 * then be stale. Calls share the array: each call overwrites
 * every entry it later reads, so nothing needs clearing, but two calls that
 * overlap on the GPU (different streams, no ordering) race on it. */
#define TFS_NOALLOC_MAX_SEGS 12800
int tfs_mss_noalloc(const double *x_segs, const double *f_segs, double *v_segs, int num_segs,
                    double mu, double a_seg, void *stream);

/* --- diagnostics ------------------------------------------------------- */
/* CUDA-event timing of the solver's RPY product launches (the work-queue
 * kernel of each product, and the tile kernels of the kernel-sequence GMRES;
 * pack and reduce kernels excluded), on the solver's stream. Enabling resets
 * the record. tfs_solver_kernel_timing synchronises the stream, writes the
 * duration in ms of each timed launch since the last query, in launch order,
 * into ms[0..capacity), sets *launches to the number recorded, and resets.
 * At most 4096 launches are recorded between two queries. */
int tfs_solver_enable_kernel_timing(tfs_solver *s, int enable);
int tfs_solver_kernel_timing(tfs_solver *s, double *ms, int capacity, int *launches);
/* Message of the calling thread's last failed call ("" if none). */
const char *tfs_last_error(void);
/* Number of this library's kernels launched since load (all solvers). */
long long tfs_kernel_launch_count(void);
/* Measured FMA throughput of the current device in FLOP/s (2 per FMA),
 * precision TFS_FP64 or TFS_FP32C (plain FP32 FMAs), from a dependent-chain
 * microbenchmark over every SM. */
int tfs_measure_fma_peak(int precision, double *flops_per_second);
/* y[i] = x[i]^(-1/2) by the FP64 reciprocal square root the FP64 pair
 * kernels use for far-field separations (an FP32 hardware seed refined by one
 * third-order Householder step), on device arrays x[n], y[n], on `stream`;
 * valid for x in the FP32 normal range. For accuracy tests; no counterpart in
 * the reference (its unbounded pair takes 1/(sqrt(r^2) + 1e-20),
 * cuda_functions.cu:212-213). */
int tfs_rsqrt_far(const double *x, double *y, int n, void *stream);
/* Phase trace of the cooperative inner GMRES, for profiling: in a library
 * built with -DTFS_PG_TRACE, the globaltimer stamps (ns) of thread 0 of its
 * first two CTAs at eight points of every Arnoldi step of the last solve run,
 * stamps[(cta * steps + k) * 8 + phase] (phases: step start, M_bb done, w
 * formed, first-pass dots reduced, h1 summed, second-pass dots reduced, h2
 * summed, Q_k and z_k done); *steps gets the steps the buffer holds.
 * TFS_ESTATE in other builds. No counterpart in the reference. */
int tfs_pg_trace(unsigned long long *stamps, int capacity, int *steps);

#ifdef __cplusplus
}
#endif

#endif /* TFS_GB300_H */
