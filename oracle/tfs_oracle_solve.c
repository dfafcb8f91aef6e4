/* tfs_oracle_solve.c -- CPU restatement of the reference's free-body
 * mobility solve (TEST INFRASTRUCTURE ONLY; see tfs_oracle.h).
 *
 * One swimmer (NSWIM = 1): blobs on a rigid body with body-frame references
 * ref_m, segments with forces/torques. Unknowns x = [lambda (3 Nb blob
 * forces); U, Omega (body velocity)], n = 3 Nb + 6. Follows
 * src/cilia/mobility/mobility_solver.cpp:
 *   read_positions_and_forces   :176-236  (barrier forces; blob repulsion
 *                                          added to the swimmer's force)
 *   compute_velocities          :2574-2659 (free-body branch :2599-2636)
 *   assemble_rhs                :439-570   (rhs = [-v_blobs; -f_swimmer])
 *   apply_preconditioner_new    :1437-1509
 *   system_matrix_mult_new      :2027-2084
 *   solve_linear_system (GMRES) :2092-2570
 *   make_body_reference_matrices:2950-3047
 * Matrices are stored column-major like the reference's `matrix` class.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "tfs_oracle.h"

struct orc_solver {
  orc_params p;
  int nfil, nseg, nblob, ns, n;
  int end_force_magnitude;
  double repulsive_force_factor;
  double tol;
  int max_iter;
  double *refs;       /* 3 nblob, body frame */
  double body_x[3];
  double R[9];        /* rotation matrix, column-major */
  double body_mob[36], ktkinv[36];
  double *f_blobs;    /* 3 nblob: warm start / solution */
  double v_bodies[6];
  /* workspace */
  double *x_blobs, *diff, *f_dev, *frep, *v_blobs, *rhs, *Q, *H, *beta, *cs, *sn, *w, *z, *soln,
      *y, *tmp;
};

static const double ORC_PI2 = 3.14159265358979323846264338327950288;

/* quaternion::rot_mat (quaternion.cpp:327-369), column-major R(i,j) = R[i + 3j] */
static void rot_mat(double *R, const double *q) {
  const double s = q[0], a = q[1], b = q[2], c = q[3];
#define RM(i, j) R[(i) + 3 * (j)]
  RM(0, 0) = 1.0 - 2.0 * b * b - 2.0 * c * c;
  RM(1, 1) = 1.0 - 2.0 * a * a - 2.0 * c * c;
  RM(2, 2) = 1.0 - 2.0 * a * a - 2.0 * b * b;
  RM(1, 0) = 2.0 * a * b + 2.0 * s * c;
  RM(0, 1) = 2.0 * a * b - 2.0 * s * c;
  RM(2, 0) = 2.0 * a * c - 2.0 * s * b;
  RM(0, 2) = 2.0 * a * c + 2.0 * s * b;
  RM(2, 1) = 2.0 * b * c + 2.0 * s * a;
  RM(1, 2) = 2.0 * b * c - 2.0 * s * a;
#undef RM
}

static void matvec3(double *out, const double *M, const double *v) {
  for (int i = 0; i < 3; ++i) out[i] = M[i] * v[0] + M[i + 3] * v[1] + M[i + 6] * v[2];
}

/* out = M v for a 6x6 column-major M */
static void matvec6(double *out, const double *M, const double *v) {
  for (int i = 0; i < 6; ++i) {
    double s = 0.0;
    for (int k = 0; k < 6; ++k) s += M[i + 6 * k] * v[k];
    out[i] = s;
  }
}

/* Each 3x3 block B of a 6x6 matrix becomes R B R^T (mobility_solver.cpp:1455-1467). */
static void rotate_blocks(double *out, const double *in, const double *R) {
  for (int bi = 0; bi < 2; ++bi)
    for (int bj = 0; bj < 2; ++bj) {
      double B[9], RB[9];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) B[i + 3 * j] = in[(3 * bi + i) + 6 * (3 * bj + j)];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
          double s = 0.0;
          for (int k = 0; k < 3; ++k) s += R[i + 3 * k] * B[k + 3 * j];
          RB[i + 3 * j] = s;
        }
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
          double s = 0.0;
          for (int k = 0; k < 3; ++k) s += RB[i + 3 * k] * R[j + 3 * k];
          out[(3 * bi + i) + 6 * (3 * bj + j)] = s;
        }
    }
}

/* 6x6 inverse by Gauss-Jordan with partial pivoting (matrix::invert uses
 * LAPACK getrf/getri, matrix.cpp:538-561). Column-major in place. */
static void invert6(double *A) {
  double M[6][12];
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < 6; ++j) {
      M[i][j] = A[i + 6 * j];
      M[i][6 + j] = (i == j) ? 1.0 : 0.0;
    }
  for (int k = 0; k < 6; ++k) {
    int p = k;
    for (int i = k + 1; i < 6; ++i)
      if (fabs(M[i][k]) > fabs(M[p][k])) p = i;
    if (p != k)
      for (int j = 0; j < 12; ++j) {
        const double t = M[k][j];
        M[k][j] = M[p][j];
        M[p][j] = t;
      }
    const double piv = M[k][k];
    for (int j = 0; j < 12; ++j) M[k][j] /= piv;
    for (int i = 0; i < 6; ++i) {
      if (i == k) continue;
      const double f = M[i][k];
      for (int j = 0; j < 12; ++j) M[i][j] -= f * M[k][j];
    }
  }
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < 6; ++j) A[i + 6 * j] = M[i][6 + j];
}

orc_solver *orc_solver_create(const orc_params *p, int nfil, int nseg, int nblob,
                              const double *blob_refs, int end_force_magnitude,
                              double repulsive_force_factor, double tol, int max_iter) {
  orc_solver *s = (orc_solver *)calloc(1, sizeof *s);
  s->p = *p;
  s->nfil = nfil;
  s->nseg = nseg;
  s->nblob = nblob;
  s->ns = nfil * nseg;
  s->n = 3 * nblob + 6;
  s->end_force_magnitude = end_force_magnitude;
  s->repulsive_force_factor = repulsive_force_factor;
  s->tol = tol;
  s->max_iter = max_iter < s->n ? max_iter : s->n; /* min(system size, MAX_LINEAR_SYSTEM_ITER) */
  const size_t nb3 = 3 * (size_t)nblob, n = (size_t)s->n, m = (size_t)s->max_iter;
  s->refs = (double *)malloc(sizeof(double) * nb3);
  memcpy(s->refs, blob_refs, sizeof(double) * nb3);
  s->f_blobs = (double *)calloc(nb3, sizeof(double));
  s->x_blobs = (double *)calloc(nb3, sizeof(double));
  s->diff = (double *)calloc(nb3, sizeof(double));
  s->frep = (double *)calloc(nb3, sizeof(double));
  s->v_blobs = (double *)calloc(nb3, sizeof(double));
  s->f_dev = (double *)calloc(6 * (size_t)s->ns, sizeof(double));
  s->rhs = (double *)calloc(n, sizeof(double));
  s->Q = (double *)calloc(n * (m + 1), sizeof(double));
  s->H = (double *)calloc((m + 1) * (m + 1), sizeof(double));
  s->beta = (double *)calloc(m + 1, sizeof(double));
  s->cs = (double *)calloc(m, sizeof(double));
  s->sn = (double *)calloc(m, sizeof(double));
  s->w = (double *)calloc(n, sizeof(double));
  s->z = (double *)calloc(n, sizeof(double));
  s->soln = (double *)calloc(n, sizeof(double));
  s->tmp = (double *)calloc(n, sizeof(double));
  s->y = (double *)calloc(m + 1, sizeof(double));
  const double q1[4] = {1, 0, 0, 0};
  rot_mat(s->R, q1);
  for (int i = 0; i < 6; ++i) {
    s->body_mob[i + 6 * i] = 1.0; /* identity(6), mobility_solver.cpp:112-114 */
    s->ktkinv[i + 6 * i] = 1.0;
  }
  return s;
}

void orc_solver_destroy(orc_solver *s) {
  if (!s) return;
  double *bufs[] = {s->refs, s->f_blobs, s->x_blobs, s->diff, s->frep, s->v_blobs, s->f_dev,
                    s->rhs, s->Q, s->H, s->beta, s->cs, s->sn, s->w, s->z, s->soln, s->tmp, s->y};
  for (size_t k = 0; k < sizeof bufs / sizeof bufs[0]; ++k) free(bufs[k]);
  free(s);
}

void orc_solver_set_body(orc_solver *s, const double *x, const double *q) {
  memcpy(s->body_x, x, sizeof s->body_x);
  rot_mat(s->R, q);
}

/* rigid_body::blob_positions (rigid_body.cpp:482-500); diff = R ref */
static void blob_positions(orc_solver *s) {
  for (int m = 0; m < s->nblob; ++m) {
    matvec3(&s->diff[3 * m], s->R, &s->refs[3 * m]);
    for (int k = 0; k < 3; ++k) s->x_blobs[3 * m + k] = s->body_x[k] + s->diff[3 * m + k];
  }
}

/* system_matrix_mult_new, free body (mobility_solver.cpp:2027-2084):
 * out = [M_bb in_l - K in_V ; -K^T in_l] */
static void system_mult(orc_solver *s, double *out, const double *in) {
  const int nb = s->nblob, vel = 3 * nb;
  memset(out, 0, sizeof(double) * s->n);
  for (int m = 0; m < nb; ++m) {
    const double *d = &s->diff[3 * m];
    const double *l = &in[3 * m];
    out[vel] -= l[0];
    out[vel + 1] -= l[1];
    out[vel + 2] -= l[2];
    out[vel + 3] -= d[1] * l[2] - d[2] * l[1];
    out[vel + 4] -= d[2] * l[0] - d[0] * l[2];
    out[vel + 5] -= d[0] * l[1] - d[1] * l[0];
    out[3 * m] -= in[vel] - d[1] * in[vel + 5] + d[2] * in[vel + 4];
    out[3 * m + 1] -= in[vel + 1] - d[2] * in[vel + 3] + d[0] * in[vel + 5];
    out[3 * m + 2] -= in[vel + 2] - d[0] * in[vel + 4] + d[1] * in[vel + 3];
  }
  orc_mbb(&s->p, s->tmp, in, s->x_blobs, nb); /* v_blobs = M_bb in_l */
  for (int k = 0; k < 3 * nb; ++k) out[k] += s->tmp[k];
}

/* apply_preconditioner_new, free body (mobility_solver.cpp:1437-1509) */
static void precondition(orc_solver *s, double *out, const double *in) {
  const int nb = s->nblob, vel = 3 * nb;
  double bm[36], kt[36], b[6] = {0, 0, 0, 0, 0, 0}, t1[6], t2[6];
  rotate_blocks(bm, s->body_mob, s->R);
  rotate_blocks(kt, s->ktkinv, s->R);
  for (int m = 0; m < nb; ++m) {
    const double *d = &s->diff[3 * m];
    const double *l = &in[3 * m];
    b[0] -= l[0];
    b[1] -= l[1];
    b[2] -= l[2];
    b[3] -= d[1] * l[2] - d[2] * l[1];
    b[4] -= d[2] * l[0] - d[0] * l[2];
    b[5] -= d[0] * l[1] - d[1] * l[0];
  }
  matvec6(t1, kt, b);
  matvec6(t2, bm, &in[vel]);
  for (int k = 0; k < 6; ++k) out[vel + k] = t1[k] - t2[k];
  const double *U = &out[vel];
  for (int m = 0; m < nb; ++m) {
    const double *d = &s->diff[3 * m];
    double blk[3] = {in[3 * m] + U[0], in[3 * m + 1] + U[1], in[3 * m + 2] + U[2]};
    blk[0] += U[4] * d[2] - U[5] * d[1];
    blk[1] += U[5] * d[0] - U[3] * d[2];
    blk[2] += U[3] * d[1] - U[4] * d[0];
    out[3 * m] = blk[0];
    out[3 * m + 1] = blk[1];
    out[3 * m + 2] = blk[2];
  }
  const double minv = 6.0 * ORC_PI2 * s->p.mu * s->p.a_blob;
  for (int k = 0; k < vel; ++k) out[k] *= minv;
}

static double norm2(const double *v, int n) {
  double s = 0.0;
  for (int i = 0; i < n; ++i) s += v[i] * v[i];
  return sqrt(s);
}

/* solve_linear_system (mobility_solver.cpp:2092-2570), right preconditioned
 * GMRES without restarts, warm-started from (f_blobs, v_bodies). Returns the
 * iteration count (0 if the warm start or a zero right-hand side sufficed). */
int orc_solver_gmres(orc_solver *s) {
  const int n = s->n, nb = s->nblob, vel = 3 * nb, mi = s->max_iter;
  double *Q = s->Q, *H = s->H, *beta = s->beta;
#define QC(j) (Q + (size_t)(j) * n)
#define HH(i, j) H[(i) + (size_t)(j) * (mi + 1)]
  const double norm_rhs = norm2(s->rhs, n);
  if (norm_rhs == 0.0) {
    memset(s->f_blobs, 0, sizeof(double) * vel);
    memset(s->v_bodies, 0, sizeof s->v_bodies);
    return 0;
  }
  memcpy(s->soln, s->f_blobs, sizeof(double) * vel);
  memcpy(s->soln + vel, s->v_bodies, sizeof s->v_bodies);
  system_mult(s, s->w, s->soln);
  for (int i = 0; i < n; ++i) QC(0)[i] = s->rhs[i] - s->w[i];
  beta[0] = norm2(QC(0), n);
  if (fabs(beta[0]) <= s->tol * norm_rhs) return 0;
  if (fabs(beta[0]) > norm_rhs) {
    memset(s->soln, 0, sizeof(double) * n);
    beta[0] = norm_rhs;
    memcpy(QC(0), s->rhs, sizeof(double) * n);
  }
  for (int i = 0; i < n; ++i) QC(0)[i] /= beta[0];
  for (int iter = 1; iter <= mi; ++iter) {
    precondition(s, s->z, QC(iter - 1));
    system_mult(s, QC(iter), s->z);
    for (int i = 0; i < iter; ++i) {
      double h = 0.0;
      for (int k = 0; k < n; ++k) h += QC(iter)[k] * QC(i)[k];
      HH(i, iter - 1) = h;
      for (int k = 0; k < n; ++k) QC(iter)[k] -= h * QC(i)[k];
    }
    const double qn = norm2(QC(iter), n);
    HH(iter, iter - 1) = qn;
    for (int k = 0; k < n; ++k) QC(iter)[k] /= qn;
    for (int i = 1; i < iter; ++i) {
      const double t = s->cs[i - 1] * HH(i - 1, iter - 1) + s->sn[i - 1] * HH(i, iter - 1);
      HH(i, iter - 1) = s->cs[i - 1] * HH(i, iter - 1) - s->sn[i - 1] * HH(i - 1, iter - 1);
      HH(i - 1, iter - 1) = t;
    }
    const double a = HH(iter - 1, iter - 1), b = HH(iter, iter - 1);
    if (b == 0.0) {
      s->cs[iter - 1] = 1.0;
      s->sn[iter - 1] = 0.0;
    } else if (fabs(b) > fabs(a)) {
      const double t = a / b;
      s->sn[iter - 1] = (2.0 * (double)(b > 0) - 1.0) / sqrt(1.0 + t * t);
      s->cs[iter - 1] = t * s->sn[iter - 1];
    } else {
      const double t = b / a;
      s->cs[iter - 1] = (2.0 * (double)(a > 0) - 1.0) / sqrt(1.0 + t * t);
      s->sn[iter - 1] = t * s->cs[iter - 1];
    }
    HH(iter - 1, iter - 1) = s->cs[iter - 1] * a + s->sn[iter - 1] * b;
    HH(iter, iter - 1) = 0.0;
    beta[iter] = -s->sn[iter - 1] * beta[iter - 1];
    beta[iter - 1] = s->cs[iter - 1] * beta[iter - 1];
    const double rel = fabs(beta[iter]) / norm_rhs;
    if (rel <= s->tol || iter == mi) {
      double *y = s->y;
      y[iter - 1] = beta[iter - 1] / HH(iter - 1, iter - 1);
      for (int i = iter - 2; i >= 0; --i) {
        y[i] = beta[i];
        for (int j = iter - 1; j > i; --j) y[i] -= HH(i, j) * y[j];
        y[i] /= HH(i, i);
      }
      memset(s->tmp, 0, sizeof(double) * n);
      for (int i = 0; i < iter; ++i)
        for (int k = 0; k < n; ++k) s->tmp[k] += y[i] * QC(i)[k];
      precondition(s, s->z, s->tmp);
      for (int k = 0; k < n; ++k) s->soln[k] += s->z[k];
      memcpy(s->f_blobs, s->soln, sizeof(double) * vel);
      memcpy(s->v_bodies, s->soln + vel, sizeof s->v_bodies);
      return iter;
    }
  }
#undef QC
#undef HH
  return 0;
}

/* read_positions_and_forces (free body, mobility_solver.cpp:176-236) */
static void read_positions_and_forces(orc_solver *s, const double *x_segs, const double *f_segs,
                                      double *swimmer_f) {
  memcpy(s->f_dev, f_segs, sizeof(double) * 6 * s->ns);
  blob_positions(s);
  orc_barrier_forces(&s->p, s->f_dev, s->frep, x_segs, s->x_blobs, s->ns, s->nblob,
                             s->nseg, s->end_force_magnitude, s->repulsive_force_factor, 1);
  for (int m = 0; m < s->nblob; ++m) {
    const double *r = &s->diff[3 * m], *f = &s->frep[3 * m];
    swimmer_f[0] += f[0];
    swimmer_f[1] += f[1];
    swimmer_f[2] += f[2];
    swimmer_f[3] += r[1] * f[2] - r[2] * f[1];
    swimmer_f[4] += r[2] * f[0] - r[0] * f[2];
    swimmer_f[5] += r[0] * f[1] - r[1] * f[0];
  }
}

int orc_solver_compute_velocities(orc_solver *s, const double *x_segs, const double *f_segs,
                                  double *swimmer_f, double *v_segs, double *v_blobs) {
  read_positions_and_forces(s, x_segs, f_segs, swimmer_f);
  orc_mss(&s->p, v_segs, s->f_dev, x_segs, s->ns);
  orc_mbs(&s->p, s->v_blobs, s->f_dev, s->x_blobs, x_segs, s->nblob, s->ns);
  if (v_blobs) memcpy(v_blobs, s->v_blobs, sizeof(double) * 3 * s->nblob);
  for (int k = 0; k < 3 * s->nblob; ++k) s->rhs[k] = -s->v_blobs[k];
  for (int k = 0; k < 6; ++k) s->rhs[3 * s->nblob + k] = -swimmer_f[k];
  const int iters = orc_solver_gmres(s);
  orc_msb(&s->p, v_segs, s->f_blobs, x_segs, s->x_blobs, s->ns, s->nblob);
  return iters;
}

void orc_solver_make_body_reference_matrices(orc_solver *s, const double *x_segs,
                                             const double *f_segs) {
  /* KTK (mobility_solver.cpp:2954-2971); rcross(v) a = a x v */
  double KTK[36];
  memset(KTK, 0, sizeof KTK);
  KTK[0] = KTK[7] = KTK[14] = (double)s->nblob;
  for (int m = 0; m < s->nblob; ++m) {
    const double *v = &s->refs[3 * m];
    /* rcross(v) column-major: (0,0)=0 (1,0)=-v2 (2,0)=v1 (0,1)=v2 (1,1)=0 (2,1)=-v0
     * (0,2)=-v1 (1,2)=v0 (2,2)=0 */
    const double rc[9] = {0, -v[2], v[1], v[2], 0, -v[0], -v[1], v[0], 0};
    double rc2[9];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        double t = 0.0;
        for (int k = 0; k < 3; ++k) t += rc[i + 3 * k] * rc[k + 3 * j];
        rc2[i + 3 * j] = t;
      }
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        KTK[i + 6 * (3 + j)] += rc[i + 3 * j];
        KTK[(3 + i) + 6 * j] -= rc[i + 3 * j];
        KTK[(3 + i) + 6 * (3 + j)] -= rc2[i + 3 * j];
      }
  }
  invert6(KTK);
  memcpy(s->ktkinv, KTK, sizeof KTK);
  /* six solves with rhs = -e_{5-n}: column 5-n of the body mobility */
  double swimmer_f[6] = {0, 0, 0, 0, 0, 0};
  read_positions_and_forces(s, x_segs, f_segs, swimmer_f);
  for (int k = 0; k < 6; ++k) {
    memset(s->rhs, 0, sizeof(double) * s->n);
    s->rhs[s->n - 1 - k] = -1.0;
    orc_solver_gmres(s);
    for (int i = 0; i < 6; ++i) s->body_mob[i + 6 * (5 - k)] = s->v_bodies[i];
  }
}

void orc_solver_state(const orc_solver *s, double *f_blobs, double *v_bodies, double *body_mob,
                      double *ktkinv) {
  if (f_blobs) memcpy(f_blobs, s->f_blobs, sizeof(double) * 3 * s->nblob);
  if (v_bodies) memcpy(v_bodies, s->v_bodies, sizeof s->v_bodies);
  if (body_mob) memcpy(body_mob, s->body_mob, sizeof s->body_mob);
  if (ktkinv) memcpy(ktkinv, s->ktkinv, sizeof s->ktkinv);
}

void orc_solver_set_state(orc_solver *s, const double *f_blobs, const double *v_bodies,
                          const double *body_mob, const double *ktkinv) {
  if (f_blobs) memcpy(s->f_blobs, f_blobs, sizeof(double) * 3 * s->nblob);
  if (v_bodies) memcpy(s->v_bodies, v_bodies, sizeof s->v_bodies);
  if (body_mob) memcpy(s->body_mob, body_mob, sizeof s->body_mob);
  if (ktkinv) memcpy(s->ktkinv, ktkinv, sizeof s->ktkinv);
}
