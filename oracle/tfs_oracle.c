/* tfs_oracle.c -- CPU restatement of the reference's RPY mobility path.
 * TEST INFRASTRUCTURE ONLY (see tfs_oracle.h). */
#include "tfs_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <stddef.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static const double ORC_PI = 3.14159265358979323846264338327950288;

static int g_threads = 1;

void orc_set_threads(int n) {
#ifdef _OPENMP
  g_threads = n > 0 ? n : omp_get_max_threads();
#else
  (void)n;
  g_threads = 1;
#endif
}

int orc_get_threads(void) { return g_threads; }

/* ------------------------------------------------------------------------ */
/* RPY pair: cuda_functions.cu:205-356.                                      */
/* Three regimes of the separation r: far (r > ai + aj), overlapping         */
/* (|ai - aj| < r <= ai + aj, Zuk et al. 2014) and nested (r <= |ai - aj|,   */
/* which includes the self term r = 0). Blocks: translation-translation      */
/* (:221-260), translation-rotation (:262-284), rotation-translation         */
/* (:286-306), rotation-rotation (:308-352).                                 */
/* ------------------------------------------------------------------------ */
void orc_rpy_pair(int vd, int fd, double *V, const double *F, double xi, double yi, double zi,
                  double ai, double xj, double yj, double zj, double aj, double mu) {
  double ex = xi - xj, ey = yi - yj, ez = zi - zj;
  const double r = sqrt(ex * ex + ey * ey + ez * ez);
  /* :213 -- no special case for r = 0; the unit vector becomes 0. */
  const double inv_r = 1.0 / (r + 1e-20);
  const double adiff = fabs(ai - aj);
  const double asum = ai + aj;
  ex *= inv_r;
  ey *= inv_r;
  ez *= inv_r;

  double A, B;
  /* translation-translation: V_t += A F + B (e.F) e */
  double e_dot = ex * F[0] + ey * F[1] + ez * F[2];
  if (r > asum) {
    const double s = inv_r * inv_r * (ai * ai + aj * aj) / 3.0;
    const double c = inv_r / (8.0 * ORC_PI * mu);
    A = (1.0 + s) * c;
    B = (1.0 - 3.0 * s) * c * e_dot;
  } else if (r > adiff) {
    const double r3x32 = 32.0 * r * r * r;
    const double p = adiff * adiff + 3.0 * r * r;
    const double q = adiff * adiff - r * r;
    const double c = 1.0 / (6.0 * ORC_PI * mu * ai * aj);
    A = (0.5 * asum - p * p / r3x32) * c;
    B = (3.0 * q * q / r3x32) * c * e_dot;
  } else {
    A = 1.0 / (6.0 * ORC_PI * mu * (ai > aj ? ai : aj));
    B = 0.0;
  }
  V[0] += A * F[0] + B * ex;
  V[1] += A * F[1] + B * ey;
  V[2] += A * F[2] + B * ez;

  if (fd > 3) {
    /* translation-rotation: V_t += A (T x e) */
    if (r > asum) {
      A = inv_r * inv_r / (8.0 * ORC_PI * mu);
    } else if (r > adiff) {
      const double g = aj - ai + r;
      A = inv_r * inv_r * g * g * (ai * ai + 2.0 * ai * (r + aj) - 3.0 * (aj - r) * (aj - r)) /
          (128.0 * ORC_PI * mu * ai * aj * aj * aj);
    } else {
      A = (aj > ai ? 1.0 : 0.0) * r / (8.0 * ORC_PI * mu * aj * aj * aj);
    }
    V[0] += A * (F[4] * ez - F[5] * ey);
    V[1] += A * (F[5] * ex - F[3] * ez);
    V[2] += A * (F[3] * ey - F[4] * ex);
  }

  if (vd > 3) {
    /* rotation-translation: the translation-rotation block with ai and aj
     * swapped; V_r += A (F x e) */
    if (r > asum) {
      A = inv_r * inv_r / (8.0 * ORC_PI * mu);
    } else if (r > adiff) {
      const double g = ai - aj + r;
      A = inv_r * inv_r * g * g * (aj * aj + 2.0 * aj * (r + ai) - 3.0 * (ai - r) * (ai - r)) /
          (128.0 * ORC_PI * mu * aj * ai * ai * ai);
    } else {
      A = (ai > aj ? 1.0 : 0.0) * r / (8.0 * ORC_PI * mu * ai * ai * ai);
    }
    V[3] += A * (F[1] * ez - F[2] * ey);
    V[4] += A * (F[2] * ex - F[0] * ez);
    V[5] += A * (F[0] * ey - F[1] * ex);

    if (fd > 3) {
      /* rotation-rotation: V_r += A T + B (e.T) e */
      e_dot = ex * F[3] + ey * F[4] + ez * F[5];
      if (r > asum) {
        A = -inv_r * inv_r * inv_r / (16.0 * ORC_PI * mu);
        B = -3.0 * e_dot * A;
      } else if (r > adiff) {
        const double r2 = r * r, r3 = r2 * r;
        const double ai2 = ai * ai, aj2 = aj * aj;
        const double ai3 = ai2 * ai, aj3 = aj2 * aj;
        const double ad4 = adiff * adiff * adiff * adiff;
        double num = 5.0 * r3 * r3 - 27.0 * r2 * r2 * (ai2 + aj2) + 32.0 * r3 * (ai3 + aj3) -
                     9.0 * r2 * (ai2 - aj2) * (ai2 - aj2) - ad4 * (ai2 + aj2 + 4.0 * ai * aj);
        const double q = (ai - aj) * (ai - aj) - r2;
        const double den = 1.0 / (512.0 * ORC_PI * mu * r3 * ai3 * aj3);
        A = num * den;
        B = 3.0 * q * q * (ai2 + aj2 + 4.0 * ai * aj - r2) * den * e_dot;
      } else {
        const double am = ai > aj ? ai : aj;
        A = 1.0 / (8.0 * ORC_PI * mu * am * am * am);
        B = 0.0;
      }
      V[3] += A * F[3] + B * ex;
      V[4] += A * F[4] + B * ey;
      V[5] += A * F[5] + B * ez;
    }
  }
}

/* ------------------------------------------------------------------------ */
/* Weakly coupled filaments (the reference's                                 */
/* weakly_coupled_filaments_rpy_mobility_solver.cu:50-107: filament means    */
/* and total forces on upload, then Msf_mult, cuda_functions.cu:991-1080 and */
/* :1129-1229, free space). Z_f = sum_k x_{f,k} / NSEG and Ftot_f = sum_k    */
/* F_{f,k}; segment i of filament f sums, over filaments j in order, the     */
/* translation-only RPY pairs of its own filament's segments (j = f) or the  */
/* Stokeslet (1/8 pi mu)(Ftot_j / r + (r.Ftot_j) r / r^3), r = x_i - Z_j     */
/* (j != f). The rotational velocities are zero (:1220-1225).                */
/* ------------------------------------------------------------------------ */
void orc_msf(const orc_params *p, double *v_segs, const double *f_segs, const double *x_segs,
             int nfil, int nseg) {
  double *Z = (double *)calloc(3 * (size_t)nfil, sizeof(double));
  double *Ft = (double *)calloc(3 * (size_t)nfil, sizeof(double));
  for (int fi = 0; fi < nfil; ++fi)
    for (int k = 0; k < nseg; ++k) {
      const size_t sg = (size_t)fi * nseg + k;
      for (int d = 0; d < 3; ++d) {
        Z[3 * fi + d] += x_segs[3 * sg + d] / (double)nseg;
        Ft[3 * fi + d] += f_segs[6 * sg + d];
      }
    }
  const double ff = 1.0 / (8.0 * ORC_PI * p->mu);
  const int ns = nfil * nseg;
#pragma omp parallel for schedule(dynamic, 16) num_threads(g_threads)
  for (int i = 0; i < ns; ++i) {
    const int fil = i / nseg;
    const double *xi = x_segs + 3 * (size_t)i;
    double v[3] = {0, 0, 0};
    for (int j = 0; j < nfil; ++j) {
      if (j == fil) {
        for (int k = 0; k < nseg; ++k) {
          const size_t jj = (size_t)j * nseg + k;
          const double *xj = x_segs + 3 * jj;
          orc_rpy_pair(3, 3, v, f_segs + 6 * jj, xi[0], xi[1], xi[2], p->a_seg, xj[0], xj[1],
                       xj[2], p->a_seg, p->mu);
        }
      } else {
        const double rx = xi[0] - Z[3 * j], ry = xi[1] - Z[3 * j + 1], rz = xi[2] - Z[3 * j + 2];
        const double rm1 = 1.0 / sqrt(rx * rx + ry * ry + rz * rz);
        const double rm3 = rm1 * rm1 * rm1;
        const double *F = Ft + 3 * j;
        const double rF = rx * F[0] + ry * F[1] + rz * F[2];
        v[0] += ff * (rm1 * F[0] + rm3 * rx * rF);
        v[1] += ff * (rm1 * F[1] + rm3 * ry * rF);
        v[2] += ff * (rm1 * F[2] + rm3 * rz * rF);
      }
    }
    double *o = v_segs + 6 * (size_t)i;
    o[0] = v[0];
    o[1] = v[1];
    o[2] = v[2];
    o[3] = o[4] = o[5] = 0.0;
  }
  free(Z);
  free(Ft);
}

/* ------------------------------------------------------------------------ */
/* The four mobility blocks. Each target i sums over all sources j in index   */
/* order (cuda_functions.cu:399-457 and the matching loops of the others).   */
/* ------------------------------------------------------------------------ */
void orc_mss(const orc_params *p, double *v_segs, const double *f_segs, const double *x_segs,
             int num_segs) {
#pragma omp parallel for schedule(dynamic, 16) num_threads(g_threads)
  for (int i = 0; i < num_segs; ++i) {
    double v[6] = {0, 0, 0, 0, 0, 0};
    const double *xi = x_segs + 3 * (size_t)i;
    for (int j = 0; j < num_segs; ++j) {
      const double *xj = x_segs + 3 * (size_t)j;
      orc_rpy_pair(6, 6, v, f_segs + 6 * (size_t)j, xi[0], xi[1], xi[2], p->a_seg, xj[0], xj[1],
                   xj[2], p->a_seg, p->mu);
    }
    memcpy(v_segs + 6 * (size_t)i, v, sizeof v); /* :463-468 assigns */
  }
}

void orc_msb(const orc_params *p, double *v_segs, const double *f_blobs, const double *x_segs,
             const double *x_blobs, int num_segs, int num_blobs) {
#pragma omp parallel for schedule(dynamic, 16) num_threads(g_threads)
  for (int i = 0; i < num_segs; ++i) {
    double v[6] = {0, 0, 0, 0, 0, 0};
    const double *xi = x_segs + 3 * (size_t)i;
    for (int j = 0; j < num_blobs; ++j) {
      const double *xj = x_blobs + 3 * (size_t)j;
      orc_rpy_pair(6, 3, v, f_blobs + 3 * (size_t)j, xi[0], xi[1], xi[2], p->a_seg, xj[0], xj[1],
                   xj[2], p->a_blob, p->mu);
    }
    for (int k = 0; k < 6; ++k) v_segs[6 * (size_t)i + k] += v[k]; /* :625-630 accumulates */
  }
}

void orc_mbb(const orc_params *p, double *v_blobs, const double *f_blobs, const double *x_blobs,
             int num_blobs) {
#pragma omp parallel for schedule(dynamic, 16) num_threads(g_threads)
  for (int i = 0; i < num_blobs; ++i) {
    double v[3] = {0, 0, 0};
    const double *xi = x_blobs + 3 * (size_t)i;
    for (int j = 0; j < num_blobs; ++j) {
      const double *xj = x_blobs + 3 * (size_t)j;
      orc_rpy_pair(3, 3, v, f_blobs + 3 * (size_t)j, xi[0], xi[1], xi[2], p->a_blob, xj[0], xj[1],
                   xj[2], p->a_blob, p->mu);
    }
    memcpy(v_blobs + 3 * (size_t)i, v, sizeof v); /* :539-544 assigns */
  }
}

void orc_mbs(const orc_params *p, double *v_blobs, const double *f_segs, const double *x_blobs,
             const double *x_segs, int num_blobs, int num_segs) {
#pragma omp parallel for schedule(dynamic, 16) num_threads(g_threads)
  for (int i = 0; i < num_blobs; ++i) {
    double v[3] = {0, 0, 0};
    const double *xi = x_blobs + 3 * (size_t)i;
    for (int j = 0; j < num_segs; ++j) {
      const double *xj = x_segs + 3 * (size_t)j;
      orc_rpy_pair(3, 6, v, f_segs + 6 * (size_t)j, xi[0], xi[1], xi[2], p->a_blob, xj[0], xj[1],
                   xj[2], p->a_seg, p->mu);
    }
    memcpy(v_blobs + 3 * (size_t)i, v, sizeof v); /* :745-751 assigns */
  }
}

void orc_rpy_block(const orc_params *p, int vd, int fd, double *v, const double *x_tgt, int n_tgt,
                   double a_tgt, const double *x_src, const double *f_src, int n_src,
                   double a_src, int accumulate) {
#pragma omp parallel for schedule(dynamic, 16) num_threads(g_threads)
  for (int i = 0; i < n_tgt; ++i) {
    double acc[6] = {0, 0, 0, 0, 0, 0};
    const double *xi = x_tgt + 3 * (size_t)i;
    for (int j = 0; j < n_src; ++j) {
      const double *xj = x_src + 3 * (size_t)j;
      orc_rpy_pair(vd, fd, acc, f_src + (size_t)fd * j, xi[0], xi[1], xi[2], a_tgt, xj[0], xj[1],
                   xj[2], a_src, p->mu);
    }
    for (int k = 0; k < vd; ++k) {
      double *o = v + (size_t)vd * i + k;
      *o = accumulate ? *o + acc[k] : acc[k];
    }
  }
}

/* ------------------------------------------------------------------------ */
/* barrier_forces: cuda_functions.cu:1240-1436 (no plane wall).             */
/* A segment i feels every segment and blob j within 1.1 (ai + aj), except  */
/* itself and its nearest neighbours on the same filament (:1319); a blob   */
/* feels every segment and every other blob (:1410).                        */
/* The magnitude is factor * E * fac^4 with fac = min(1, 1 - 10/asum (d -    */
/* asum)), E the integer end-force magnitude (:1321-1322).                   */
/* ------------------------------------------------------------------------ */
static void orc_repulsion_from(double *f, double xi, double yi, double zi, double xj, double yj,
                               double zj, double asum, double emag) {
  const double chi = 10.0 / asum;
  const double dx = xi - xj, dy = yi - yj, dz = zi - zj;
  const double dist = sqrt(dx * dx + dy * dy + dz * dz);
  if (dist < 1.1 * asum) {
    double fac = fmin(1.0, 1.0 - chi * (dist - asum));
    fac *= emag * fac * fac * fac;
    const double inv_d = 1.0 / dist;
    f[0] += fac * dx * inv_d;
    f[1] += fac * dy * inv_d;
    f[2] += fac * dz * inv_d;
  }
}

void orc_barrier_forces(const orc_params *p, double *f_segs, double *f_blobs_repulsion,
                        const double *x_segs, const double *x_blobs, int num_segs, int num_blobs,
                        int nseg, int end_force_magnitude, double repulsive_force_factor,
                        int free_body) {
  const double emag = repulsive_force_factor * (double)end_force_magnitude;
  const double ass = 2.0 * p->a_seg, asb = p->a_seg + p->a_blob, abb = 2.0 * p->a_blob;
#pragma omp parallel for schedule(dynamic, 16) num_threads(g_threads)
  for (int i = 0; i < num_segs; ++i) {
    double f[3] = {0, 0, 0};
    const double *xi = x_segs + 3 * (size_t)i;
    const int fil_i = i / nseg;
    for (int j = 0; j < num_segs; ++j) {
      const int fil_j = j / nseg;
      if (fil_i == fil_j && (i - j <= 1 && j - i <= 1)) continue;
      const double *xj = x_segs + 3 * (size_t)j;
      orc_repulsion_from(f, xi[0], xi[1], xi[2], xj[0], xj[1], xj[2], ass, emag);
    }
    for (int j = 0; j < num_blobs; ++j) {
      const double *xj = x_blobs + 3 * (size_t)j;
      orc_repulsion_from(f, xi[0], xi[1], xi[2], xj[0], xj[1], xj[2], asb, emag);
    }
    f_segs[6 * (size_t)i] += f[0];
    f_segs[6 * (size_t)i + 1] += f[1];
    f_segs[6 * (size_t)i + 2] += f[2];
  }
  if (!free_body) return;
#pragma omp parallel for schedule(dynamic, 16) num_threads(g_threads)
  for (int i = 0; i < num_blobs; ++i) {
    double f[3] = {0, 0, 0};
    const double *xi = x_blobs + 3 * (size_t)i;
    for (int j = 0; j < num_segs; ++j) {
      const double *xj = x_segs + 3 * (size_t)j;
      orc_repulsion_from(f, xi[0], xi[1], xi[2], xj[0], xj[1], xj[2], asb, emag);
    }
    for (int j = 0; j < num_blobs; ++j) {
      if (j == i) continue;
      const double *xj = x_blobs + 3 * (size_t)j;
      orc_repulsion_from(f, xi[0], xi[1], xi[2], xj[0], xj[1], xj[2], abb, emag);
    }
    memcpy(f_blobs_repulsion + 3 * (size_t)i, f, sizeof f);
  }
}

/* ------------------------------------------------------------------------ */
/* flow_velocities: flow_field_evaluator.cu:13-228.                          */
/* ------------------------------------------------------------------------ */
static void orc_stokeslet(double *v, double dx, double dy, double dz, const double *f, double sgn) {
  const double rm2 = 1.0 / (dx * dx + dy * dy + dz * dz);
  const double rm1 = sqrt(rm2);
  const double w = rm2 * (dx * f[0] + dy * f[1] + dz * f[2]);
  v[0] += sgn * rm1 * (f[0] + dx * w);
  v[1] += sgn * rm1 * (f[1] + dy * w);
  v[2] += sgn * rm1 * (f[2] + dz * w);
}

void orc_flow_velocities(double *v_flow, const double *x_flow, int num_flow, const double *f_segs,
                         const double *x_segs, int segs_per_body, const double *f_blobs,
                         const double *x_blobs, int blobs_per_body, const double *x_bodies,
                         int num_bodies, double prefac, int remove_net_force) {
  const int ns = segs_per_body * num_bodies, nb = blobs_per_body * num_bodies;
#pragma omp parallel for schedule(dynamic, 64) num_threads(g_threads)
  for (int i = 0; i < num_flow; ++i) {
    const double xi = x_flow[3 * (size_t)i], yi = x_flow[3 * (size_t)i + 1],
                 zi = x_flow[3 * (size_t)i + 2];
    double v[3] = {0, 0, 0};
    for (int j = 0; j < ns; ++j) {
      const double *xj = x_segs + 3 * (size_t)j;
      const double *fj = f_segs + 6 * (size_t)j;
      const double dx = xi - xj[0], dy = yi - xj[1], dz = zi - xj[2];
      /* Stokeslet (:72-82) */
      const double rm2 = 1.0 / (dx * dx + dy * dy + dz * dz);
      const double rm1 = sqrt(rm2);
      const double w = rm2 * (dx * fj[0] + dy * fj[1] + dz * fj[2]);
      v[0] += rm1 * (fj[0] + dx * w);
      v[1] += rm1 * (fj[1] + dy * w);
      v[2] += rm1 * (fj[2] + dz * w);
      if (blobs_per_body == 0) {
        /* Blakelet correction for a no-slip wall at z = 0 (:83-116): minus the
         * image Stokeslet, plus the source-doublet/stresslet terms. */
        const double Rz = zi + xj[2];
        const double R2 = dx * dx + dy * dy + Rz * Rz;
        const double Rm1 = sqrt(1.0 / R2);
        const double W = (dx * fj[0] + dy * fj[1] + Rz * fj[2]) * Rm1 * Rm1;
        v[0] -= Rm1 * (fj[0] + dx * W);
        v[1] -= Rm1 * (fj[1] + dy * W);
        v[2] -= Rm1 * (fj[2] + Rz * W);
        const double Dxx = (3.0 * dx * dx - R2) * zi;
        const double Dxy = 3.0 * dx * dy * zi;
        const double Dxz = (R2 - 3.0 * Rz * zi) * dx;
        const double Dyy = (3.0 * dy * dy - R2) * zi;
        const double Dyz = (R2 - 3.0 * Rz * zi) * dy;
        const double Dzx = (3.0 * Rz * zi + R2) * dx;
        const double Dzy = (3.0 * Rz * zi + R2) * dy;
        const double Dzz = (R2 - 3.0 * Rz * Rz) * zi;
        const double Dfac = 2.0 * xj[2] * Rm1 * Rm1 * Rm1 * Rm1 * Rm1;
        v[0] += Dfac * (Dxx * fj[0] + Dxy * fj[1] + Dxz * fj[2]);
        v[1] += Dfac * (Dxy * fj[0] + Dyy * fj[1] + Dyz * fj[2]);
        v[2] += Dfac * (Dzx * fj[0] + Dzy * fj[1] + Dzz * fj[2]);
      }
      /* Rotlet (:118-123) */
      const double rm3 = rm1 * rm2;
      v[0] += rm3 * (fj[4] * dz - fj[5] * dy);
      v[1] += rm3 * (fj[5] * dx - fj[3] * dz);
      v[2] += rm3 * (fj[3] * dy - fj[4] * dx);
      if (remove_net_force) {
        /* (:125-143) */
        const double *xb = x_bodies + 3 * (size_t)(j / segs_per_body);
        orc_stokeslet(v, xi - xb[0], yi - xb[1], zi - xb[2], fj, -1.0);
      }
    }
    for (int j = 0; j < nb; ++j) {
      const double *xj = x_blobs + 3 * (size_t)j;
      const double *fj = f_blobs + 3 * (size_t)j;
      orc_stokeslet(v, xi - xj[0], yi - xj[1], zi - xj[2], fj, 1.0); /* :177-187 */
      if (remove_net_force) {
        const double *xb = x_bodies + 3 * (size_t)(j / blobs_per_body);
        orc_stokeslet(v, xi - xb[0], yi - xb[1], zi - xb[2], fj, -1.0);
      }
    }
    v_flow[3 * (size_t)i] = prefac * v[0];
    v_flow[3 * (size_t)i + 1] = prefac * v[1];
    v_flow[3 * (size_t)i + 2] = prefac * v[2];
  }
}
