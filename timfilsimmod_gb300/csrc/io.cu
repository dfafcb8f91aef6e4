// io.cu -- the reference's data files for the implicit step: the text records
// a plot step writes (cilia_sim_main.cu:563-600 with swimmer::write_data,
// rigid_body::write_data, filament::write_data and
// mobility_solver::write_data, mobility_solver.cpp:3051-3173) and the backup
// it overwrites (swimmer::write_backup), and resuming from such a backup
// (cilia_sim_main.cu:118-166, 336-350). Numbers are written as the reference's
// streams write them: std::scientific with 10 digits after the point (the
// printf form %.10e), space separated with a trailing space, one record per
// line, step numbers as plain integers.
#include <cuda_runtime.h>

#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "tfs_solver.h"

using tfs::fail;

namespace tfs {
size_t backup_values(const tfs_stepper *st);
int stepper_backup(tfs_stepper *st, std::vector<double> &out);
int stepper_load(tfs_stepper *st, const double *v);
int stepper_internal_forces(tfs_stepper *st, double *f);
int stepper_dims(const tfs_stepper *st, int *nfil, int *nseg);
tfs_solver *stepper_solver(tfs_stepper *st);
}  // namespace tfs

namespace {

struct File {
  FILE *f = nullptr;
  File(const std::string &path, const char *mode) : f(std::fopen(path.c_str(), mode)) {}
  ~File() {
    if (f) std::fclose(f);
  }
};

void put(FILE *f, double v) { std::fprintf(f, "%.10e ", v); }

}  // namespace

extern "C" {

int tfs_stepper_backup_size(tfs_stepper *st, size_t *n) {
  if (st == nullptr || n == nullptr) return fail(TFS_EINVAL, "null argument");
  *n = tfs::backup_values(st);
  return TFS_OK;
}

int tfs_stepper_get_backup(tfs_stepper *st, double *values) {
  if (st == nullptr || values == nullptr) return fail(TFS_EINVAL, "null argument");
  std::vector<double> v;
  int rc = tfs::stepper_backup(st, v);
  if (rc != TFS_OK) return rc;
  std::memcpy(values, v.data(), sizeof(double) * v.size());
  return TFS_OK;
}

int tfs_stepper_set_backup(tfs_stepper *st, const double *values) {
  if (st == nullptr || values == nullptr) return fail(TFS_EINVAL, "null argument");
  return tfs::stepper_load(st, values);
}

int tfs_stepper_write_backup(tfs_stepper *st, int save_step, const char *path) {
  if (st == nullptr || path == nullptr) return fail(TFS_EINVAL, "null argument");
  std::vector<double> v;
  int rc = tfs::stepper_backup(st, v);
  if (rc != TFS_OK) return rc;
  File out(path, "w");
  if (!out.f) return fail(TFS_EINVAL, "cannot write %s: %s", path, std::strerror(errno));
  std::fprintf(out.f, "%d ", save_step);
  for (double x : v) put(out.f, x);
  std::fprintf(out.f, "\n");
  return std::ferror(out.f) ? fail(TFS_EINVAL, "write error on %s", path) : TFS_OK;
}

int tfs_stepper_read_backup(tfs_stepper *st, const char *path, int *save_step) {
  if (st == nullptr || path == nullptr) return fail(TFS_EINVAL, "null argument");
  File in(path, "r");
  if (!in.f) return fail(TFS_EINVAL, "cannot read %s: %s", path, std::strerror(errno));
  int step = 0;
  if (std::fscanf(in.f, "%d", &step) != 1) return fail(TFS_EINVAL, "%s: no step number", path);
  const size_t n = tfs::backup_values(st);
  std::vector<double> v(n);
  for (size_t i = 0; i < n; ++i)
    if (std::fscanf(in.f, "%lf", &v[i]) != 1)
      return fail(TFS_EINVAL, "%s: %zu numbers after the step, expected %zu", path, i, n);
  double extra;
  if (std::fscanf(in.f, "%lf", &extra) == 1)
    return fail(TFS_EINVAL, "%s: more than the %zu numbers of this swimmer", path, n);
  int rc = tfs::stepper_load(st, v.data());
  if (rc != TFS_OK) return rc;
  if (save_step) *save_step = step;
  return TFS_OK;
}

int tfs_stepper_write_files(tfs_stepper *st, int nt, const char *prefix, int backup) {
  if (st == nullptr || prefix == nullptr) return fail(TFS_EINVAL, "null argument");
  tfs_solver *s = tfs::stepper_solver(st);
  int nfil = 0, nseg = 0;
  tfs::stepper_dims(st, &nfil, &nseg);
  const size_t ns = (size_t)nfil * nseg, nb = (size_t)s->nb;
  const int save_step = nt + 1;  // the implicit description
  std::vector<double> v;
  int rc = tfs::stepper_backup(st, v);
  if (rc != TFS_OK) return rc;
  std::vector<double> vs(6 * ns), fb(3 * nb), fs(6 * ns);
  double vb[6];
  if ((rc = tfs_copy_segment_velocities_to_host(s, vs.data())) != TFS_OK) return rc;
  if ((rc = tfs_copy_blob_forces_to_host(s, fb.data())) != TFS_OK) return rc;
  if ((rc = tfs_wait_for_device(s)) != TFS_OK) return rc;
  if ((rc = tfs_get_body_velocities(s, vb)) != TFS_OK) return rc;
  if ((rc = tfs::stepper_internal_forces(st, fs.data())) != TFS_OK) return rc;
  const std::string p(prefix);
  const size_t per_fil = 9 + 28 * (size_t)nseg, body0 = (size_t)nfil * per_fil;
  {
    File f(p + "_seg_states.dat", "a"), b(p + "_body_states.dat", "a"), t(p + "_tether_force.dat", "a");
    if (!f.f || !b.f || !t.f) return fail(TFS_EINVAL, "cannot append to the %s_*.dat files", prefix);
    std::fprintf(f.f, "%d ", save_step);
    std::fprintf(b.f, "%d ", save_step);
    std::fprintf(t.f, "%d ", save_step);
    for (int k = 0; k < 3; ++k) put(b.f, v[body0 + 4 + k]);  // body x, then q
    for (int k = 0; k < 4; ++k) put(b.f, v[body0 + k]);
    for (int i = 0; i < nfil; ++i) {
      const double *r = &v[i * per_fil];
      for (int j = 0; j < nseg; ++j)
        for (int k = 0; k < 4; ++k) put(f.f, r[19 * j + k]);
      for (int k = 0; k < 3; ++k) put(t.f, r[19 * nseg + k]);
    }
    std::fprintf(f.f, "\n");
    std::fprintf(b.f, "\n");
    std::fprintf(t.f, "\n");
  }
  {
    File bv(p + "_body_vels.dat", "a"), bf(p + "_blob_forces.dat", "a"), sv(p + "_seg_vels.dat", "a"),
        sf(p + "_seg_forces.dat", "a");
    if (!bv.f || !bf.f || !sv.f || !sf.f) return fail(TFS_EINVAL, "cannot append to the %s_*.dat files", prefix);
    std::fprintf(bf.f, "%d ", nt);
    std::fprintf(sv.f, "%d ", nt);
    std::fprintf(sf.f, "%d ", nt);
    for (int k = 0; k < 6; ++k) put(bv.f, vb[k]);
    for (size_t i = 0; i < 3 * nb; ++i) put(bf.f, fb[i]);
    for (size_t i = 0; i < 6 * ns; ++i) {
      put(sv.f, vs[i]);
      put(sf.f, fs[i]);
    }
    std::fprintf(bv.f, "\n");
    std::fprintf(bf.f, "\n");
    std::fprintf(sv.f, "\n");
    std::fprintf(sf.f, "\n");
  }
  if (backup) return tfs_stepper_write_backup(st, save_step, (p + ".backup").c_str());
  return TFS_OK;
}

}  // extern "C"
