// flow_field_evaluator_gb300.cpp -- flow_field_evaluator::velocities for the
// reference's flow-field program (src/flow_field/flow_field_evaluator.{hpp,cu},
// velocities :546-579, kernel flow_velocities :13-228), backed by
// libtfs_gb300.so. It replaces that one member; setup and
// read_positions_and_forces (file reading into the host arrays) stay the
// reference's. The library's flow evaluator is created on the first call,
// sized from the evaluator's own counts.
//
// The reference's header does not compile as shipped: its members MU, RSEG
// and DT collide with the macros of config.hpp (pulled in through
// matrix.hpp). The shim includes matrix.hpp first and removes those three
// macros before the evaluator's header, changing nothing in either file.
#include <vector>

#include "matrix.hpp"
#undef MU
#undef RSEG
#undef DT
#include "flow_field_evaluator.hpp"
#include "tfs_shim.hpp"

namespace {
tfs_flow *g_flow = nullptr;

std::vector<double> widen(const Real *p, size_t n) {
  return p ? std::vector<double>(p, p + n) : std::vector<double>();
}
}  // namespace

void flow_field_evaluator::velocities() {
  const size_t nsegs = (size_t)NBOD * NFIL * NSEG, nblobs = (size_t)NBOD * NBLOB;
  if (g_flow == nullptr)
    tfs_check(tfs_flow_create(NFLOW, NBOD, NFIL * NSEG, NBLOB, TFS_FP64, &g_flow));
  // the library takes float64 host arrays; Real = float is widened here
  const std::vector<double> xf = widen(x_flow_host, 3 * (size_t)NFLOW),
                            xs = widen(x_segs_host, 3 * nsegs), fs = widen(f_segs_host, 6 * nsegs),
                            xb = widen(NBLOB ? x_blobs_host : nullptr, 3 * nblobs),
                            fb = widen(NBLOB ? f_blobs_host : nullptr, 3 * nblobs),
                            xo = widen(x_bods_host, 3 * (size_t)NBOD);
  tfs_check(tfs_flow_copy_inputs_to_device(g_flow, xf.data(), xs.data(), fs.data(),
                                           NBLOB ? xb.data() : nullptr,
                                           NBLOB ? fb.data() : nullptr, xo.data()));
  tfs_check(tfs_flow_velocities(g_flow, MU, REMOVE_NET_FORCE_STOKESLET ? 1 : 0));
  std::vector<double> v(3 * (size_t)NFLOW);
  tfs_check(tfs_flow_copy_velocities_to_host(g_flow, v.data()));
  for (size_t i = 0; i < v.size(); ++i) v_flow_host[i] = (Real)v[i];
}
