// ref_flow_harness.cpp -- runs the reference's flow_velocities kernel
// (src/flow_field/flow_field_evaluator.cu:13-228) on the CPU.
//
// TEST INFRASTRUCTURE ONLY. The kernel text is cut out of the reference file
// by oracle/Makefile at build time (the rest of that file does not compile
// as shipped: flow_field_evaluator.hpp:21-23 collides with config.hpp macros)
// and included here under cuda_emu.hpp; nothing of it is committed.
#include "cuda_emu.hpp"

typedef double Real;
#define THREADS_PER_BLOCK 64

#include "flow_velocities_kernel.inc"

extern "C" void ref_flow_velocities(double *v_flow, const double *x_flow, const double *f_segs,
                                    const double *f_blobs, const double *x_segs,
                                    const double *x_bodies, const double *x_blobs, int num_flow,
                                    int segs_per_body, int num_bodies, int blobs_per_body,
                                    double prefac, int remove_net_force) {
  const int blocks = (num_flow + THREADS_PER_BLOCK - 1) / THREADS_PER_BLOCK;
  emu_launch(blocks, THREADS_PER_BLOCK, [&] {
    flow_velocities(v_flow, x_flow, f_segs, f_blobs, x_segs, x_bodies, x_blobs, num_flow,
                    segs_per_body, num_bodies, blobs_per_body, prefac, remove_net_force);
  });
}
