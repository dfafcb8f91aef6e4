// rpy_queue.cu -- host side of the work-queue products (rpy_queue.cuh):
// source chunking, grid sizing and the launch.
#include <cuda_runtime.h>

#include <algorithm>

#include "tfs_kernels.h"

namespace tfs {

void queue_chunking(int n_src, int n_particles, int *chunk, int *n_chunks) {
  if (n_src <= 0) {
    *chunk = kQueueQuantum;
    *n_chunks = 0;
    return;
  }
  constexpr long kUnits = 8192;  // units of 128 targets over the whole system
  const long blocks = std::max(1L, ((long)n_particles + 127) / 128);
  const long want = std::max(1L, std::min<long>(kMaxSplits, (kUnits + blocks - 1) / blocks));
  long c = ((long)n_src + want - 1) / want;
  c = ((c + kQueueQuantum - 1) / kQueueQuantum) * kQueueQuantum;
  *chunk = (int)c;
  *n_chunks = (int)(((long)n_src + c - 1) / c);
}

long long queue_units(const QueueJob *jobs_host, int n_jobs, int block_targets) {
  long long u = 0;
  for (int j = 0; j < n_jobs; ++j)
    u += (long long)((jobs_host[j].n_tgt + block_targets - 1) / block_targets) *
         jobs_host[j].n_chunks;
  return u;
}

cudaError_t launch_queue(int fp32, int variant, int sources, const QueueJob *jobs,
                         const QueueJob *jobs_host, int n_jobs, unsigned *counters,
                         cudaStream_t st, cudaEvent_t *ev) {
  if (sources < 0 || sources >= kNumQueueSources || n_jobs < 0 || n_jobs > kQueueMaxJobs)
    return cudaErrorInvalidValue;
  const int nvar = fp32 ? kNumQueueVariantsF32 : kNumQueueVariantsF64;
  if (variant < 0 || variant >= nvar) variant = 0;
  const QueueVariant var = fp32 ? g_qvariants_f32[variant] : g_qvariants_f64[variant];
  const QueueFn fn = fp32 ? g_queue_f32[variant][sources] : g_queue_f64[variant][sources];
  const long long units = queue_units(jobs_host, n_jobs, var.block * var.tpt);
  if (units <= 0) return cudaSuccess;
  int resident = 1;
  cudaError_t e = fn(QueueArgs{}, 0, st, &resident);
  if (e != cudaSuccess) return e;
  const long long slots = (long long)resident * num_sms();
  const int ctas = (int)std::min(slots, units);
  if (ev) cudaEventRecord(ev[0], st);
  e = fn(QueueArgs{jobs, n_jobs, counters}, ctas, st, nullptr);
  count_launch();
  if (ev) cudaEventRecord(ev[1], st);
  return e;
}

}  // namespace tfs
