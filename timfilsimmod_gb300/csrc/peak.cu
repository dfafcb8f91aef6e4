// peak.cu -- FMA-throughput microbenchmark (the roofline denominator for the
// FP64 and FP32 pair kernels; the measured-peaks file of the GPU pool has no
// FP32/FP64 FMA figure).
#include <cuda_runtime.h>

#include "../../include/tfs_gb300.h"
#include "tfs_device.cuh"
#include "tfs_kernels.h"

namespace tfs {
int fail(int code, const char *fmt, ...);
int cuda_fail(cudaError_t e, const char *what);

// Each thread runs kChains independent FMA chains of `iters` steps; the
// multiplier is data dependent so nothing folds at compile time.
template <typename T>
__global__ void __launch_bounds__(256) fma_chain_kernel(T *out, int iters, T m) {
  constexpr int kChains = 8;
  T a[kChains];
#pragma unroll
  for (int k = 0; k < kChains; ++k) a[k] = T(threadIdx.x + k);
  const T c = T(1e-7) * m;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int k = 0; k < kChains; ++k) a[k] = fma(a[k], m, c);
  }
  T s = 0;
#pragma unroll
  for (int k = 0; k < kChains; ++k) s += a[k];
  if (s == T(-12345.678)) out[0] = s;  // keep the chains live
}
}  // namespace tfs

using namespace tfs;

extern "C" int tfs_measure_fma_peak(int precision, double *flops_per_second) {
  if (flops_per_second == nullptr) return fail(TFS_EINVAL, "null output");
  const int blocks = num_sms() * 8, threads = 256;
  const int iters = precision == TFS_FP64 ? 2048 : 65536;
  void *buf = nullptr;
  cudaError_t e = cudaMalloc(&buf, 64);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc");
  cudaEvent_t t0, t1;
  cudaEventCreate(&t0);
  cudaEventCreate(&t1);
  float best_ms = 1e30f;
  for (int rep = 0; rep < 4; ++rep) {
    cudaEventRecord(t0);
    if (precision == TFS_FP64)
      fma_chain_kernel<double><<<blocks, threads>>>((double *)buf, iters, 0.9999999);
    else
      fma_chain_kernel<float><<<blocks, threads>>>((float *)buf, iters, 0.9999999f);
    count_launch();
    cudaEventRecord(t1);
    e = cudaEventSynchronize(t1);
    if (e != cudaSuccess) break;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, t0, t1);
    if (rep > 0 && ms < best_ms) best_ms = ms;  // rep 0 is warm-up
  }
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  cudaFree(buf);
  if (e != cudaSuccess) return cuda_fail(e, "FMA microbenchmark");
  const double flops = 2.0 * 8.0 * (double)iters * blocks * threads;
  *flops_per_second = flops / (best_ms * 1e-3);
  return TFS_OK;
}

// ---------------------------------------------------------------------------
// The FP64 reciprocal square root of far-field separations (rsqrt_far), on a
// device array, for accuracy tests against CUDA's rsqrt and a host reference.
// ---------------------------------------------------------------------------
namespace {
__global__ void rsqrt_far_kernel(const double *__restrict__ x, double *__restrict__ y, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = tfs::rsqrt_far(x[i]);
}
}  // namespace

extern "C" int tfs_rsqrt_far(const double *x, double *y, int n, void *stream) {
  using namespace tfs;
  if (n < 0) return fail(TFS_EINVAL, "negative count");
  if (n == 0) return TFS_OK;
  if (x == nullptr || y == nullptr) return fail(TFS_EINVAL, "null device pointer");
  rsqrt_far_kernel<<<(n + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(x, y, n);
  count_launch();
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "rsqrt_far kernel");
  return TFS_OK;
}
