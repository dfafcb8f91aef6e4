// cuda_emu.hpp -- host emulation of the CUDA C++ dialect used by the
// reference's kernel file, so that the reference's own kernels can be
// compiled unchanged by g++ and run on the CPU as a parity pin.
//
// TEST INFRASTRUCTURE ONLY: this header is force-included (-include) when
// oracle/Makefile compiles the reference sources in place; nothing in the
// product library includes it.
//
// Model: one CUDA thread = one std::thread; one thread block runs at a time,
// so `__shared__` arrays become function-local statics shared by the threads
// of the running block, and `__syncthreads()` is a std::barrier over those
// threads. Blocks run one after another in blockIdx order.
#pragma once
#include <barrier>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <thread>
#include <vector>

using std::abs;
using std::fmin;
using std::sqrt;

struct uint3_emu {
  unsigned int x = 0, y = 0, z = 0;
};
struct dim3 {
  unsigned int x = 1, y = 1, z = 1;
  dim3() = default;
  dim3(unsigned int x_, unsigned int y_ = 1, unsigned int z_ = 1) : x(x_), y(y_), z(z_) {}
};

#define __global__
#define __device__
#define __host__
#define __forceinline__ inline
#define __shared__ static

extern thread_local uint3_emu threadIdx;
extern thread_local uint3_emu blockIdx;
extern dim3 blockDim;
extern dim3 gridDim;

void __syncthreads();

// Only referenced by reference code paths that are not compiled in or not
// run (wall-bounded RPY, weakly-coupled filaments); provided so they compile.
inline double rsqrt(double x) { return 1.0 / std::sqrt(x); }
inline float rsqrt(float x) { return 1.0f / std::sqrt(x); }
inline long long __double_as_longlong(double d) {
  long long r;
  std::memcpy(&r, &d, sizeof r);
  return r;
}
inline double __longlong_as_double(long long l) {
  double r;
  std::memcpy(&r, &l, sizeof r);
  return r;
}
unsigned long long atomicCAS(unsigned long long *address, unsigned long long compare,
                             unsigned long long val);

// Launch `body` as a <<<grid, block>>> kernel, one block at a time.
void emu_launch(int grid, int block, const std::function<void()> &body);
