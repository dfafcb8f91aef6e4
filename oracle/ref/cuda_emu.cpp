// cuda_emu.cpp -- runtime half of cuda_emu.hpp (test infrastructure only).
#include "cuda_emu.hpp"

#include <mutex>

thread_local uint3_emu threadIdx;
thread_local uint3_emu blockIdx;
dim3 blockDim;
dim3 gridDim;

static std::barrier<> *g_block_barrier = nullptr;
static std::mutex g_atomic_mutex;

void __syncthreads() { g_block_barrier->arrive_and_wait(); }

unsigned long long atomicCAS(unsigned long long *address, unsigned long long compare,
                             unsigned long long val) {
  std::lock_guard<std::mutex> lock(g_atomic_mutex);
  const unsigned long long old = *address;
  if (old == compare) *address = val;
  return old;
}

void emu_launch(int grid, int block, const std::function<void()> &body) {
  gridDim = dim3(grid);
  blockDim = dim3(block);
  for (int b = 0; b < grid; ++b) {
    std::barrier<> bar(block);
    g_block_barrier = &bar;
    std::vector<std::thread> threads;
    threads.reserve(block);
    for (int t = 0; t < block; ++t) {
      threads.emplace_back([&body, b, t] {
        threadIdx.x = t;
        blockIdx.x = b;
        body();
      });
    }
    for (auto &th : threads) th.join();
    g_block_barrier = nullptr;
  }
}
