// TEST INFRASTRUCTURE ONLY.  A CPU executor for CUDA kernels compiled as
// plain C++: the grid's blocks run one after another (so function-local
// statics stand in for __shared__ arrays), and each block runs blockDim
// std::threads that meet at __syncthreads() through a barrier which stops
// counting a thread once it has returned from the kernel, as CUDA does.
#pragma once
#include <condition_variable>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

struct uint3;
struct dim3;

namespace emu {

struct Barrier {
  std::mutex m;
  std::condition_variable cv;
  int active = 0, arrived = 0;
  unsigned long long gen = 0;
  void reset(int n) {
    std::lock_guard<std::mutex> l(m);
    active = n;
    arrived = 0;
  }
  void sync() {
    std::unique_lock<std::mutex> l(m);
    const unsigned long long g = gen;
    if (++arrived == active) {
      arrived = 0;
      ++gen;
      cv.notify_all();
    } else {
      cv.wait(l, [&] { return gen != g; });
    }
  }
  void retire() {
    std::lock_guard<std::mutex> l(m);
    --active;
    if (arrived > 0 && arrived == active) {
      arrived = 0;
      ++gen;
      cv.notify_all();
    }
  }
};

inline Barrier &block_barrier() {
  static Barrier b;
  return b;
}

}  // namespace emu

struct EmuIdx {
  unsigned x, y, z;
};
extern thread_local EmuIdx threadIdx;
extern EmuIdx blockIdx, blockDim, gridDim;

inline void __syncthreads() { emu::block_barrier().sync(); }

namespace emu {

// Run `body` (a call of the kernel with its arguments) over grid x block.
inline void launch(unsigned gx, unsigned gy, unsigned bx, unsigned by,
                   const std::function<void()> &body) {
  const int nthr = int(bx * by);
  blockDim = {bx, by, 1};
  gridDim = {gx, gy, 1};
  Barrier &bar = block_barrier();
  const unsigned long long nblocks = (unsigned long long)gx * gy;
  Barrier start, finish;
  start.reset(nthr + 1);
  finish.reset(nthr + 1);
  std::vector<std::thread> threads;
  threads.reserve(nthr);
  for (int t = 0; t < nthr; ++t) {
    threads.emplace_back([&, t] {
      threadIdx = {unsigned(t) % bx, unsigned(t) / bx, 0};
      for (unsigned long long b = 0; b < nblocks; ++b) {
        start.sync();
        body();
        bar.retire();
        finish.sync();
      }
    });
  }
  for (unsigned long long b = 0; b < nblocks; ++b) {
    blockIdx = {unsigned(b % gx), unsigned(b / gx), 0};
    bar.reset(nthr);
    start.sync();
    finish.sync();
  }
  for (auto &th : threads) th.join();
}

}  // namespace emu
