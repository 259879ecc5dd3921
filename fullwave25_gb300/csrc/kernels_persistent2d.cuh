// Persistent 2D step kernel: one cooperative launch advances a simulation by many time steps.
//
// Small 2D grids (the plain 2D workload is 944 x 688 cells, a 60 MB working set) sit in L2, and
// a time step there takes a few microseconds of work per kernel; with two launches per step the
// gaps between dependent launches cost as much as the work. Here every block of a cooperative
// launch (all blocks co-resident) owns a fixed set of the 32 (y) x 8 (x) tiles and runs
//   for each step: velocity of its tiles | grid barrier | pressure + epilogue of its tiles |
//                  grid barrier
// with the same cell bodies as the direct kernels (bit-identical results). p and v change inside
// the launch, so their stencil reads use coherent loads instead of the read-only path.
//
// The grid barrier lives in a small per-handle buffer (zeroed before each launch): a generation
// word and one arrival counter. Every spin is bounded by %globaltimer; a block that gives up sets
// status bit 4, and every block leaves the step loop at its next barrier.
//
// One flat counter measured faster than a two-level arrival tree on GB300 at every block count
// (152 / 304 / 608 / 1216 blocks: 2.1 / 2.2 / 2.5 / 3.8 us per barrier against 3.4 / 3.6 / 4.0 /
// 6.4 us for a tree of groups of 16): the cost is the latency of the atomics and of the
// generation's visibility across the chip, not contention on the counter.
#pragma once
#include "engine_common.cuh"
#include "kernels_direct.cuh"
#include "tma.cuh"

namespace fwgb {

constexpr uint64_t kGridBarrierTimeoutNs = 1000000000ull;   // 1 s
constexpr int kBarWords = 2;                  // generation, arrival counter
constexpr int kBarMaxBlocks = 2048;

__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Returns false when the launch must stop (a barrier wait timed out somewhere).
__device__ __forceinline__ bool grid_barrier(unsigned* bar, int* status, unsigned n_blocks) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    unsigned* gen = bar;
    unsigned* cnt = bar + 1;
    volatile int* vstatus = status;
    // the generation cannot advance before this block arrives, so reading it first is safe
    const unsigned g0 = ld_acquire_gpu(gen);
    int ok = 1;
    __threadfence();   // the block's writes (ordered before this thread by __syncthreads)
    unsigned old;
    asm volatile("atom.add.acq_rel.gpu.global.u32 %0, [%1], 1;" : "=r"(old) : "l"(cnt) : "memory");
    if (old == n_blocks - 1) {
      *cnt = 0;        // ordered before the release below; no block arrives again before it
      asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(gen) : "memory");
    } else {
      const uint64_t t0 = global_timer_ns();
      unsigned it = 0;
      while (ld_acquire_gpu(gen) == g0) {
        if ((++it & 63u) == 0 &&
            ((*vstatus & 4) || global_timer_ns() - t0 > kGridBarrierTimeoutNs)) {
          atomicOr(status, 4);
          ok = 0;
          break;
        }
      }
    }
    __threadfence();
    s_ok = ok && !(*vstatus & 4);
  }
  __syncthreads();
  return s_ok;
}

// grid = blocks of (32, 8) threads, each owning tiles blockIdx.x + k * gridDim.x; n_tiles and
// n_ty (tiles along y) describe the 32 x 8 tiling; steps n0 .. n0 + n_steps - 1.
template <class CV, class CP>
__global__ void __launch_bounds__(256)
step2d_persistent(const StepArgs A, unsigned* bar, int n0, int n_steps, int n_tiles, int n_ty) {
  int* status = A.step + 1;
  for (int s = 0; s < n_steps; ++s) {
    const int n = n0 + s;
    if (blockIdx.x == 0 && threadIdx.x == 0 && threadIdx.y == 0) *A.step = n + 1;
    for (int t = blockIdx.x; t < n_tiles; t += gridDim.x)
      vel2d_body<CV, true>(A, t % n_ty, t / n_ty);
    if (!grid_barrier(bar, status, gridDim.x)) return;
    for (int t = blockIdx.x; t < n_tiles; t += gridDim.x)
      prs2d_body<CP, true>(A, t % n_ty, t / n_ty, t, n);
    if (!grid_barrier(bar, status, gridDim.x)) return;
  }
}

}  // namespace fwgb
