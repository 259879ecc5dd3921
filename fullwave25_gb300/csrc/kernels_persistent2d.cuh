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
// The grid barrier lives in a small per-handle buffer of counters (zeroed before each launch).
// Every spin is bounded by %globaltimer; a block that gives up sets status bit 4, and every block
// leaves the step loop at its next barrier.
#pragma once
#include "engine_common.cuh"
#include "kernels_direct.cuh"
#include "tma.cuh"

namespace fwgb {

constexpr uint64_t kGridBarrierTimeoutNs = 1000000000ull;   // 1 s

// Barrier words (zeroed before each launch): gen, root counter, then one arrival counter per
// group of kBarGroup blocks. Arrival is a two-level tree (a block counts in at its group, the
// group's last block counts the group in at the root, the root's last arrival bumps the
// generation), so no counter sees more than kBarGroup arrivals; waiters poll the generation with
// a short sleep between reads.
constexpr int kBarGroup = 16;
constexpr int kBarMaxGroups = 128;            // up to 2048 blocks
constexpr int kBarWords = 2 + kBarMaxGroups;

// Returns false when the launch must stop (a barrier wait timed out somewhere).
__device__ __forceinline__ bool grid_barrier(unsigned* bar, int* status, unsigned n_blocks) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    unsigned* gen = bar;
    unsigned* root = bar + 1;
    const unsigned grp = blockIdx.x / kBarGroup;
    const unsigned n_groups = (n_blocks + kBarGroup - 1) / kBarGroup;
    const unsigned grp_size = min((unsigned)kBarGroup, n_blocks - grp * kBarGroup);
    volatile unsigned* vgen = gen;
    volatile int* vstatus = status;
    const unsigned g0 = *vgen;
    int ok = 1;
    __threadfence();
    bool waiting = true;
    if (atomicAdd(bar + 2 + grp, 1u) == grp_size - 1) {
      atomicExch(bar + 2 + grp, 0u);
      __threadfence();
      if (atomicAdd(root, 1u) == n_groups - 1) {
        atomicExch(root, 0u);
        __threadfence();
        atomicAdd(gen, 1u);
        waiting = false;
      }
    }
    if (waiting) {
      const uint64_t t0 = global_timer_ns();
      while (*vgen == g0) {
        if ((*vstatus & 4) || global_timer_ns() - t0 > kGridBarrierTimeoutNs) {
          atomicOr(status, 4);
          ok = 0;
          break;
        }
        __nanosleep(32);
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
