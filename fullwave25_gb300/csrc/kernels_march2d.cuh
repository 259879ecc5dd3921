// 2D step kernels that march along x (depth, the slow axis).
//
// Block = TY threads, one per y column (y is contiguous), walking XC consecutive x rows. Per row:
//   * x taps come from a 16-entry register queue of the thread's column (one new coalesced load
//     per row, prefetched one row ahead);
//   * y taps and the off-axis taps come from shared-memory copies of rows x-1, x, x+1 with the y
//     halo they need, brought in by TMA (2D tiled loads) into a 4-slot ring, row x+2 in flight
//     while row x is computed; one mbarrier per slot, bounded waits;
//   * the point-wise state and maps of the cell are loaded before the row barrier and written
//     once, coalesced.
// Same arithmetic (operation order, fused multiply-adds) as the 2D direct kernels, so the results
// are bit-identical to theirs. The per-tile source/air/sensor lists stay those of the direct
// kernels' 32 (y) x 8 (x) tiles: TY is a multiple of 32 and XC of 8, so a march block owns a
// rectangle of list tiles and the tile shape can change without rebuilding the lists.
#pragma once
#include "engine_common.cuh"
#include "kernels_direct.cuh"
#include "kernels_persistent2d.cuh"
#include "tma.cuh"

namespace fwgb {

constexpr int kRing2 = 4;

// Row boxes: p and vy with a y halo of 8 (start y0 - 8), vx with a halo of 4 (start y0 - 4).
template <int TY>
struct Row2 {
  static constexpr int kWide = TY + 16;   // floats, multiple of 4
  static constexpr int kNarrow = TY + 8;
  static constexpr int kWideSlot = (kWide * 4 + 127) / 128 * 32;   // floats, 128-byte aligned
  static constexpr int kNarrowSlot = (kNarrow * 4 + 127) / 128 * 32;
};

// Tensor maps of one 2D simulation for the row-march kernels: the three halo-row maps, then the
// point-wise maps of the streaming bodies (isotropic engine): 3D boxes {TY, 1, F} over the state
// and map allocations (fields stacked on the third axis) and the tap-index map.
struct March2Maps {
  CUtensorMap p, vx, vy;        // halo rows
  CUtensorMap vst, vmp;         // velocity: v_x v_y psi_x1 psi_x2 psi_y1 psi_y2 | rdt_rho .. bu2
  CUtensorMap pp, phi;          // pressure: p | phi_x1 phi_x2 phi_y1 phi_y2
  CUtensorMap pmp6, pmp7;       // pressure maps dt_k .. bx2 (+ beta2dt)
  CUtensorMap dc;               // int32 tap index
};
constexpr int kMarch2Maps = sizeof(March2Maps) / sizeof(CUtensorMap);   // 10

// Point-wise field counts of the streaming 2D bodies and their first fields in the stacks.
constexpr int kV2StateF = 6, kV2MapF = 6, kP2PhiF = 4;
constexpr int kState2V0 = 1, kState2Phi0 = 7;

// Column-queue load: the read-only path, or (kPersist: the field changes inside the launch) a load
// that bypasses L1 and reads the coherent L2.
template <bool kPersist>
__device__ __forceinline__ float ld_col(const float* q) {
  if constexpr (kPersist) return __ldcg(q);
  else return __ldg(q);
}

__device__ __forceinline__ void tma_load_3d_row(void* dst, const CUtensorMap* map, uint64_t* bar,
                                                int y, int x, int f) {
  tma_load_3d(dst, map, bar, y, x, f);
}

// Bodies take the block's y block (by) and x chunk (bx) explicitly and the tensor maps by address
// (kernel parameters or global memory), so that the single-simulation kernels and the group
// kernels (block from a work list, one argument block and map set per simulation) share them.
// kStream (isotropic engine): the point-wise operands of a row come by TMA too — state, maps and
// tap index of row x+1 are in flight (two-stage ring) while row x is computed; the cell update
// is CellVelT's / CellPrsT's, so results stay bit-identical.
// kPersist: the body runs many times inside one launch (the persistent group kernel), where p and
// v change between calls: the column queues load from L2 instead of the read-only path,
// the ring is refilled only after a proxy fence (its slots were read by the previous call), and
// the mbarriers are invalidated at the end so the next call can initialise them again.
// Shared memory of one row-march body (the kernels declare it; the persistent group kernel
// overlays the velocity and pressure bodies' in a union).
template <int TY, bool kStream>
struct VelMarchSmem {
  alignas(128) float ring[kRing2][Row2<TY>::kWideSlot];
  alignas(128) float pst[kStream ? 2 : 1][kStream ? kV2StateF : 1][kStream ? TY : 1];
  alignas(128) float pmp[kStream ? 2 : 1][kStream ? kV2MapF : 1][kStream ? TY : 1];
  alignas(128) uint16_t pdc[kStream ? 2 : 1][kStream ? TY : 1];
  alignas(8) uint64_t bar[kRing2];
  alignas(8) uint64_t pbar[2];
};
template <int TY, bool kStream, bool kBeta>
struct PrsMarchSmem {
  static constexpr int kMapF = kV2MapF + (kBeta ? 1 : 0);
  alignas(128) float rx[kRing2][Row2<TY>::kNarrowSlot];
  alignas(128) float ry[kRing2][Row2<TY>::kWideSlot];
  alignas(128) float ppp[kStream ? 2 : 1][kStream ? TY : 1];
  alignas(128) float pph[kStream ? 2 : 1][kStream ? kP2PhiF : 1][kStream ? TY : 1];
  alignas(128) float pmp[kStream ? 2 : 1][kStream ? kMapF : 1][kStream ? TY : 1];
  alignas(128) uint16_t pdc[kStream ? 2 : 1][kStream ? TY : 1];
  alignas(8) uint64_t bar[kRing2];
  alignas(8) uint64_t pbar[2];
};

template <int TY, int XC, class CV, bool kStream = false, int kMapSlotVel = 0,
          bool kPersist = false>
__device__ __forceinline__ void vel2d_march_body(VelMarchSmem<TY, kStream>& S, const StepArgs& A,
                                                 const March2Maps* tm, int by, int bx) {
  using R = Row2<TY>;
  const CUtensorMap* tm_p = &tm->p;
  auto& ring = S.ring;
  auto& bar = S.bar;
  auto& pst = S.pst;
  auto& pmp = S.pmp;
  auto& pdc = S.pdc;
  auto& pbar = S.pbar;
  const Grid& g = A.g;
  int* status = A.step + 1;
  const int tj = threadIdx.x;
  const int y0 = kGhost + by * TY;
  const int xb = kGhost + bx * XC;
  const int xe = min(xb + XC, g.nx - kGhost);
  const int j = y0 + tj;
  const bool active = j < g.ny - kGhost;
  if (tj == 0) {
    for (int s = 0; s < kRing2; ++s) mbar_init(&bar[s], 1);
    if constexpr (kStream) for (int s = 0; s < 2; ++s) mbar_init(&pbar[s], 1);
    fence_barrier_init();
  }
  __syncthreads();
  constexpr uint32_t kBytes = R::kWide * 4;
  constexpr uint32_t kPBytes = (kV2StateF + kV2MapF) * TY * 4 + TY * sizeof(uint16_t);
  static_assert(!kStream || (TY * sizeof(uint16_t)) % 128 == 0, "tap-index row slots: 128 B");
  auto issue_pw = [&](int slot, int x) {
    if constexpr (kStream) {
      mbar_arrive_expect_tx(&pbar[slot], kPBytes);
      tma_load_3d_row(pst[slot], &tm->vst, &pbar[slot], y0, x, kState2V0);
      tma_load_3d_row(pmp[slot], &tm->vmp, &pbar[slot], y0, x, kMapSlotVel);
      tma_load_2d(pdc[slot], &tm->dc, &pbar[slot], y0, x);
    }
  };
  if (tj == 0) {
    if constexpr (kPersist) fence_proxy_async_smem();
    for (int s = 0; s < 3; ++s) {
      mbar_arrive_expect_tx(&bar[s], kBytes);
      tma_load_2d(ring[s], tm_p, &bar[s], y0 - 8, xb - 1 + s);
    }
    issue_pw(0, xb);
  }
  const int64_t sx = g.sx;
  const float* __restrict__ p = A.f.p;
  float q[16];  // q[t] = p[x - 7 + t]
#pragma unroll
  for (int t = 0; t < 16; ++t)
    q[t] = active ? ld_col<kPersist>(p + (int64_t)(xb - 7 + t) * sx + j) : 0.f;
  const int si = tj + 8;
  for (int x = xb; x < xe; ++x) {
    const int it = x - xb;
    const int64_t c = (int64_t)x * sx + j;
    CV cv;
    if constexpr (!kStream) {
      if (active) cv.load(A, c);
    }
    const float qn = (active && x + 9 < g.nx) ? ld_col<kPersist>(p + (int64_t)(x + 9) * sx + j) : 0.f;
    __syncthreads();  // the halo slot of row x-2 and the point-wise slot of row x-1 are free
    if (tj == 0 && x + 1 < xe) {
      const int s = (it + 3) % kRing2;
      fence_proxy_async_smem();
      mbar_arrive_expect_tx(&bar[s], kBytes);
      tma_load_2d(ring[s], tm_p, &bar[s], y0 - 8, x + 2);
      issue_pw((it + 1) & 1, x + 1);
    }
    if (it == 0) {
      mbar_wait_bounded(&bar[0], 0, status);
      mbar_wait_bounded(&bar[1], 0, status);
    }
    mbar_wait_bounded(&bar[(it + 2) % kRing2], ((it + 2) / kRing2) & 1, status);
    if constexpr (kStream) {
      const int ps = it & 1;
      mbar_wait_bounded(&pbar[ps], (it >> 1) & 1, status);
      if (active) {
        static_assert(!kStream || CV::NA == 1, "streaming bodies: isotropic engine only");
        cv.dc = pdc[ps][tj];
        cv.rr = pmp[ps][0][tj];
        cv.iku[0] = pmp[ps][1][tj];
        cv.a1[0] = pmp[ps][2][tj];
        cv.b1[0] = pmp[ps][3][tj];
        cv.a2[0] = pmp[ps][4][tj];
        cv.b2[0] = pmp[ps][5][tj];
#pragma unroll
        for (int a = 0; a < 2; ++a) {
          cv.v[a] = pst[ps][a][tj];
          cv.s1[a] = pst[ps][2 + 2 * a][tj];
          cv.s2[a] = pst[ps][3 + 2 * a][tj];
        }
      }
    }
    const float* Rm = ring[it % kRing2];
    const float* R0 = ring[(it + 1) % kRing2];
    const float* R1 = ring[(it + 2) % kRing2];
    if (active) {
      float cm[8], co;
      load_taps(A.m.taps, cv.dc, cm, co);
      float gx = 0.f, gy = 0.f;
#pragma unroll
      for (int m = 1; m <= 8; ++m) {
        gx = fmaf(cm[m - 1], q[7 + m] - q[8 - m], gx);
        gy = fmaf(cm[m - 1], R0[si + m] - R0[si - (m - 1)], gy);
      }
      gx = fmaf(co, (R1[si + 1] - R0[si + 1]) + (R1[si - 1] - R0[si - 1]), gx);
      gy = fmaf(co, (R1[si + 1] - R1[si]) + (Rm[si + 1] - Rm[si]), gy);
      const float gg[2] = {gx * g.inv_h[0], gy * g.inv_h[1]};
      cv.update_store(A, c, gg);
    }
#pragma unroll
    for (int t = 0; t < 15; ++t) q[t] = q[t + 1];
    q[15] = qn;
  }
  if constexpr (kPersist) {
    __syncthreads();   // every wait on the ring is over
    if (tj == 0) {
      for (int s = 0; s < kRing2; ++s) mbar_inval(&bar[s]);
      if constexpr (kStream) for (int s = 0; s < 2; ++s) mbar_inval(&pbar[s]);
    }
  }
}

// `n`: the time step being completed (-1: read the simulation's device step counter).
template <int TY, int XC, class CP, bool kStream = false, bool kBeta = false,
          int kMapSlotPrs = 0, bool kPersist = false>
__device__ __forceinline__ void prs2d_march_body(PrsMarchSmem<TY, kStream, kBeta>& S,
                                                 const StepArgs& A, const March2Maps* tm,
                                                 int by, int bx, int n = -1) {
  static_assert(TY % kD2TY == 0 && XC % kD2TX == 0, "a march block must own whole list tiles");
  using R = Row2<TY>;
  constexpr int kMapF = PrsMarchSmem<TY, kStream, kBeta>::kMapF;
  const CUtensorMap* tm_vx = &tm->vx;
  const CUtensorMap* tm_vy = &tm->vy;
  auto& rx = S.rx;
  auto& ry = S.ry;
  auto& bar = S.bar;
  auto& ppp = S.ppp;
  auto& pph = S.pph;
  auto& pmp = S.pmp;
  auto& pdc = S.pdc;
  auto& pbar = S.pbar;
  const Grid& g = A.g;
  int* status = A.step + 1;
  const int tj = threadIdx.x;
  const int y0 = kGhost + by * TY;
  const int xb = kGhost + bx * XC;
  const int xe = min(xb + XC, g.nx - kGhost);
  const int j = y0 + tj;
  const bool active = j < g.ny - kGhost;
  if (tj == 0) {
    for (int s = 0; s < kRing2; ++s) mbar_init(&bar[s], 1);
    if constexpr (kStream) for (int s = 0; s < 2; ++s) mbar_init(&pbar[s], 1);
    fence_barrier_init();
  }
  __syncthreads();
  constexpr uint32_t kBytes = (R::kNarrow + R::kWide) * 4;
  constexpr uint32_t kPBytes = (1 + kP2PhiF + kMapF) * TY * 4 + TY * sizeof(uint16_t);
  static_assert(!kStream || (TY * sizeof(uint16_t)) % 128 == 0, "tap-index row slots: 128 B");
  auto issue = [&](int s, int x) {
    mbar_arrive_expect_tx(&bar[s], kBytes);
    tma_load_2d(rx[s], tm_vx, &bar[s], y0 - 4, x);
    tma_load_2d(ry[s], tm_vy, &bar[s], y0 - 8, x);
  };
  auto issue_pw = [&](int slot, int x) {
    if constexpr (kStream) {
      mbar_arrive_expect_tx(&pbar[slot], kPBytes);
      tma_load_3d_row(ppp[slot], &tm->pp, &pbar[slot], y0, x, 0);
      tma_load_3d_row(pph[slot], &tm->phi, &pbar[slot], y0, x, kState2Phi0);
      tma_load_3d_row(pmp[slot], kBeta ? &tm->pmp7 : &tm->pmp6, &pbar[slot], y0, x, kMapSlotPrs);
      tma_load_2d(pdc[slot], &tm->dc, &pbar[slot], y0, x);
    }
  };
  if (tj == 0) {
    if constexpr (kPersist) fence_proxy_async_smem();
    for (int s = 0; s < 3; ++s) issue(s, xb - 1 + s);
    issue_pw(0, xb);
  }
  const int64_t sx = g.sx;
  const float* __restrict__ vx = A.f.v[0];
  float* p = A.f.p;
  float r[16];  // r[t] = vx[x - 8 + t]
#pragma unroll
  for (int t = 0; t < 16; ++t)
    r[t] = active ? ld_col<kPersist>(vx + (int64_t)(xb - 8 + t) * sx + j) : 0.f;
  const int xi = tj + 4, yi = tj + 8;
  for (int x = xb; x < xe; ++x) {
    const int it = x - xb;
    const int64_t c = (int64_t)x * sx + j;
    CP cp;
    if constexpr (!kStream) {
      if (active) cp.load(A, c);
    }
    const float rn = active ? ld_col<kPersist>(vx + (int64_t)(x + 8) * sx + j) : 0.f;
    __syncthreads();
    if (tj == 0 && x + 1 < xe) {
      fence_proxy_async_smem();
      issue((it + 3) % kRing2, x + 2);
      issue_pw((it + 1) & 1, x + 1);
    }
    if (it == 0) {
      mbar_wait_bounded(&bar[0], 0, status);
      mbar_wait_bounded(&bar[1], 0, status);
    }
    mbar_wait_bounded(&bar[(it + 2) % kRing2], ((it + 2) / kRing2) & 1, status);
    if constexpr (kStream) {
      const int ps = it & 1;
      mbar_wait_bounded(&pbar[ps], (it >> 1) & 1, status);
      if (active) {
        static_assert(!kStream || CP::NA == 1, "streaming bodies: isotropic engine only");
        cp.dc = pdc[ps][tj];
        cp.dtk = pmp[ps][0][tj];
        cp.ikx[0] = pmp[ps][1][tj];
        cp.a1[0] = pmp[ps][2][tj];
        cp.b1[0] = pmp[ps][3][tj];
        cp.a2[0] = pmp[ps][4][tj];
        cp.b2[0] = pmp[ps][5][tj];
        cp.b2dt = kBeta ? pmp[ps][kMapF - 1][tj] : 0.f;
        cp.pc = ppp[ps][tj];
#pragma unroll
        for (int a = 0; a < 2; ++a) {
          cp.f1[a] = pph[ps][2 * a][tj];
          cp.f2[a] = pph[ps][2 * a + 1][tj];
        }
      }
    }
    const float* Xm = rx[it % kRing2];
    const float* X0 = rx[(it + 1) % kRing2];
    const float* Ym = ry[it % kRing2];
    const float* Y0 = ry[(it + 1) % kRing2];
    const float* Y1 = ry[(it + 2) % kRing2];
    if (active) {
      float cm[8], co;
      load_taps(A.m.taps, cp.dc, cm, co);
      float dx = 0.f, dy = 0.f;
#pragma unroll
      for (int m = 1; m <= 8; ++m) {
        dx = fmaf(cm[m - 1], r[7 + m] - r[8 - m], dx);
        dy = fmaf(cm[m - 1], Y0[yi + (m - 1)] - Y0[yi - m], dy);
      }
      dx = fmaf(co, (X0[xi + 1] - Xm[xi + 1]) + (X0[xi - 1] - Xm[xi - 1]), dx);
      dy = fmaf(co, (Y1[yi] - Y1[yi - 1]) + (Ym[yi] - Ym[yi - 1]), dy);
      const float dd[2] = {dx * g.inv_h[0], dy * g.inv_h[1]};
      cp.update_store(A, c, dd);
    }
#pragma unroll
    for (int t = 0; t < 15; ++t) r[t] = r[t + 1];
    r[15] = rn;
  }
  if constexpr (kPersist) {
    __syncthreads();   // every wait on the ring is over
    if (tj == 0) {
      for (int s = 0; s < kRing2; ++s) mbar_inval(&bar[s]);
      if constexpr (kStream) for (int s = 0; s < 2; ++s) mbar_inval(&pbar[s]);
    }
  }
  // the block's list tiles: rows [tx0, tx0 + XC / kD2TX) x columns [ty0, ty0 + TY / kD2TY)
  const int n_tx = (g.nx - 2 * kGhost + kD2TX - 1) / kD2TX;
  const int n_ty = (g.ny - 2 * kGhost + kD2TY - 1) / kD2TY;
  const int tx0 = bx * (XC / kD2TX), ty0 = by * (TY / kD2TY);
  span_epilogue(A, p, tx0, min(tx0 + XC / kD2TX, n_tx), ty0, min(ty0 + TY / kD2TY, n_ty), n_ty,
                tj, TY, n);
}

// Single simulation: grid (y blocks, x chunks); the tensor maps travel as one kernel parameter.
template <int TY, int XC, class CV, bool kStream = false, int kMapSlotVel = 0>
__global__ void __launch_bounds__(TY, 1024 / TY)
vel2d_march(const StepArgs A, const __grid_constant__ March2Maps tm) {
  __shared__ VelMarchSmem<TY, kStream> S;
  pdl_entry();
  if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) *A.step += 1;
  vel2d_march_body<TY, XC, CV, kStream, kMapSlotVel>(S, A, &tm, blockIdx.x, blockIdx.y);
}

template <int TY, int XC, class CP, bool kStream = false, bool kBeta = false, int kMapSlotPrs = 0>
__global__ void __launch_bounds__(TY, 1024 / TY)
prs2d_march(const StepArgs A, const __grid_constant__ March2Maps tm) {
  __shared__ PrsMarchSmem<TY, kStream, kBeta> S;
  pdl_entry();
  prs2d_march_body<TY, XC, CP, kStream, kBeta, kMapSlotPrs>(S, A, &tm, blockIdx.x, blockIdx.y);
}

// Group (batched) kernels: block b works on work[b] = {simulation, y block, x chunk, 1 if the
// block advances that simulation's step counter}. `sims` holds one argument block per simulation
// and `maps` one March2Maps per simulation, in global memory. The argument block is copied to
// shared memory first: stores to the fields then cannot alias it.
__device__ __forceinline__ void stage_args(StepArgs& dst, const StepArgs& src) {
  static_assert(sizeof(StepArgs) % 4 == 0, "word copy");
  const int* s = reinterpret_cast<const int*>(&src);
  int* d = reinterpret_cast<int*>(&dst);
  for (int w = threadIdx.x; w < (int)(sizeof(StepArgs) / 4); w += blockDim.x) d[w] = s[w];
  __syncthreads();
}

template <int TY, int XC, bool kStream = false, int kMapSlotVel = 0>
__global__ void __launch_bounds__(TY, 1024 / TY)
vel2d_march_group(const StepArgs* __restrict__ sims, const March2Maps* __restrict__ maps,
                  const int4* __restrict__ work) {
  __shared__ alignas(16) StepArgs A;
  __shared__ VelMarchSmem<TY, kStream> S;
  pdl_entry();
  const int4 t = work[blockIdx.x];
  stage_args(A, sims[t.x]);
  if (t.w && threadIdx.x == 0) *A.step += 1;
  vel2d_march_body<TY, XC, CellVelT<2, false>, kStream, kMapSlotVel>(S, A, maps + t.x, t.y, t.z);
}

template <int TY, int XC, bool kBeta, bool kStream = false, int kMapSlotPrs = 0>
__global__ void __launch_bounds__(TY, 1024 / TY)
prs2d_march_group(const StepArgs* __restrict__ sims, const March2Maps* __restrict__ maps,
                  const int4* __restrict__ work) {
  __shared__ alignas(16) StepArgs A;
  __shared__ PrsMarchSmem<TY, kStream, kBeta> S;
  pdl_entry();
  const int4 t = work[blockIdx.x];
  stage_args(A, sims[t.x]);
  prs2d_march_body<TY, XC, CellPrsT<2, kBeta, false>, kStream, kBeta, kMapSlotPrs>(
      S, A, maps + t.x, t.y, t.z);
}

// Persistent group kernel: the whole run of a group in one cooperative launch (all blocks
// co-resident). Members are ordered by nt (descending), so at step n the active members are a
// prefix and their work items the first tiles_upto[k] entries of the work list. Per step:
//   velocity bodies of the active items | grid barrier |
//   pressure bodies (+ epilogue) of the active items | grid barrier
// Blocks claim items from one 64-bit ticket counter (zeroed before the launch): in a phase with
// `items` items every block draws tickets until one falls past the phase's items, so each phase
// consumes exactly items + gridDim.x tickets and every block knows where the next phase starts.
// with the same bodies, and so the same results bit for bit, as the per-step group launches. A
// barrier that gives up (bounded wait) stops the launch and marks every member's status word.
// Between phases every thread fences its global writes against the async proxy, and the thread
// that issues a block's TMA loads fences again after the barrier: the loads read rows written by
// other blocks inside the same launch.
template <int TY, int XC, bool kBeta, int kMapSlotVel, int kMapSlotPrs>
__global__ void __launch_bounds__(TY, 1024 / TY)
step2d_group_persistent(const StepArgs* __restrict__ sims, const March2Maps* __restrict__ maps,
                        const int4* __restrict__ work, const int* __restrict__ member_nt,
                        const int* __restrict__ tiles_upto, int n_members, int max_nt,
                        unsigned* bar) {
  __shared__ alignas(16) StepArgs A;
  __shared__ union Rings {
    VelMarchSmem<TY, true> v;
    PrsMarchSmem<TY, true, kBeta> p;
  } S;
  __shared__ long long s_item;
  int* gstatus = reinterpret_cast<int*>(bar + kBarWords);
  unsigned long long* tickets = reinterpret_cast<unsigned long long*>(bar + kBarWords + 2);
  unsigned long long base = 0;   // first ticket of the current phase
  // next item of the phase, or -1 (every thread of the block gets the same answer)
  auto claim = [&](int items) -> int {
    __syncthreads();   // the previous item is done with A and s_item
    if (threadIdx.x == 0) {
      const unsigned long long t = atomicAdd(tickets, 1ull) - base;
      s_item = t < (unsigned long long)items ? (long long)t : -1;
    }
    __syncthreads();
    return (int)s_item;
  };
  auto phase_end = [&]() -> bool {
    fence_proxy_async_global();
    if (!grid_barrier(bar, gstatus, gridDim.x)) {
      if (blockIdx.x == 0)
        for (int r = threadIdx.x; r < n_members; r += blockDim.x) atomicOr(sims[r].step + 1, 4);
      return false;
    }
    if (threadIdx.x == 0) fence_proxy_async_global();
    return true;
  };
  for (int n = 0; n < max_nt; ++n) {
    int k = 0;
    while (k < n_members && member_nt[k] > n) ++k;
    const int items = tiles_upto[k];
    for (int w; (w = claim(items)) >= 0;) {
      const int4 t = work[w];
      stage_args(A, sims[t.x]);
      if (t.w && threadIdx.x == 0) *A.step += 1;
      vel2d_march_body<TY, XC, CellVelT<2, false>, true, kMapSlotVel, true>(S.v, A, maps + t.x,
                                                                            t.y, t.z);
    }
    base += (unsigned long long)items + gridDim.x;
    if (!phase_end()) return;
    for (int w; (w = claim(items)) >= 0;) {
      const int4 t = work[w];
      stage_args(A, sims[t.x]);
      prs2d_march_body<TY, XC, CellPrsT<2, kBeta, false>, true, kBeta, kMapSlotPrs, true>(
          S.p, A, maps + t.x, t.y, t.z, n);
    }
    base += (unsigned long long)items + gridDim.x;
    if (!phase_end()) return;
  }
}

}  // namespace fwgb
