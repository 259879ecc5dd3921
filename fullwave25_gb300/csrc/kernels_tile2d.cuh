// 2D step kernels over one 32 (y) x 8 (x) tile per block with every operand staged in shared
// memory by TMA (isotropic relaxation engine).
//
// The direct kernels load each operand with a thread load when it is needed, so a warp has only
// a few loads in flight and the kernels are latency-bound (long-scoreboard stalls) on grids that
// are too small for the row-march shapes to fill the GPU. Here one thread issues, at block start,
// TMA boxes for the stencil field with its halo, the point-wise state, the coefficient maps and
// the tap-index map, all completing on one mbarrier (bounded wait): the whole tile input (18-20 KB)
// is in flight at once, with up to eight such blocks per SM. The arithmetic is that of
// vel2d_body / prs2d_body (same cell classes, same operation order), so the results are bitwise
// equal to the direct kernels'; the pressure kernel ends with the same tile epilogue.
//
// kStore: the step runs out of place over a store of states (the discrete adjoint's
// recomputation): the boxes are read from store slot `slot` (state n; the pressure kernel's
// velocity halos from slot + 1) through 4D tensor maps (pitch, nx, field, slot), and the results
// are written through the field pointers of A, which point at slot + 1. Every body cell of every
// field of slot + 1 is written; its ghost layer is not (the caller keeps it zero).
#pragma once
#include "engine_common.cuh"
#include "kernels_direct.cuh"
#include "tma.cuh"

namespace fwgb {

// State boxes are 3D over the state (pitch, nx, field), or 4D over a state store (pitch, nx,
// field, slot) with one more unit box dimension.
struct Tile2Maps {
  CUtensorMap p_halo;    // state stack: box {48, 24, 1} (p: rows i0 - 8.., columns j0 - 8..)
  CUtensorMap vx_halo;   // state stack: box {40, 24, 1} (v_x: rows i0 - 8.., columns j0 - 4..)
  CUtensorMap vy_halo;   // state stack: box {48, 10, 1} (v_y: rows i0 - 1.., columns j0 - 8..)
  CUtensorMap st1, st4, st6;   // state stack: boxes {32, 8, f}
  CUtensorMap maps6, maps7;    // coefficient-map stack: boxes {32, 8, 6} and {32, 8, 7}
  CUtensorMap dc;              // tap-index map: box {32, 8}
};

struct VelTileSmem {
  float p[24][48];
  float st[6][kD2TX][kD2TY];   // v_x v_y psi_x1 psi_x2 psi_y1 psi_y2
  float mp[6][kD2TX][kD2TY];   // rdt_rho inv_ku au1 bu1 au2 bu2
  int dc[kD2TX][kD2TY];
  uint64_t bar;
};
struct PrsTileSmem {
  float vx[24][40];
  float vy[10][48];
  float p[kD2TX][kD2TY];
  float phi[4][kD2TX][kD2TY];  // phi_x1 phi_x2 phi_y1 phi_y2
  float mp[7][kD2TX][kD2TY];   // dt_k inv_kx ax1 bx1 ax2 bx2 [beta2dt]
  int dc[kD2TX][kD2TY];
  uint64_t bar;
};
static_assert(offsetof(VelTileSmem, st) % 128 == 0 && offsetof(VelTileSmem, mp) % 128 == 0 &&
                  offsetof(VelTileSmem, dc) % 128 == 0,
              "TMA destinations must be 128-byte aligned");
static_assert(offsetof(PrsTileSmem, vy) % 128 == 0 && offsetof(PrsTileSmem, p) % 128 == 0 &&
                  offsetof(PrsTileSmem, phi) % 128 == 0 && offsetof(PrsTileSmem, mp) % 128 == 0 &&
                  offsetof(PrsTileSmem, dc) % 128 == 0,
              "TMA destinations must be 128-byte aligned");
constexpr uint32_t kVelTileTx = sizeof(float) * (24 * 48 + 12 * kD2TX * kD2TY) + 4 * kD2TX * kD2TY;
__host__ __device__ constexpr uint32_t prs_tile_tx(bool beta) {
  return sizeof(float) * (24 * 40 + 10 * 48 + (beta ? 12 : 11) * kD2TX * kD2TY) +
         4 * kD2TX * kD2TY;
}

// One box of state fields: from the state (3D map) or from a slot of a state store (4D map).
template <bool kStore>
__device__ __forceinline__ void tma_state(void* dst, const CUtensorMap* map, uint64_t* bar, int x,
                                          int y, int field, int slot) {
  if constexpr (kStore) tma_load_4d(dst, map, bar, x, y, field, slot);
  else tma_load_3d(dst, map, bar, x, y, field);
}

// Block prologue of the tile kernels: alignment guard and barrier init (one thread).
template <class SmemT>
__device__ __forceinline__ bool tile_begin(SmemT& S, const unsigned char* base, int* status,
                                           int tid, uint32_t tx_bytes) {
  if (smem_u32(base) & 127u) {
    if (tid == 0) atomicOr(status, kStatusAlign);
    return false;
  }
  if (tid == 0) {
    mbar_init(&S.bar, 1);
    fence_barrier_init();
    mbar_arrive_expect_tx(&S.bar, tx_bytes);
  }
  return true;
}

template <int kMapVel, bool kStore = false>
__global__ void __launch_bounds__(256) vel2d_tile(const StepArgs A,
                                                  const __grid_constant__ Tile2Maps M, int slot) {
  pdl_entry();
  extern __shared__ __align__(128) unsigned char tile_smem[];
  VelTileSmem& S = *reinterpret_cast<VelTileSmem*>(tile_smem);
  const Grid& g = A.g;
  int* status = A.step + 1;
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * kD2TY + tx;
  const int i0 = kGhost + blockIdx.y * kD2TX, j0 = kGhost + blockIdx.x * kD2TY;
  if (!tile_begin(S, tile_smem, status, tid, kVelTileTx)) return;
  if (blockIdx.x == 0 && blockIdx.y == 0 && tid == 0) *A.step += 1;
  if (tid == 0) {
    tma_state<kStore>(S.p, &M.p_halo, &S.bar, j0 - 8, i0 - 8, 0, slot);
    tma_state<kStore>(S.st, &M.st6, &S.bar, j0, i0, 1, slot);
    tma_load_3d(S.mp, &M.maps6, &S.bar, j0, i0, kMapVel);
    tma_load_2d(S.dc, &M.dc, &S.bar, j0, i0);
  }
  __syncthreads();   // barrier initialised before anyone polls it
  mbar_wait_bounded(&S.bar, 0, status);
  const int i = i0 + ty, j = j0 + tx;
  if (i >= g.nx - kGhost || j >= g.ny - kGhost) return;
  const int64_t c = (int64_t)i * g.sx + j;
  CellVelT<2, false> cv;
  cv.dc = S.dc[ty][tx];
  cv.rr = S.mp[0][ty][tx];
  cv.iku[0] = S.mp[1][ty][tx];
  cv.a1[0] = S.mp[2][ty][tx];
  cv.b1[0] = S.mp[3][ty][tx];
  cv.a2[0] = S.mp[4][ty][tx];
  cv.b2[0] = S.mp[5][ty][tx];
#pragma unroll
  for (int a = 0; a < 2; ++a) {
    cv.v[a] = S.st[a][ty][tx];
    cv.s1[a] = S.st[2 + 2 * a][ty][tx];
    cv.s2[a] = S.st[3 + 2 * a][ty][tx];
  }
  float cm[8], co;
  load_taps(A.m.taps, cv.dc, cm, co);
  auto P = [&](int di, int dj) { return S.p[ty + 8 + di][tx + 8 + dj]; };
  float gx = 0.f, gy = 0.f;
#pragma unroll
  for (int m = 1; m <= 8; ++m) {
    gx = fmaf(cm[m - 1], P(m, 0) - P(-(m - 1), 0), gx);
    gy = fmaf(cm[m - 1], P(0, m) - P(0, -(m - 1)), gy);
  }
  gx = fmaf(co, (P(1, 1) - P(0, 1)) + (P(1, -1) - P(0, -1)), gx);
  gy = fmaf(co, (P(1, 1) - P(1, 0)) + (P(-1, 1) - P(-1, 0)), gy);
  const float gg[2] = {gx * g.inv_h[0], gy * g.inv_h[1]};
  cv.update_store(A, c, gg);
}

template <bool kBeta, int kMapPrs, bool kStore = false>
__global__ void __launch_bounds__(256) prs2d_tile(const StepArgs A,
                                                  const __grid_constant__ Tile2Maps M, int slot) {
  pdl_entry();
  extern __shared__ __align__(128) unsigned char tile_smem[];
  PrsTileSmem& S = *reinterpret_cast<PrsTileSmem*>(tile_smem);
  const Grid& g = A.g;
  int* status = A.step + 1;
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * kD2TY + tx;
  const int i0 = kGhost + blockIdx.y * kD2TX, j0 = kGhost + blockIdx.x * kD2TY;
  if (!tile_begin(S, tile_smem, status, tid, prs_tile_tx(kBeta))) return;
  if (tid == 0) {
    tma_state<kStore>(S.vx, &M.vx_halo, &S.bar, j0 - 4, i0 - 8, 1, slot + 1);
    tma_state<kStore>(S.vy, &M.vy_halo, &S.bar, j0 - 8, i0 - 1, 2, slot + 1);
    tma_state<kStore>(S.p, &M.st1, &S.bar, j0, i0, 0, slot);
    tma_state<kStore>(S.phi, &M.st4, &S.bar, j0, i0, 7, slot);
    tma_load_3d(S.mp, kBeta ? &M.maps7 : &M.maps6, &S.bar, j0, i0, kMapPrs);
    tma_load_2d(S.dc, &M.dc, &S.bar, j0, i0);
  }
  __syncthreads();
  mbar_wait_bounded(&S.bar, 0, status);
  const int i = i0 + ty, j = j0 + tx;
  if (i < g.nx - kGhost && j < g.ny - kGhost) {
    const int64_t c = (int64_t)i * g.sx + j;
    CellPrsT<2, kBeta, false> cp;
    cp.dc = S.dc[ty][tx];
    cp.dtk = S.mp[0][ty][tx];
    cp.b2dt = kBeta ? S.mp[6][ty][tx] : 0.f;
    cp.ikx[0] = S.mp[1][ty][tx];
    cp.a1[0] = S.mp[2][ty][tx];
    cp.b1[0] = S.mp[3][ty][tx];
    cp.a2[0] = S.mp[4][ty][tx];
    cp.b2[0] = S.mp[5][ty][tx];
    cp.pc = S.p[ty][tx];
#pragma unroll
    for (int a = 0; a < 2; ++a) {
      cp.f1[a] = S.phi[2 * a][ty][tx];
      cp.f2[a] = S.phi[2 * a + 1][ty][tx];
    }
    float cm[8], co;
    load_taps(A.m.taps, cp.dc, cm, co);
    auto X = [&](int di, int dj) { return S.vx[ty + 8 + di][tx + 4 + dj]; };
    auto Y = [&](int di, int dj) { return S.vy[ty + 1 + di][tx + 8 + dj]; };
    float dx = 0.f, dy = 0.f;
#pragma unroll
    for (int m = 1; m <= 8; ++m) {
      dx = fmaf(cm[m - 1], X(m - 1, 0) - X(-m, 0), dx);
      dy = fmaf(cm[m - 1], Y(0, m - 1) - Y(0, -m), dy);
    }
    dx = fmaf(co, (X(0, 1) - X(-1, 1)) + (X(0, -1) - X(-1, -1)), dx);
    dy = fmaf(co, (Y(1, 0) - Y(1, -1)) + (Y(-1, 0) - Y(-1, -1)), dy);
    const float dd[2] = {dx * g.inv_h[0], dy * g.inv_h[1]};
    cp.update_store(A, c, dd);
  }
  tile_epilogue(A, A.f.p, blockIdx.y * gridDim.x + blockIdx.x, tid, kD2TY * kD2TX);
}

}  // namespace fwgb
