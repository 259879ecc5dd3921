// 2D step kernels over one 32 (y) x 8 (x) tile per block with every operand staged in shared
// memory by TMA, for every cell physics (isotropic and anisotropic relaxation, exponential
// attenuation).
//
// The direct kernels load each operand with a thread load when it is needed, so a warp has only
// a few loads in flight and the kernels are latency-bound (long-scoreboard stalls) on grids that
// are too small for the row-march shapes to fill the GPU. Here one thread issues, at block start,
// TMA boxes for the stencil field with its halo, the point-wise state, the coefficient maps and
// the tap-index map, all completing on one mbarrier (bounded wait): the whole tile input (10-25 KB)
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
#include <type_traits>
#include "engine_common.cuh"
#include "kernels_direct.cuh"
#include "tma.cuh"

namespace fwgb {

// State boxes are 3D over the state (pitch, nx, field), or 4D over a state store (pitch, nx,
// field, slot) with one more unit box dimension. Map boxes are 3D over the coefficient-map stack.
struct Tile2Maps {
  CUtensorMap p_halo;    // state: box {48, 24, 1} (p: rows i0 - 8.., columns j0 - 8..)
  CUtensorMap vx_halo;   // state: box {40, 24, 1} (v_x: rows i0 - 8.., columns j0 - 4..)
  CUtensorMap vy_halo;   // state: box {48, 10, 1} (v_y: rows i0 - 1.., columns j0 - 8..)
  CUtensorMap st1, st2, st4, st6;          // state: boxes {32, 8, f}
  CUtensorMap mp1, mp3, mp5, mp6;          // coefficient maps: boxes {32, 8, f}
  CUtensorMap dc;                          // tap-index map: box {32, 8}
};

enum TilePhysics { kTileIso = 0, kTileAniso = 1, kTileExp = 2 };

// Map-stack slots the tile kernels read (the engine's map order): velocity maps 0-5 (rdt_rho and
// the x-gradient set inv_ku au1 bu1 au2 bu2), pressure maps 6-11 (dt_k and the x-divergence
// set), beta 2 dt at 12; anisotropic y sets at 13-17 (gradient) and 18-22 (divergence); the
// exponential engine's a_exp in slot 2.
constexpr int kTileMapVel = 0, kTileMapPrs = 6, kTileMapBeta = 12, kTileMapGradY = 13,
              kTileMapDivY = 18, kTileMapAexp = 2;

// Planes of each kernel's point-wise boxes, per physics.
template <int P> struct TileVelPlanes {
  static constexpr int kSt = P == kTileExp ? 2 : 6;                           // v (+ psi)
  static constexpr int kMp = P == kTileExp ? 3 : P == kTileAniso ? 11 : 6;    // maps
};
template <int P, bool kBeta> struct TilePrsPlanes {
  static constexpr int kPhi = P == kTileExp ? 0 : 4;
  static constexpr int kMp = (P == kTileExp ? 2 : P == kTileAniso ? 11 : 6) + (kBeta ? 1 : 0);
};

template <int P>
struct VelTileSmem {
  float p[24][48];
  float st[TileVelPlanes<P>::kSt][kD2TX][kD2TY];
  float mp[TileVelPlanes<P>::kMp][kD2TX][kD2TY];
  uint16_t dc[kD2TX][kD2TY];
  uint64_t bar;
  static constexpr uint32_t kTx =
      sizeof(float) * (24 * 48 + (TileVelPlanes<P>::kSt + TileVelPlanes<P>::kMp) * kD2TX * kD2TY) +
      sizeof(uint16_t) * kD2TX * kD2TY;
};
template <int P, bool kBeta>
struct PrsTileSmem {
  static constexpr int kPhi = TilePrsPlanes<P, kBeta>::kPhi;
  static constexpr int kMp = TilePrsPlanes<P, kBeta>::kMp;
  float vx[24][40];
  float vy[10][48];
  float p[kD2TX][kD2TY];
  float phi[kPhi > 0 ? kPhi : 1][kD2TX][kD2TY];
  float mp[kMp][kD2TX][kD2TY];
  uint16_t dc[kD2TX][kD2TY];
  uint64_t bar;
  static constexpr uint32_t kTx =
      sizeof(float) * (24 * 40 + 10 * 48 + (1 + kPhi + kMp) * kD2TX * kD2TY) +
      sizeof(uint16_t) * kD2TX * kD2TY;
};
// Every TMA destination starts on a 128-byte boundary: the halo boxes are 4608, 3840 and 1920
// bytes, every float plane 1024 bytes and the 16-bit tap-index plane 512 bytes.
static_assert(sizeof(float) * 24 * 48 % 128 == 0 && sizeof(float) * 24 * 40 % 128 == 0 &&
                  sizeof(float) * 10 * 48 % 128 == 0 && sizeof(float) * kD2TX * kD2TY % 128 == 0,
              "TMA destinations must be 128-byte aligned");

// One box of state fields: from the state (3D map) or from a slot of a state store (4D map).
template <bool kStore>
__device__ __forceinline__ void tma_state(void* dst, const CUtensorMap* map, uint64_t* bar, int x,
                                          int y, int field, int slot) {
  if constexpr (kStore) tma_load_4d(dst, map, bar, x, y, field, slot);
  else tma_load_3d(dst, map, bar, x, y, field);
}

// The loads of one tile (one thread issues them; completion on S.bar).
template <int P, bool kStore>
__device__ __forceinline__ void vel_tile_issue(VelTileSmem<P>& S, const Tile2Maps& M, int i0,
                                               int j0, int slot) {
  mbar_arrive_expect_tx(&S.bar, VelTileSmem<P>::kTx);
  tma_state<kStore>(S.p, &M.p_halo, &S.bar, j0 - 8, i0 - 8, 0, slot);
  if constexpr (P == kTileExp) {
    tma_state<kStore>(S.st, &M.st2, &S.bar, j0, i0, 1, slot);
    tma_load_3d(S.mp, &M.mp3, &S.bar, j0, i0, kTileMapVel);
  } else {
    tma_state<kStore>(S.st, &M.st6, &S.bar, j0, i0, 1, slot);
    tma_load_3d(S.mp, &M.mp6, &S.bar, j0, i0, kTileMapVel);
    if constexpr (P == kTileAniso) tma_load_3d(S.mp[6], &M.mp5, &S.bar, j0, i0, kTileMapGradY);
  }
  tma_load_2d(S.dc, &M.dc, &S.bar, j0, i0);
}

template <int P, bool kBeta, bool kStore>
__device__ __forceinline__ void prs_tile_issue(PrsTileSmem<P, kBeta>& S, const Tile2Maps& M,
                                               int i0, int j0, int slot) {
  using Smem = PrsTileSmem<P, kBeta>;
  mbar_arrive_expect_tx(&S.bar, Smem::kTx);
  tma_state<kStore>(S.vx, &M.vx_halo, &S.bar, j0 - 4, i0 - 8, 1, slot + 1);
  tma_state<kStore>(S.vy, &M.vy_halo, &S.bar, j0 - 8, i0 - 1, 2, slot + 1);
  tma_state<kStore>(S.p, &M.st1, &S.bar, j0, i0, 0, slot);
  if constexpr (P == kTileExp) {
    tma_load_3d(S.mp[0], &M.mp1, &S.bar, j0, i0, kTileMapPrs);
    tma_load_3d(S.mp[1], &M.mp1, &S.bar, j0, i0, kTileMapAexp);
  } else {
    tma_state<kStore>(S.phi, &M.st4, &S.bar, j0, i0, 7, slot);
    tma_load_3d(S.mp, &M.mp6, &S.bar, j0, i0, kTileMapPrs);
    if constexpr (P == kTileAniso) tma_load_3d(S.mp[6], &M.mp5, &S.bar, j0, i0, kTileMapDivY);
  }
  if constexpr (kBeta) tma_load_3d(S.mp[Smem::kMp - 1], &M.mp1, &S.bar, j0, i0, kTileMapBeta);
  tma_load_2d(S.dc, &M.dc, &S.bar, j0, i0);
}

// Tap set of the calling thread's cell (zeros outside the body), read from global memory before
// the block waits for its tile, so that its latency overlaps the TMA transfer.
__device__ __forceinline__ void tile_taps(const StepArgs& A, int i0, int j0, float (&cm)[8],
                                          float& co) {
  const Grid& g = A.g;
  const int i = i0 + threadIdx.y, j = j0 + threadIdx.x;
  if (i < g.nx - kGhost && j < g.ny - kGhost) {
    load_taps(A.m.taps, __ldg(A.m.dcmap + (int64_t)i * g.sx + j), cm, co);
  } else {
#pragma unroll
    for (int m = 0; m < 8; ++m) cm[m] = 0.f;
    co = 0.f;
  }
}

// Velocity update of the calling thread's cell of the staged tile at (i0, j0); cm / co: the
// cell's tap set (tile_taps).
template <int P>
__device__ __forceinline__ void vel_tile_compute(const StepArgs& A, const VelTileSmem<P>& S,
                                                 int i0, int j0, const float (&cm)[8],
                                                 float co) {
  const Grid& g = A.g;
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int i = i0 + ty, j = j0 + tx;
  if (i >= g.nx - kGhost || j >= g.ny - kGhost) return;
  const int64_t c = (int64_t)i * g.sx + j;
  auto Q = [&](int q) { return S.mp[q][ty][tx]; };
  using CV = typename std::conditional<P == kTileExp, CellVelExpT<2>,
                                       CellVelT<2, P == kTileAniso>>::type;
  CV cv;
  cv.dc = S.dc[ty][tx];
  cv.rr = Q(0);
  if constexpr (P == kTileExp) {
    cv.ae = Q(2);
#pragma unroll
    for (int a = 0; a < 2; ++a) cv.v[a] = S.st[a][ty][tx];
  } else {
#pragma unroll
    for (int q = 0; q < CV::NA; ++q) {   // x set in maps 1-5, y set (anisotropic) in 6-10
      cv.iku[q] = Q(1 + 5 * q);
      cv.a1[q] = Q(2 + 5 * q);
      cv.b1[q] = Q(3 + 5 * q);
      cv.a2[q] = Q(4 + 5 * q);
      cv.b2[q] = Q(5 + 5 * q);
    }
#pragma unroll
    for (int a = 0; a < 2; ++a) {
      cv.v[a] = S.st[a][ty][tx];
      cv.s1[a] = S.st[2 + 2 * a][ty][tx];
      cv.s2[a] = S.st[3 + 2 * a][ty][tx];
    }
  }
  auto Pp = [&](int di, int dj) { return S.p[ty + 8 + di][tx + 8 + dj]; };
  float gx = 0.f, gy = 0.f;
#pragma unroll
  for (int m = 1; m <= 8; ++m) {
    gx = fmaf(cm[m - 1], Pp(m, 0) - Pp(-(m - 1), 0), gx);
    gy = fmaf(cm[m - 1], Pp(0, m) - Pp(0, -(m - 1)), gy);
  }
  gx = fmaf(co, (Pp(1, 1) - Pp(0, 1)) + (Pp(1, -1) - Pp(0, -1)), gx);
  gy = fmaf(co, (Pp(1, 1) - Pp(1, 0)) + (Pp(-1, 1) - Pp(-1, 0)), gy);
  const float gg[2] = {gx * g.inv_h[0], gy * g.inv_h[1]};
  cv.update_store(A, c, gg);
}

// Pressure update of the calling thread's cell of the staged tile, then the tile's epilogue
// (every thread of the block calls it).
template <int P, bool kBeta>
__device__ __forceinline__ void prs_tile_compute(const StepArgs& A,
                                                 const PrsTileSmem<P, kBeta>& S, int i0, int j0,
                                                 int tile, const float (&cm)[8], float co) {
  using Smem = PrsTileSmem<P, kBeta>;
  constexpr int kBetaPlane = Smem::kMp - 1;   // beta 2 dt, when present, is the last map plane
  const Grid& g = A.g;
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * kD2TY + tx;
  const int i = i0 + ty, j = j0 + tx;
  if (i < g.nx - kGhost && j < g.ny - kGhost) {
    const int64_t c = (int64_t)i * g.sx + j;
    auto Q = [&](int q) { return S.mp[q][ty][tx]; };
    using CP = typename std::conditional<P == kTileExp, CellPrsExpT<2, kBeta>,
                                         CellPrsT<2, kBeta, P == kTileAniso>>::type;
    CP cp;
    cp.dc = S.dc[ty][tx];
    cp.dtk = Q(0);
    cp.b2dt = kBeta ? Q(kBetaPlane) : 0.f;
    cp.pc = S.p[ty][tx];
    if constexpr (P == kTileExp) {
      cp.ae = Q(1);
    } else {
#pragma unroll
      for (int q = 0; q < CP::NA; ++q) {   // x set in maps 1-5, y set (anisotropic) in 6-10
        cp.ikx[q] = Q(1 + 5 * q);
        cp.a1[q] = Q(2 + 5 * q);
        cp.b1[q] = Q(3 + 5 * q);
        cp.a2[q] = Q(4 + 5 * q);
        cp.b2[q] = Q(5 + 5 * q);
      }
#pragma unroll
      for (int a = 0; a < 2; ++a) {
        cp.f1[a] = S.phi[2 * a][ty][tx];
        cp.f2[a] = S.phi[2 * a + 1][ty][tx];
      }
    }
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
  tile_epilogue(A, A.f.p, tile, tid, kD2TY * kD2TX);
}

// ---- one tile per block ----------------------------------------------------------------------
template <int P, bool kStore = false>
__global__ void __launch_bounds__(256) vel2d_tile(const StepArgs A,
                                                  const __grid_constant__ Tile2Maps M, int slot) {
  pdl_entry();
  extern __shared__ __align__(128) unsigned char tile_smem[];
  VelTileSmem<P>& S = *reinterpret_cast<VelTileSmem<P>*>(tile_smem);
  int* status = A.step + 1;
  const int tid = threadIdx.y * kD2TY + threadIdx.x;
  const int i0 = kGhost + blockIdx.y * kD2TX, j0 = kGhost + blockIdx.x * kD2TY;
  if (smem_u32(tile_smem) & 127u) {   // TMA destinations need 128-byte alignment: refuse
    if (tid == 0) atomicOr(status, kStatusAlign);
    return;
  }
  if (tid == 0) {
    mbar_init(&S.bar, 1);
    fence_barrier_init();
    vel_tile_issue<P, kStore>(S, M, i0, j0, slot);
    if (blockIdx.x == 0 && blockIdx.y == 0) *A.step += 1;
  }
  float cm[8], co;
  tile_taps(A, i0, j0, cm, co);
  __syncthreads();   // barrier initialised before anyone polls it
  mbar_wait_bounded(&S.bar, 0, status);
  vel_tile_compute<P>(A, S, i0, j0, cm, co);
}

template <int P, bool kBeta, bool kStore = false>
__global__ void __launch_bounds__(256) prs2d_tile(const StepArgs A,
                                                  const __grid_constant__ Tile2Maps M, int slot) {
  pdl_entry();
  extern __shared__ __align__(128) unsigned char tile_smem[];
  PrsTileSmem<P, kBeta>& S = *reinterpret_cast<PrsTileSmem<P, kBeta>*>(tile_smem);
  int* status = A.step + 1;
  const int tid = threadIdx.y * kD2TY + threadIdx.x;
  const int i0 = kGhost + blockIdx.y * kD2TX, j0 = kGhost + blockIdx.x * kD2TY;
  if (smem_u32(tile_smem) & 127u) {
    if (tid == 0) atomicOr(status, kStatusAlign);
    return;
  }
  if (tid == 0) {
    mbar_init(&S.bar, 1);
    fence_barrier_init();
    prs_tile_issue<P, kBeta, kStore>(S, M, i0, j0, slot);
  }
  float cm[8], co;
  tile_taps(A, i0, j0, cm, co);
  __syncthreads();
  mbar_wait_bounded(&S.bar, 0, status);
  prs_tile_compute<P, kBeta>(A, S, i0, j0, blockIdx.y * gridDim.x + blockIdx.x, cm, co);
}

}  // namespace fwgb
