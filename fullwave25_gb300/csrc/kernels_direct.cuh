// Direct-addressed step kernels: one thread per body cell, stencil operands read through the
// read-only data path (L1/L2). Each time step is two launches:
//   velocity kernel: v += -dt/rho * (D1 p / kappau + psi1 + psi2), psi_nu <- b psi_nu + a D1 p
//   pressure kernel: p += -dt (K + 2 beta p) sum_axes (D2 v / kappax + phi1 + phi2), then the
//                    tile's source injection, air zeroing and sensor recording.
// Tiles: 2D block (32 y) x (8 x); 3D block (32 z) x (4 y) x (2 x). The host builds the
// per-tile source/air/sensor lists with the same tiling (see engine.cu: tile_of).
#pragma once
#include "engine_common.cuh"

namespace fwgb {

constexpr int kD2TY = 32, kD2TX = 8;             // 2D tile: 32 cells along y, 8 along x
constexpr int kD3TZ = 32, kD3TY = 4, kD3TX = 2;  // 3D tile

// ---------------------------------------------------------------------------------------- 2D
// Bodies take the tile (ty along y, tx along x) explicitly so that the single-simulation kernels
// (tile = block index) and the group kernels (tile from a work list) share them.
// Stencil operand load: through the read-only path (__ldg) when the field is constant for the
// whole launch, or a plain coherent load (ld.global.ca) in the persistent kernel, where the field
// is rewritten by other blocks between grid barriers inside the same launch.
template <bool kCoherent>
__device__ __forceinline__ float ld_field(const float* q) {
  if constexpr (kCoherent) return __ldca(q);
  else return __ldg(q);
}

template <class CV, bool kCoherent = false>
__device__ __forceinline__ void vel2d_body(const StepArgs& A, int tile_y, int tile_x) {
  const Grid& g = A.g;
  const int j = kGhost + tile_y * kD2TY + threadIdx.x;
  const int i = kGhost + tile_x * kD2TX + threadIdx.y;
  if (i >= g.nx - kGhost || j >= g.ny - kGhost) return;
  const int64_t sx = g.sx;
  const int64_t c = i * sx + j;
  const float* p = A.f.p;
  auto P = [&](int64_t o) { return ld_field<kCoherent>(p + c + o); };
  CV cv;
  cv.load(A, c);
  float cm[8], co;
  load_taps(A.m.taps, cv.dc, cm, co);
  float gx = 0.f, gy = 0.f;
#pragma unroll
  for (int m = 1; m <= 8; ++m) {
    gx = fmaf(cm[m - 1], P(m * sx) - P(-(m - 1) * sx), gx);
    gy = fmaf(cm[m - 1], P(m) - P(-(m - 1)), gy);
  }
  gx = fmaf(co, (P(sx + 1) - P(1)) + (P(sx - 1) - P(-1)), gx);
  gy = fmaf(co, (P(1 + sx) - P(sx)) + (P(1 - sx) - P(-sx)), gy);
  const float gg[2] = {gx * g.inv_h[0], gy * g.inv_h[1]};
  cv.update_store(A, c, gg);
}

// `n`: the time step being completed (-1: read the device step counter in the epilogue).
template <class CP, bool kCoherent = false>
__device__ __forceinline__ void prs2d_body(const StepArgs& A, int tile_y, int tile_x, int tile,
                                           int n = -1) {
  const Grid& g = A.g;
  const int j = kGhost + tile_y * kD2TY + threadIdx.x;
  const int i = kGhost + tile_x * kD2TX + threadIdx.y;
  float* p = A.f.p;
  if (i < g.nx - kGhost && j < g.ny - kGhost) {
    const int64_t sx = g.sx;
    const int64_t c = i * sx + j;
    const float* vx = A.f.v[0];
    const float* vy = A.f.v[1];
    auto X = [&](int64_t o) { return ld_field<kCoherent>(vx + c + o); };
    auto Y = [&](int64_t o) { return ld_field<kCoherent>(vy + c + o); };
    CP cp;
    cp.load(A, c);
    float cm[8], co;
    load_taps(A.m.taps, cp.dc, cm, co);
    float dx = 0.f, dy = 0.f;
#pragma unroll
    for (int m = 1; m <= 8; ++m) {
      dx = fmaf(cm[m - 1], X((m - 1) * sx) - X(-m * sx), dx);
      dy = fmaf(cm[m - 1], Y(m - 1) - Y(-m), dy);
    }
    dx = fmaf(co, (X(1) - X(-sx + 1)) + (X(-1) - X(-sx - 1)), dx);
    dy = fmaf(co, (Y(sx) - Y(sx - 1)) + (Y(-sx) - Y(-sx - 1)), dy);
    const float dd[2] = {dx * g.inv_h[0], dy * g.inv_h[1]};
    cp.update_store(A, c, dd);
  }
  tile_epilogue(A, p, tile, threadIdx.y * blockDim.x + threadIdx.x, blockDim.x * blockDim.y, n);
}

template <class CV>
__global__ void __launch_bounds__(256) vel2d_direct(const StepArgs A) {
  pdl_entry();
  if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0 && threadIdx.y == 0) *A.step += 1;
  vel2d_body<CV>(A, blockIdx.x, blockIdx.y);
}

template <class CP>
__global__ void __launch_bounds__(256) prs2d_direct(const StepArgs A) {
  pdl_entry();
  prs2d_body<CP>(A, blockIdx.x, blockIdx.y, blockIdx.y * gridDim.x + blockIdx.x);
}

// Group (batched) kernels: block b works on tiles[b] = {simulation, tile_y, tile_x, tile index
// within that simulation}; `sims` holds one argument block per simulation, each with its own step
// counter, advanced by the block that owns the simulation's tile 0. One launch per phase advances
// every listed simulation by one step; simulations may be at different steps.
static __global__ void __launch_bounds__(256) vel2d_group(const StepArgs* __restrict__ sims,
                                                   const int4* __restrict__ tiles) {
  pdl_entry();
  const int4 t = tiles[blockIdx.x];
  const StepArgs& A = sims[t.x];
  if (t.w == 0 && threadIdx.x == 0 && threadIdx.y == 0) *A.step += 1;
  vel2d_body<CellVelT<2, false>>(A, t.y, t.z);
}

template <bool kBeta>
__global__ void __launch_bounds__(256) prs2d_group(const StepArgs* __restrict__ sims,
                                                   const int4* __restrict__ tiles) {
  pdl_entry();
  const int4 t = tiles[blockIdx.x];
  prs2d_body<CellPrsT<2, kBeta, false>>(sims[t.x], t.y, t.z, t.w);
}

// ---------------------------------------------------------------------------------------- 3D
template <class CV>
__global__ void __launch_bounds__(256) vel3d_direct(const StepArgs A) {
  pdl_entry();
  const Grid& g = A.g;
  const int k = kGhost + blockIdx.x * kD3TZ + threadIdx.x;
  const int j = kGhost + blockIdx.y * kD3TY + threadIdx.y;
  const int i = kGhost + blockIdx.z * kD3TX + threadIdx.z;
  if (blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0 && threadIdx.x == 0 &&
      threadIdx.y == 0 && threadIdx.z == 0)
    *A.step += 1;
  if (i >= g.nx - kGhost || j >= g.ny - kGhost || k >= g.nz - kGhost) return;
  const int64_t sx = g.sx, sy = g.sy;
  const int64_t c = i * sx + j * sy + k;
  const float* __restrict__ p = A.f.p;
  CV cv;
  cv.load(A, c);
  float cm[8], co;
  load_taps(A.m.taps, cv.dc, cm, co);
  float gx = 0.f, gy = 0.f, gz = 0.f;
#pragma unroll
  for (int m = 1; m <= 8; ++m) {
    gx = fmaf(cm[m - 1], __ldg(p + c + m * sx) - __ldg(p + c - (m - 1) * sx), gx);
    gy = fmaf(cm[m - 1], __ldg(p + c + m * sy) - __ldg(p + c - (m - 1) * sy), gy);
    gz = fmaf(cm[m - 1], __ldg(p + c + m) - __ldg(p + c - (m - 1)), gz);
  }
  auto P = [&](int64_t o) { return __ldg(p + c + o); };
  gx = fmaf(co, ((P(sx + sy) - P(sy)) + (P(sx - sy) - P(-sy))) + ((P(sx + 1) - P(1)) + (P(sx - 1) - P(-1))), gx);
  gy = fmaf(co, ((P(sy + sx) - P(sx)) + (P(sy - sx) - P(-sx))) + ((P(sy + 1) - P(1)) + (P(sy - 1) - P(-1))), gy);
  gz = fmaf(co, ((P(1 + sx) - P(sx)) + (P(1 - sx) - P(-sx))) + ((P(1 + sy) - P(sy)) + (P(1 - sy) - P(-sy))), gz);
  const float gg[3] = {gx * g.inv_h[0], gy * g.inv_h[1], gz * g.inv_h[2]};
  cv.update_store(A, c, gg);
}

template <class CP>
__global__ void __launch_bounds__(256) prs3d_direct(const StepArgs A) {
  pdl_entry();
  const Grid& g = A.g;
  const int k = kGhost + blockIdx.x * kD3TZ + threadIdx.x;
  const int j = kGhost + blockIdx.y * kD3TY + threadIdx.y;
  const int i = kGhost + blockIdx.z * kD3TX + threadIdx.z;
  float* p = A.f.p;
  if (i < g.nx - kGhost && j < g.ny - kGhost && k < g.nz - kGhost) {
    const int64_t sx = g.sx, sy = g.sy;
    const int64_t c = i * sx + j * sy + k;
    const float* __restrict__ vx = A.f.v[0];
    const float* __restrict__ vy = A.f.v[1];
    const float* __restrict__ vz = A.f.v[2];
    CP cp;
    cp.load(A, c);
    float cm[8], co;
    load_taps(A.m.taps, cp.dc, cm, co);
    float dx = 0.f, dy = 0.f, dz = 0.f;
#pragma unroll
    for (int m = 1; m <= 8; ++m) {
      dx = fmaf(cm[m - 1], __ldg(vx + c + (m - 1) * sx) - __ldg(vx + c - m * sx), dx);
      dy = fmaf(cm[m - 1], __ldg(vy + c + (m - 1) * sy) - __ldg(vy + c - m * sy), dy);
      dz = fmaf(cm[m - 1], __ldg(vz + c + (m - 1)) - __ldg(vz + c - m), dz);
    }
    auto X = [&](int64_t o) { return __ldg(vx + c + o); };
    auto Y = [&](int64_t o) { return __ldg(vy + c + o); };
    auto Z = [&](int64_t o) { return __ldg(vz + c + o); };
    dx = fmaf(co, ((X(sy) - X(sy - sx)) + (X(-sy) - X(-sy - sx))) + ((X(1) - X(1 - sx)) + (X(-1) - X(-1 - sx))), dx);
    dy = fmaf(co, ((Y(sx) - Y(sx - sy)) + (Y(-sx) - Y(-sx - sy))) + ((Y(1) - Y(1 - sy)) + (Y(-1) - Y(-1 - sy))), dy);
    dz = fmaf(co, ((Z(sx) - Z(sx - 1)) + (Z(-sx) - Z(-sx - 1))) + ((Z(sy) - Z(sy - 1)) + (Z(-sy) - Z(-sy - 1))), dz);
    const float dd[3] = {dx * g.inv_h[0], dy * g.inv_h[1], dz * g.inv_h[2]};
    cp.update_store(A, c, dd);
  }
  tile_epilogue(A, p, (blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x,
                (threadIdx.z * blockDim.y + threadIdx.y) * blockDim.x + threadIdx.x,
                blockDim.x * blockDim.y * blockDim.z);
}

}  // namespace fwgb
