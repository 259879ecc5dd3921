// 3D step kernels that march along the slowest axis (x, depth).
//
// Block = 32 (z, one warp) x 8 (y) threads; each thread owns one (y, z) column and walks
// XC consecutive x planes. Per plane:
//   * the x-derivative taps come from a 16-entry register queue of that column (one new
//     coalesced load per plane, prefetched one plane ahead);
//   * the y/z taps and all off-axis taps come from shared-memory copies of planes x-1, x, x+1
//     (with the y/z halos they need), brought in by TMA into a 4-slot ring: while plane x is
//     computed, plane x+2 is in flight. Each slot has one mbarrier; waits are bounded.
//   * the point-wise state and maps of the cell are read and written once, coalesced.
// The arithmetic (operation order and fused multiply-adds) is the same as the direct kernels.
#pragma once
#include "engine_common.cuh"
#include "tma.cuh"

namespace fwgb {

constexpr int kMTZ = 32, kMTY = 8, kMThreads = kMTZ * kMTY, kRing = 4;
// velocity kernel: p planes with y and z halos of 8
constexpr int kPW = kMTZ + 16, kPH = kMTY + 16;
constexpr int kPSlot = kPW * kPH;                     // 1152 floats = 4608 B
// pressure kernel: vx (halo 1 in y, z window [-4, 36)), vy (halo 8 in y), vz (halo 8 in z)
constexpr int kXW = kMTZ + 8, kXH = kMTY + 2;         // 40 x 10
constexpr int kYW = kMTZ + 8, kYH = kMTY + 16;        // 40 x 24
constexpr int kZW = kMTZ + 16, kZH = kMTY + 2;        // 48 x 10
constexpr int kXSlot = 416, kYSlot = kYW * kYH, kZSlot = kZW * kZH;  // vx slot padded to 128 B
static_assert(kXSlot >= kXW * kXH && (kXSlot * 4) % 128 == 0, "vx slot");
static_assert((kYSlot * 4) % 128 == 0 && (kZSlot * 4) % 128 == 0 && (kPSlot * 4) % 128 == 0, "slots");

// The plane loops below run in unrolled groups of 16 planes starting at multiples of 16 from the
// block's first plane, so a plane's ring slot and mbarrier phase follow from its position u in the
// group alone: (it + k) % kRing == (u + k) % kRing and ((it + 2) / kRing) & 1 == ((u + 2) / kRing) & 1.
static_assert(16 % kRing == 0 && (16 / kRing) % 2 == 0, "ring slots and phases repeat every 16 planes");

struct MarchMaps {
  CUtensorMap p, vx, vy, vz;
};

template <int XC, class CV, int kMinBlocks = 3>
__global__ void __launch_bounds__(kMThreads, kMinBlocks)
vel3d_march(const StepArgs A, const __grid_constant__ CUtensorMap tm_p) {
  pdl_entry();
  __shared__ alignas(128) float ring[kRing][kPSlot];
  __shared__ alignas(8) uint64_t bar[kRing];
  const Grid& g = A.g;
  int* status = A.step + 1;
  const int tz = threadIdx.x, ty = threadIdx.y, tid = ty * kMTZ + tz;
  const int z0 = kGhost + blockIdx.x * kMTZ, y0 = kGhost + blockIdx.y * kMTY;
  const int xb = kGhost + blockIdx.z * XC;
  const int xe = min(xb + XC, g.nx - kGhost);
  const int k = z0 + tz, j = y0 + ty;
  const bool active = k < g.nz - kGhost && j < g.ny - kGhost;
  if (blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0 && tid == 0) *A.step += 1;
  if (tid == 0) {
    for (int s = 0; s < kRing; ++s) mbar_init(&bar[s], 1);
    fence_barrier_init();
  }
  __syncthreads();
  constexpr uint32_t kBytes = kPSlot * 4;
  if (tid == 0) {
    for (int s = 0; s < 3; ++s) {  // planes xb-1, xb, xb+1
      mbar_arrive_expect_tx(&bar[s], kBytes);
      tma_load_3d(ring[s], &tm_p, &bar[s], z0 - 8, y0 - 8, xb - 1 + s);
    }
  }
  const int64_t sx = g.sx;
  const int64_t col = (int64_t)j * g.sy + k;
  const float* __restrict__ p = A.f.p;
  // x-direction register queue, rotated instead of shifted: at plane x = xb + 16 m + u the
  // sample p[x - 7 + t] is q[(u + t) & 15]; the plane loop is unrolled by 16 so that every index
  // is a compile-time register
  float q[16];
#pragma unroll
  for (int t = 0; t < 16; ++t) q[t] = active ? __ldg(p + (int64_t)(xb - 7 + t) * sx + col) : 0.f;
  const int si = (ty + 8) * kPW + (tz + 8);
  for (int x0 = xb; x0 < xe; x0 += 16) {
#pragma unroll
  for (int u = 0; u < 16; ++u) {
    const int x = x0 + u;
    if (x >= xe) break;  // uniform over the block
    const int64_t c = (int64_t)x * sx + col;
    // point-wise operands of this plane: issued before the block barrier and the TMA wait so
    // their HBM latency overlaps them
    CV cv;
    if (active) cv.load(A, c);
    const float qn = (active && x + 9 < g.nx) ? __ldg(p + (int64_t)(x + 9) * sx + col) : 0.f;
    __syncthreads();  // the slot of plane x-2 is no longer read
    if (tid == 0 && x + 1 < xe) {
      const int s = (u + 3) % kRing;
      fence_proxy_async_smem();
      mbar_arrive_expect_tx(&bar[s], kBytes);
      tma_load_3d(ring[s], &tm_p, &bar[s], z0 - 8, y0 - 8, x + 2);
    }
    if (u == 0 && x0 == xb) {
      mbar_wait_bounded(&bar[0], 0, status);
      mbar_wait_bounded(&bar[1], 0, status);
    }
    mbar_wait_bounded(&bar[(u + 2) % kRing], ((u + 2) / kRing) & 1, status);
    const float* Pm = ring[u % kRing];
    const float* P0 = ring[(u + 1) % kRing];
    const float* P1 = ring[(u + 2) % kRing];
    if (active) {
      float cm[8], co;
      load_taps(A.m.taps, cv.dc, cm, co);
      float gx = 0.f, gy = 0.f, gz = 0.f;
#pragma unroll
      for (int m = 1; m <= 8; ++m) {
        gx = fmaf(cm[m - 1], q[(u + 7 + m) & 15] - q[(u + 8 - m) & 15], gx);
        gy = fmaf(cm[m - 1], P0[si + m * kPW] - P0[si - (m - 1) * kPW], gy);
        gz = fmaf(cm[m - 1], P0[si + m] - P0[si - (m - 1)], gz);
      }
      gx = fmaf(co, ((P1[si + kPW] - P0[si + kPW]) + (P1[si - kPW] - P0[si - kPW])) +
                        ((P1[si + 1] - P0[si + 1]) + (P1[si - 1] - P0[si - 1])), gx);
      gy = fmaf(co, ((P1[si + kPW] - P1[si]) + (Pm[si + kPW] - Pm[si])) +
                        ((P0[si + kPW + 1] - P0[si + 1]) + (P0[si + kPW - 1] - P0[si - 1])), gy);
      gz = fmaf(co, ((P1[si + 1] - P1[si]) + (Pm[si + 1] - Pm[si])) +
                        ((P0[si + kPW + 1] - P0[si + kPW]) + (P0[si - kPW + 1] - P0[si - kPW])), gz);
      const float gg[3] = {gx * g.inv_h[0], gy * g.inv_h[1], gz * g.inv_h[2]};
      cv.update_store(A, c, gg);
    }
    q[u] = qn;  // p[x + 9]: the sample at t = 15 of plane x + 1
  }
  }
}

template <int XC, class CP, int kMinBlocks = 3>
__global__ void __launch_bounds__(kMThreads, kMinBlocks)
prs3d_march(const StepArgs A, const __grid_constant__ CUtensorMap tm_vx,
            const __grid_constant__ CUtensorMap tm_vy, const __grid_constant__ CUtensorMap tm_vz) {
  pdl_entry();
  __shared__ alignas(128) float rx[kRing][kXSlot];
  __shared__ alignas(128) float ry[kRing][kYSlot];
  __shared__ alignas(128) float rz[kRing][kZSlot];
  __shared__ alignas(8) uint64_t bar[kRing];
  const Grid& g = A.g;
  int* status = A.step + 1;
  const int tz = threadIdx.x, ty = threadIdx.y, tid = ty * kMTZ + tz;
  const int z0 = kGhost + blockIdx.x * kMTZ, y0 = kGhost + blockIdx.y * kMTY;
  const int xb = kGhost + blockIdx.z * XC;
  const int xe = min(xb + XC, g.nx - kGhost);
  const int k = z0 + tz, j = y0 + ty;
  const bool active = k < g.nz - kGhost && j < g.ny - kGhost;
  if (tid == 0) {
    for (int s = 0; s < kRing; ++s) mbar_init(&bar[s], 1);
    fence_barrier_init();
  }
  __syncthreads();
  constexpr uint32_t kBytes = (kXW * kXH + kYSlot + kZSlot) * 4;
  auto issue = [&](int s, int x) {
    mbar_arrive_expect_tx(&bar[s], kBytes);
    tma_load_3d(rx[s], &tm_vx, &bar[s], z0 - 4, y0 - 1, x);
    tma_load_3d(ry[s], &tm_vy, &bar[s], z0 - 4, y0 - 8, x);
    tma_load_3d(rz[s], &tm_vz, &bar[s], z0 - 8, y0 - 1, x);
  };
  if (tid == 0)
    for (int s = 0; s < 3; ++s) issue(s, xb - 1 + s);
  const int64_t sx = g.sx;
  const int64_t col = (int64_t)j * g.sy + k;
  const float* __restrict__ vx = A.f.v[0];
  float* p = A.f.p;
  // rotated register queue as in vel3d_march: at plane x = xb + 16 m + u, vx[x - 8 + t] is
  // r[(u + t) & 15]
  float r[16];
#pragma unroll
  for (int t = 0; t < 16; ++t) r[t] = active ? __ldg(vx + (int64_t)(xb - 8 + t) * sx + col) : 0.f;
  const int xi = (ty + 1) * kXW + (tz + 4);
  const int yi = (ty + 8) * kYW + (tz + 4);
  const int zi = (ty + 1) * kZW + (tz + 8);
  for (int x0 = xb; x0 < xe; x0 += 16) {
#pragma unroll
  for (int u = 0; u < 16; ++u) {
    const int x = x0 + u;
    if (x >= xe) break;  // uniform over the block
    const int64_t c = (int64_t)x * sx + col;
    CP cp;
    if (active) cp.load(A, c);
    const float rn = active ? __ldg(vx + (int64_t)(x + 8) * sx + col) : 0.f;
    __syncthreads();
    if (tid == 0 && x + 1 < xe) {
      fence_proxy_async_smem();
      issue((u + 3) % kRing, x + 2);
    }
    if (u == 0 && x0 == xb) {
      mbar_wait_bounded(&bar[0], 0, status);
      mbar_wait_bounded(&bar[1], 0, status);
    }
    mbar_wait_bounded(&bar[(u + 2) % kRing], ((u + 2) / kRing) & 1, status);
    const float* Xm = rx[u % kRing];
    const float* X0 = rx[(u + 1) % kRing];
    const float* Ym = ry[u % kRing];
    const float* Y0 = ry[(u + 1) % kRing];
    const float* Y1 = ry[(u + 2) % kRing];
    const float* Zm = rz[u % kRing];
    const float* Z0 = rz[(u + 1) % kRing];
    const float* Z1 = rz[(u + 2) % kRing];
    if (active) {
      float cm[8], co;
      load_taps(A.m.taps, cp.dc, cm, co);
      float dx = 0.f, dy = 0.f, dz = 0.f;
#pragma unroll
      for (int m = 1; m <= 8; ++m) {
        dx = fmaf(cm[m - 1], r[(u + 7 + m) & 15] - r[(u + 8 - m) & 15], dx);
        dy = fmaf(cm[m - 1], Y0[yi + (m - 1) * kYW] - Y0[yi - m * kYW], dy);
        dz = fmaf(cm[m - 1], Z0[zi + (m - 1)] - Z0[zi - m], dz);
      }
      dx = fmaf(co, ((X0[xi + kXW] - Xm[xi + kXW]) + (X0[xi - kXW] - Xm[xi - kXW])) +
                        ((X0[xi + 1] - Xm[xi + 1]) + (X0[xi - 1] - Xm[xi - 1])), dx);
      dy = fmaf(co, ((Y1[yi] - Y1[yi - kYW]) + (Ym[yi] - Ym[yi - kYW])) +
                        ((Y0[yi + 1] - Y0[yi + 1 - kYW]) + (Y0[yi - 1] - Y0[yi - 1 - kYW])), dy);
      dz = fmaf(co, ((Z1[zi] - Z1[zi - 1]) + (Zm[zi] - Zm[zi - 1])) +
                        ((Z0[zi + kZW] - Z0[zi + kZW - 1]) + (Z0[zi - kZW] - Z0[zi - kZW - 1])), dz);
      const float dd[3] = {dx * g.inv_h[0], dy * g.inv_h[1], dz * g.inv_h[2]};
      cp.update_store(A, c, dd);
    }
    r[u] = rn;  // vx[x + 8]: the sample at t = 15 of plane x + 1
  }
  }
  tile_epilogue(A, p, (blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x, tid,
                kMThreads);
}

}  // namespace fwgb
