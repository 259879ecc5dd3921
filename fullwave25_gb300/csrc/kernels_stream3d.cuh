// 3D plane-march kernels with every operand staged by TMA (isotropic relaxation engine).
//
// Same march as vel3d_march / prs3d_march (block = 32 z x 8 y columns walking XC x-planes,
// x taps from a register queue, y/z and off-axis taps from TMA-staged halo planes in a 4-slot
// ring), but the point-wise operands of a plane — the state fields the update reads and the
// coefficient maps — are not loaded by the threads: one thread issues, per plane, three or four
// tiled TMA loads (4D boxes over the state and map allocations, whose fields are stacked along a
// fourth axis, plus the tap-index map) into a kPS-stage ring in dynamic shared memory, kPS - 1
// planes ahead of the plane being computed. The HBM latency of every read is then hidden by the
// march itself instead of by the number of resident warps. Writes stay plain coalesced stores.
// The cell updates are the CellVelT / CellPrsT ones (same operation order: bit-identical).
//
// Point-wise stage layout (floats; box order z fastest, then y, then field):
//   velocity: state fields v_x v_y v_z psi_x1 psi_x2 psi_y1 psi_y2 psi_z1 psi_z2 [9][8][32],
//             maps rdt_rho inv_ku au1 bu1 au2 bu2 [6][8][32], tap index [8][32] (int32)
//   pressure: p [8][32], phi_x1 .. phi_z2 [6][8][32], maps dt_k inv_kx ax1 bx1 ax2 bx2
//             (+ beta2dt) [6 or 7][8][32], tap index [8][32]
#pragma once
#include "engine_common.cuh"
#include "kernels_march3d.cuh"
#include "tma.cuh"

namespace fwgb {

constexpr int kCell = kMThreads;                  // cells per plane of a block (256)
constexpr int kVelStateF = 9, kVelMapF = 6;       // field counts of the velocity boxes
constexpr int kPrsPhiF = 6;
constexpr int kStateV0 = 1, kStatePhi0 = 10;      // first field of v and of phi in the state

template <int kPS>
constexpr size_t vel_stream_smem() {
  return (size_t)kPS * ((kVelStateF + kVelMapF) * kCell * 4 + kCell * sizeof(uint16_t));
}
template <int kPS, bool kBeta>
constexpr size_t prs_stream_smem() {
  return (size_t)kPS *
         ((1 + kPrsPhiF + kVelMapF + (kBeta ? 1 : 0)) * kCell * 4 + kCell * sizeof(uint16_t));
}

struct StreamMaps {
  CUtensorMap vstate;   // state, box {32, 8, 1, 9} (v, psi)
  CUtensorMap vmaps;    // maps,  box {32, 8, 1, 6} (velocity maps)
  CUtensorMap pstate;   // state, box {32, 8, 1, 1} (p)
  CUtensorMap phi;      // state, box {32, 8, 1, 6} (phi)
  CUtensorMap pmaps6;   // maps,  box {32, 8, 1, 6} (pressure maps)
  CUtensorMap pmaps7;   // maps,  box {32, 8, 1, 7} (pressure maps + beta2dt)
  CUtensorMap dcmap;    // 16-bit tap index, box {32, 8, 1}
};

template <int XC, int kPS, int kMapSlotVel>
__global__ void __launch_bounds__(kMThreads, 3)
vel3d_stream(const StepArgs A, const __grid_constant__ CUtensorMap tm_p,
             const __grid_constant__ CUtensorMap tm_st, const __grid_constant__ CUtensorMap tm_mp,
             const __grid_constant__ CUtensorMap tm_dc) {
  pdl_entry();
  __shared__ alignas(128) float ring[kRing][kPSlot];
  __shared__ alignas(8) uint64_t bar[kRing];
  __shared__ alignas(8) uint64_t pbar[kPS];
  extern __shared__ __align__(128) float dyn[];
  float* pst = dyn;                                             // [kPS][9][256]
  float* pmp = pst + kPS * kVelStateF * kCell;                  // [kPS][6][256]
  uint16_t* pdc = reinterpret_cast<uint16_t*>(pmp + kPS * kVelMapF * kCell);  // [kPS][256]
  const Grid& g = A.g;
  int* status = A.step + 1;
  const int tz = threadIdx.x, ty = threadIdx.y, tid = ty * kMTZ + tz;
  const int z0 = kGhost + blockIdx.x * kMTZ, y0 = kGhost + blockIdx.y * kMTY;
  const int xb = kGhost + blockIdx.z * XC;
  const int xe = min(xb + XC, g.nx - kGhost);
  const int k = z0 + tz, j = y0 + ty;
  const bool active = k < g.nz - kGhost && j < g.ny - kGhost;
  if (smem_u32(dyn) & 127u) {  // TMA destinations need 128-byte alignment: refuse, do not fault
    if (tid == 0) atomicOr(status, kStatusAlign);
    return;
  }
  if (blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0 && tid == 0) *A.step += 1;
  if (tid == 0) {
    for (int s = 0; s < kRing; ++s) mbar_init(&bar[s], 1);
    for (int s = 0; s < kPS; ++s) mbar_init(&pbar[s], 1);
    fence_barrier_init();
  }
  __syncthreads();
  constexpr uint32_t kBytes = kPSlot * 4;
  constexpr uint32_t kPBytes = (kVelStateF + kVelMapF) * kCell * 4 + kCell * sizeof(uint16_t);
  auto issue_pw = [&](int slot, int x) {
    mbar_arrive_expect_tx(&pbar[slot], kPBytes);
    tma_load_4d(pst + slot * kVelStateF * kCell, &tm_st, &pbar[slot], z0, y0, x, kStateV0);
    tma_load_4d(pmp + slot * kVelMapF * kCell, &tm_mp, &pbar[slot], z0, y0, x, kMapSlotVel);
    tma_load_3d(pdc + slot * kCell, &tm_dc, &pbar[slot], z0, y0, x);
  };
  if (tid == 0) {
    for (int s = 0; s < 3; ++s) {  // halo planes xb-1, xb, xb+1
      mbar_arrive_expect_tx(&bar[s], kBytes);
      tma_load_3d(ring[s], &tm_p, &bar[s], z0 - 8, y0 - 8, xb - 1 + s);
    }
    for (int d = 0; d < kPS - 1 && xb + d < xe; ++d) issue_pw(d, xb + d);
  }
  const int64_t sx = g.sx;
  const int64_t col = (int64_t)j * g.sy + k;
  const float* __restrict__ p = A.f.p;
  float q[16];  // q[t] = p[x - 7 + t]
#pragma unroll
  for (int t = 0; t < 16; ++t) q[t] = active ? __ldg(p + (int64_t)(xb - 7 + t) * sx + col) : 0.f;
  const int si = (ty + 8) * kPW + (tz + 8);
  for (int x = xb; x < xe; ++x) {
    const int it = x - xb;
    const int64_t c = (int64_t)x * sx + col;
    const float qn = (active && x + 9 < g.nx) ? __ldg(p + (int64_t)(x + 9) * sx + col) : 0.f;
    __syncthreads();  // the halo slot of plane x-2 and the point-wise slot of plane x-1 are free
    if (tid == 0) {
      fence_proxy_async_smem();
      if (x + 1 < xe) {
        const int s = (it + 3) % kRing;
        mbar_arrive_expect_tx(&bar[s], kBytes);
        tma_load_3d(ring[s], &tm_p, &bar[s], z0 - 8, y0 - 8, x + 2);
      }
      if (x + kPS - 1 < xe) issue_pw((it + kPS - 1) % kPS, x + kPS - 1);
    }
    if (it == 0) {
      mbar_wait_bounded(&bar[0], 0, status);
      mbar_wait_bounded(&bar[1], 0, status);
    }
    mbar_wait_bounded(&bar[(it + 2) % kRing], ((it + 2) / kRing) & 1, status);
    const int ps = it % kPS;
    mbar_wait_bounded(&pbar[ps], (it / kPS) & 1, status);
    const float* Pm = ring[it % kRing];
    const float* P0 = ring[(it + 1) % kRing];
    const float* P1 = ring[(it + 2) % kRing];
    if (active) {
      const float* st = pst + ps * kVelStateF * kCell + tid;
      const float* mp = pmp + ps * kVelMapF * kCell + tid;
      CellVelT<3, false> cv;
      cv.dc = pdc[ps * kCell + tid];
      cv.rr = mp[0 * kCell];
      cv.iku[0] = mp[1 * kCell];
      cv.a1[0] = mp[2 * kCell];
      cv.b1[0] = mp[3 * kCell];
      cv.a2[0] = mp[4 * kCell];
      cv.b2[0] = mp[5 * kCell];
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        cv.v[a] = st[a * kCell];
        cv.s1[a] = st[(3 + 2 * a) * kCell];
        cv.s2[a] = st[(4 + 2 * a) * kCell];
      }
      float cm[8], co;
      load_taps(A.m.taps, cv.dc, cm, co);
      float gx = 0.f, gy = 0.f, gz = 0.f;
#pragma unroll
      for (int m = 1; m <= 8; ++m) {
        gx = fmaf(cm[m - 1], q[7 + m] - q[8 - m], gx);
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
#pragma unroll
    for (int t = 0; t < 15; ++t) q[t] = q[t + 1];
    q[15] = qn;
  }
}

template <int XC, int kPS, bool kBeta, int kMapSlotPrs>
__global__ void __launch_bounds__(kMThreads, 3)
prs3d_stream(const StepArgs A, const __grid_constant__ CUtensorMap tm_vx,
             const __grid_constant__ CUtensorMap tm_vy, const __grid_constant__ CUtensorMap tm_vz,
             const __grid_constant__ CUtensorMap tm_pp, const __grid_constant__ CUtensorMap tm_phi,
             const __grid_constant__ CUtensorMap tm_mp, const __grid_constant__ CUtensorMap tm_dc) {
  pdl_entry();
  constexpr int kMapF = kVelMapF + (kBeta ? 1 : 0);
  __shared__ alignas(128) float rx[kRing][kXSlot];
  __shared__ alignas(128) float ry[kRing][kYSlot];
  __shared__ alignas(128) float rz[kRing][kZSlot];
  __shared__ alignas(8) uint64_t bar[kRing];
  __shared__ alignas(8) uint64_t pbar[kPS];
  extern __shared__ __align__(128) float dyn[];
  float* ppp = dyn;                                            // [kPS][256]
  float* pph = ppp + kPS * kCell;                              // [kPS][6][256]
  float* pmp = pph + kPS * kPrsPhiF * kCell;                   // [kPS][kMapF][256]
  uint16_t* pdc = reinterpret_cast<uint16_t*>(pmp + kPS * kMapF * kCell);  // [kPS][256]
  const Grid& g = A.g;
  int* status = A.step + 1;
  const int tz = threadIdx.x, ty = threadIdx.y, tid = ty * kMTZ + tz;
  const int z0 = kGhost + blockIdx.x * kMTZ, y0 = kGhost + blockIdx.y * kMTY;
  const int xb = kGhost + blockIdx.z * XC;
  const int xe = min(xb + XC, g.nx - kGhost);
  const int k = z0 + tz, j = y0 + ty;
  const bool active = k < g.nz - kGhost && j < g.ny - kGhost;
  if (smem_u32(dyn) & 127u) {
    if (tid == 0) atomicOr(status, kStatusAlign);
    return;
  }
  if (tid == 0) {
    for (int s = 0; s < kRing; ++s) mbar_init(&bar[s], 1);
    for (int s = 0; s < kPS; ++s) mbar_init(&pbar[s], 1);
    fence_barrier_init();
  }
  __syncthreads();
  constexpr uint32_t kBytes = (kXW * kXH + kYSlot + kZSlot) * 4;
  constexpr uint32_t kPBytes = (1 + kPrsPhiF + kMapF) * kCell * 4 + kCell * sizeof(uint16_t);
  auto issue = [&](int s, int x) {
    mbar_arrive_expect_tx(&bar[s], kBytes);
    tma_load_3d(rx[s], &tm_vx, &bar[s], z0 - 4, y0 - 1, x);
    tma_load_3d(ry[s], &tm_vy, &bar[s], z0 - 4, y0 - 8, x);
    tma_load_3d(rz[s], &tm_vz, &bar[s], z0 - 8, y0 - 1, x);
  };
  auto issue_pw = [&](int slot, int x) {
    mbar_arrive_expect_tx(&pbar[slot], kPBytes);
    tma_load_4d(ppp + slot * kCell, &tm_pp, &pbar[slot], z0, y0, x, 0);
    tma_load_4d(pph + slot * kPrsPhiF * kCell, &tm_phi, &pbar[slot], z0, y0, x, kStatePhi0);
    tma_load_4d(pmp + slot * kMapF * kCell, &tm_mp, &pbar[slot], z0, y0, x, kMapSlotPrs);
    tma_load_3d(pdc + slot * kCell, &tm_dc, &pbar[slot], z0, y0, x);
  };
  if (tid == 0) {
    for (int s = 0; s < 3; ++s) issue(s, xb - 1 + s);
    for (int d = 0; d < kPS - 1 && xb + d < xe; ++d) issue_pw(d, xb + d);
  }
  const int64_t sx = g.sx;
  const int64_t col = (int64_t)j * g.sy + k;
  const float* __restrict__ vx = A.f.v[0];
  float* p = A.f.p;
  float r[16];  // r[t] = vx[x - 8 + t]
#pragma unroll
  for (int t = 0; t < 16; ++t) r[t] = active ? __ldg(vx + (int64_t)(xb - 8 + t) * sx + col) : 0.f;
  const int xi = (ty + 1) * kXW + (tz + 4);
  const int yi = (ty + 8) * kYW + (tz + 4);
  const int zi = (ty + 1) * kZW + (tz + 8);
  for (int x = xb; x < xe; ++x) {
    const int it = x - xb;
    const int64_t c = (int64_t)x * sx + col;
    const float rn = active ? __ldg(vx + (int64_t)(x + 8) * sx + col) : 0.f;
    __syncthreads();
    if (tid == 0) {
      fence_proxy_async_smem();
      if (x + 1 < xe) issue((it + 3) % kRing, x + 2);
      if (x + kPS - 1 < xe) issue_pw((it + kPS - 1) % kPS, x + kPS - 1);
    }
    if (it == 0) {
      mbar_wait_bounded(&bar[0], 0, status);
      mbar_wait_bounded(&bar[1], 0, status);
    }
    mbar_wait_bounded(&bar[(it + 2) % kRing], ((it + 2) / kRing) & 1, status);
    const int ps = it % kPS;
    mbar_wait_bounded(&pbar[ps], (it / kPS) & 1, status);
    const float* Xm = rx[it % kRing];
    const float* X0 = rx[(it + 1) % kRing];
    const float* Ym = ry[it % kRing];
    const float* Y0 = ry[(it + 1) % kRing];
    const float* Y1 = ry[(it + 2) % kRing];
    const float* Zm = rz[it % kRing];
    const float* Z0 = rz[(it + 1) % kRing];
    const float* Z1 = rz[(it + 2) % kRing];
    if (active) {
      const float* ph = pph + ps * kPrsPhiF * kCell + tid;
      const float* mp = pmp + ps * kMapF * kCell + tid;
      CellPrsT<3, kBeta, false> cp;
      cp.dc = pdc[ps * kCell + tid];
      cp.dtk = mp[0 * kCell];
      cp.ikx[0] = mp[1 * kCell];
      cp.a1[0] = mp[2 * kCell];
      cp.b1[0] = mp[3 * kCell];
      cp.a2[0] = mp[4 * kCell];
      cp.b2[0] = mp[5 * kCell];
      cp.b2dt = kBeta ? mp[6 * kCell] : 0.f;
      cp.pc = ppp[ps * kCell + tid];
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        cp.f1[a] = ph[(2 * a) * kCell];
        cp.f2[a] = ph[(2 * a + 1) * kCell];
      }
      float cm[8], co;
      load_taps(A.m.taps, cp.dc, cm, co);
      float dx = 0.f, dy = 0.f, dz = 0.f;
#pragma unroll
      for (int m = 1; m <= 8; ++m) {
        dx = fmaf(cm[m - 1], r[7 + m] - r[8 - m], dx);
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
#pragma unroll
    for (int t = 0; t < 15; ++t) r[t] = r[t + 1];
    r[15] = rn;
  }
  tile_epilogue(A, p, (blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x, tid,
                kMThreads);
}

}  // namespace fwgb
