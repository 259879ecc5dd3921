// Discrete adjoint of the 3D time step (isotropic relaxation engine, with the kBeta variant of
// the pressure adjoint for the nonlinear term): the reverse step of kernels_adjoint2d.cuh with
// three derivative axes. One thread per body cell (blocks of
// 32 (z) x 8 (y) cells of one x plane), operands through the read-only path, the tap table in
// shared memory when it fits. Per reverse step n, in order:
//   adj3d_assemble   lam_p += sum_a D_a^T lam_g_a           (lam_g from step n+1)
//   adj2d_io/zero    lam_p[outc] += r_n ; lam_p[icczero] = 0 ; lam_p[icc] = 0 (n < nTic)
//   adj3d_prs        pressure adjoint (lam_d, lam_phi) and the pressure-map gradients
//   adj3d_vel        lam_v += D'_a^T lam_d_a, velocity adjoint (lam_g, lam_psi) and the
//                    velocity-map gradients
// and at the end of every checkpoint segment adj3d_merge adds the FP32 segment partials into the
// FP64 time sums. The point-wise algebra is adj_prs_cell / adj_vel_cell with ND = 3.
//
// Stencils (operation order of vel3d_direct / prs3d_direct): for derivative axis a with stride
// se and transverse strides sf0 < sf1 in axis order (x: sy, 1; y: sx, 1; z: sx, sy)
//   D_a f  = [sum_m c_m (f[m se] - f[-(m-1) se])
//             + c_o (((f[se+sf0] - f[sf0]) + (f[se-sf0] - f[-sf0])) + (same with sf1))] / h_a
//   D'_a v = [sum_m c_m (v[(m-1) se] - v[-m se])
//             + c_o (((v[sf0] - v[sf0-se]) + (v[-sf0] - v[-sf0-se])) + (same with sf1))] / h_a
// with the taps of the cell being updated; the transposes gather, at q, every body cell's term
// that touches q, weighted by that cell's own taps.
#pragma once
#include "kernels_adjoint2d.cuh"

namespace fwgb {

constexpr int kA3TZ = 32, kA3TY = 8;   // block: 32 z x 8 y cells of one x plane

struct Axis3 {
  int64_t se, sf0, sf1;   // stride of the derivative axis, then of the two transverse axes
  float inv_h;
};

__device__ __forceinline__ Axis3 axis3(const Grid& g, int a) {
  if (a == 0) return {g.sx, g.sy, 1, g.inv_h[0]};
  if (a == 1) return {g.sy, g.sx, 1, g.inv_h[1]};
  return {1, g.sx, g.sy, g.inv_h[2]};
}

__device__ __forceinline__ bool adj3_cell(const Grid& g, int64_t* c) {
  const int k = kGhost + blockIdx.x * kA3TZ + threadIdx.x;
  const int j = kGhost + blockIdx.y * kA3TY + threadIdx.y;
  const int i = kGhost + blockIdx.z;
  if (i >= g.nx - kGhost || j >= g.ny - kGhost || k >= g.nz - kGhost) return false;
  *c = (int64_t)i * g.sx + (int64_t)j * g.sy + k;
  return true;
}

template <bool kS>
__device__ __forceinline__ float grad3_at(const Maps& m, const TapSrc<kS>& T, const float* f,
                                          int64_t c, const Axis3& x) {
  float cm[8], co;
  T.load(__ldg(m.dcmap + c), cm, co);
  auto F = [&](int64_t o) { return __ldg(f + c + o); };
  float g = 0.f;
#pragma unroll
  for (int k = 1; k <= 8; ++k) g = fmaf(cm[k - 1], F(k * x.se) - F(-(k - 1) * x.se), g);
  g = fmaf(co, ((F(x.se + x.sf0) - F(x.sf0)) + (F(x.se - x.sf0) - F(-x.sf0))) +
                   ((F(x.se + x.sf1) - F(x.sf1)) + (F(x.se - x.sf1) - F(-x.sf1))), g);
  return g * x.inv_h;
}

template <bool kS>
__device__ __forceinline__ float div3_at(const Maps& m, const TapSrc<kS>& T, const float* v,
                                         int64_t c, const Axis3& x) {
  float cm[8], co;
  T.load(__ldg(m.dcmap + c), cm, co);
  auto V = [&](int64_t o) { return __ldg(v + c + o); };
  float d = 0.f;
#pragma unroll
  for (int k = 1; k <= 8; ++k) d = fmaf(cm[k - 1], V((k - 1) * x.se) - V(-k * x.se), d);
  d = fmaf(co, ((V(x.sf0) - V(x.sf0 - x.se)) + (V(-x.sf0) - V(-x.sf0 - x.se))) +
                   ((V(x.sf1) - V(x.sf1 - x.se)) + (V(-x.sf1) - V(-x.sf1 - x.se))), d);
  return d * x.inv_h;
}

// (D_a^T u)(q); u is zero outside the body
template <bool kS>
__device__ __forceinline__ float grad3_T_at(const Maps& m, const TapSrc<kS>& T, const float* u,
                                            int64_t q, const Axis3& x) {
  float acc = 0.f;
#pragma unroll
  for (int k = 1; k <= 8; ++k) {
    const int64_t c1 = q - k * x.se, c2 = q + (k - 1) * x.se;
    acc += tap_of(m, T, c1, k - 1) * __ldg(u + c1) - tap_of(m, T, c2, k - 1) * __ldg(u + c2);
  }
#pragma unroll
  for (int b = 0; b < 2; ++b) {
    const int64_t sf = b == 0 ? x.sf0 : x.sf1;
#pragma unroll
    for (int s = -1; s <= 1; s += 2) {
      const int64_t c1 = q - x.se - s * sf, c2 = q - s * sf;
      acc += tap_of(m, T, c1, 8) * __ldg(u + c1) - tap_of(m, T, c2, 8) * __ldg(u + c2);
    }
  }
  return acc * x.inv_h;
}

// (D'_a^T u)(q)
template <bool kS>
__device__ __forceinline__ float div3_T_at(const Maps& m, const TapSrc<kS>& T, const float* u,
                                           int64_t q, const Axis3& x) {
  float acc = 0.f;
#pragma unroll
  for (int k = 1; k <= 8; ++k) {
    const int64_t c1 = q - (k - 1) * x.se, c2 = q + k * x.se;
    acc += tap_of(m, T, c1, k - 1) * __ldg(u + c1) - tap_of(m, T, c2, k - 1) * __ldg(u + c2);
  }
#pragma unroll
  for (int b = 0; b < 2; ++b) {
    const int64_t sf = b == 0 ? x.sf0 : x.sf1;
#pragma unroll
    for (int s = -1; s <= 1; s += 2) {
      const int64_t c1 = q - s * sf, c2 = q + x.se - s * sf;
      acc += tap_of(m, T, c1, 8) * __ldg(u + c1) - tap_of(m, T, c2, 8) * __ldg(u + c2);
    }
  }
  return acc * x.inv_h;
}

// lam_p += sum_a D_a^T lam_g_a
template <bool kS>
__global__ void __launch_bounds__(256) adj3d_assemble(const AdjArgs A) {
  extern __shared__ float s_taps[];
  const TapSrc<kS> T = stage_taps<kS>(A, s_taps);
  int64_t q;
  if (!adj3_cell(A.g, &q)) return;
  float add = 0.f;
#pragma unroll
  for (int a = 0; a < 3; ++a) add += grad3_T_at(A.m, T, A.lam_g[a], q, axis3(A.g, a));
  A.lam_p[q] += add;
}

// Register caps: 5 blocks per SM for the pressure kernel (48 registers, no spills with the shared
// tap table) and 4 for the velocity kernel (64 registers, ~50 bytes of spills): the kernels are
// latency-bound, and the caps cut the 3D reverse pass at 240^3 from 1.79 to 1.63 s.
template <bool kF64, bool kS, bool kBeta = false>
__global__ void __launch_bounds__(256, 5) adj3d_prs(const AdjArgs A) {
  extern __shared__ float s_taps[];
  const TapSrc<kS> T = stage_taps<kS>(A, s_taps);
  int64_t c;
  if (!adj3_cell(A.g, &c)) return;
  float d[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) d[a] = div3_at(A.m, T, S_v(A.Sn1, A.fs, a), c, axis3(A.g, a));
  adj_prs_point<kF64, 3, kBeta>(A, c, A.lam_p[c], d);
}

template <bool kF64, bool kS>
__global__ void __launch_bounds__(256, 4) adj3d_vel(const AdjArgs A) {
  extern __shared__ float s_taps[];
  const TapSrc<kS> T = stage_taps<kS>(A, s_taps);
  int64_t c;
  if (!adj3_cell(A.g, &c)) return;
  float dT[3], gr[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const Axis3 x = axis3(A.g, a);
    dT[a] = div3_T_at(A.m, T, A.lam_d[a], c, x);
    gr[a] = grad3_at(A.m, T, S_p(A.Sn, A.fs), c, x);
  }
  adj_vel_point<kF64, 3>(A, c, dT, gr);
}

// End of a segment: FP64 time sums += FP32 segment partials; partials reset (body cells).
static __global__ void __launch_bounds__(256) adj3d_merge(const AdjArgs A) {
  int64_t c;
  if (!adj3_cell(A.g, &c)) return;
  for (int q = 0; q < A.n_grad; ++q) {
    A.grad[q][c] += (double)A.g32[q][c];
    A.g32[q][c] = 0.f;
  }
}

}  // namespace fwgb
