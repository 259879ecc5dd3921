// Reverse steps of the exponential-attenuation and anisotropic relaxation engines, for 2D and 3D
// grids alike (ND template parameter): one thread per body cell, operands through the read-only
// path, the tap table in shared memory when it fits; the stencils and their transposes are the
// 2D ones of kernels_adjoint2d.cuh or the 3D ones of kernels_adjoint3d.cuh. Every pressure
// adjoint has a kBeta variant for the nonlinear term.
#pragma once
#include "kernels_adjoint3d.cuh"

namespace fwgb {

// ---- exponential-attenuation engine, 2D and 3D -----------------------------------------------
// Forward step: v'_a = ae (v_a - r D_a p), p' = ae (p - k sum_a D'_a v'_a). Reverse of step n,
// after adj2d/adj3d_assemble and adj2d_io / adj2d_zero have formed lam_p (= dJ/dp' on the body):
//   adjx_prs: d = sum_a D'_a v'_a (S_{n+1});  lam_d = -ae k lam_p  (one field, every axis);
//             gradients dt_k -= ae d lam_p, a_exp += lam_p (p^n - k d);  lam_p <- ae lam_p
//             (kBeta: k = dt K + 2 dt beta p^n, lam_p <- ae (1 - 2 dt beta d) lam_p and
//             2 dt beta -= ae p^n d lam_p)
//   adjx_vel: lam_v_a += D'_a^T lam_d;  g_a = D_a p^n;  lam_g_a = -ae r lam_v_a;
//             gradients rdt_rho -= ae g_a lam_v_a, a_exp += lam_v_a (v_a^n - r g_a);
//             lam_v_a <- ae lam_v_a
// The a_exp gradient goes to the au1 slot (the map slot the engine keeps a_exp in).

template <int ND>
__device__ __forceinline__ bool adjn_cell(const Grid& g, int64_t* c) {
  if constexpr (ND == 2) return adj_cell(g, c);
  else return adj3_cell(g, c);
}
template <int ND, bool kS>
__device__ __forceinline__ float divn_at(const Maps& m, const TapSrc<kS>& T, const float* v,
                                         int64_t c, const Grid& g, int a) {
  if constexpr (ND == 2) return div_at(m, T, v, c, a == 0 ? g.sx : 1, a == 0 ? 1 : g.sx, g.inv_h[a]);
  else return div3_at(m, T, v, c, axis3(g, a));
}
template <int ND, bool kS>
__device__ __forceinline__ float gradn_at(const Maps& m, const TapSrc<kS>& T, const float* f,
                                          int64_t c, const Grid& g, int a) {
  if constexpr (ND == 2) return grad_at(m, T, f, c, a == 0 ? g.sx : 1, a == 0 ? 1 : g.sx, g.inv_h[a]);
  else return grad3_at(m, T, f, c, axis3(g, a));
}
template <int ND, bool kS>
__device__ __forceinline__ float divn_T_at(const Maps& m, const TapSrc<kS>& T, const float* u,
                                           int64_t q, const Grid& g, int a) {
  if constexpr (ND == 2) return div_T_at(m, T, u, q, a == 0 ? g.sx : 1, a == 0 ? 1 : g.sx, g.inv_h[a]);
  else return div3_T_at(m, T, u, q, axis3(g, a));
}

// One step's contribution v (formed in FP32) to gradient map q: into the segment's FP32 partial,
// or (kF64) straight into the FP64 time sum.
template <bool kF64>
__device__ __forceinline__ void adj_add_grad(const AdjArgs& A, int q, int64_t c, float v) {
  if constexpr (kF64) A.grad[q][c] += (double)v;
  else A.g32[q][c] += v;
}

template <int ND, bool kF64, bool kS, bool kBeta = false>
__global__ void __launch_bounds__(256) adjx_prs(const AdjArgs A) {
  extern __shared__ float s_taps[];
  const TapSrc<kS> T = stage_taps<kS>(A, s_taps);
  int64_t c;
  if (!adjn_cell<ND>(A.g, &c)) return;
  float d = 0.f;
#pragma unroll
  for (int a = 0; a < ND; ++a) d += divn_at<ND>(A.m, T, S_v(A.Sn1, A.fs, a), c, A.g, a);
  const float lp = A.lam_p[c];
  const float dtk = __ldg(A.m.dt_k + c), ae = __ldg(A.m.a_exp + c);
  const float pn = __ldg(S_p(A.Sn, A.fs) + c);
  const float b2dt = kBeta ? __ldg(A.m.beta2dt + c) : 0.f;
  const float k = kBeta ? fmaf(b2dt, pn, dtk) : dtk;
  A.lam_d[0][c] = -ae * k * lp;
  A.lam_p[c] = kBeta ? ae * (lp - b2dt * d * lp) : ae * lp;
  adj_add_grad<kF64>(A, kGDtK, c, -(ae * d * lp));
  adj_add_grad<kF64>(A, kGAu1, c, lp * (pn - k * d));
  if constexpr (kBeta) adj_add_grad<kF64>(A, A.beta_slot, c, -(ae * pn * d * lp));
}

template <int ND, bool kF64, bool kS>
__global__ void __launch_bounds__(256) adjx_vel(const AdjArgs A) {
  extern __shared__ float s_taps[];
  const TapSrc<kS> T = stage_taps<kS>(A, s_taps);
  int64_t c;
  if (!adjn_cell<ND>(A.g, &c)) return;
  const float r = __ldg(A.m.rdt_rho + c), ae = __ldg(A.m.a_exp + c);
  float g_r = 0.f, g_ae = 0.f;
#pragma unroll
  for (int a = 0; a < ND; ++a) {
    const float lv = A.lam_v[a][c] + divn_T_at<ND>(A.m, T, A.lam_d[0], c, A.g, a);
    const float g = gradn_at<ND>(A.m, T, S_p(A.Sn, A.fs), c, A.g, a);
    const float vn = __ldg(S_v(A.Sn, A.fs, a) + c);
    A.lam_g[a][c] = -ae * r * lv;
    A.lam_v[a][c] = ae * lv;
    g_r -= ae * g * lv;
    g_ae += lv * (vn - r * g);
  }
  adj_add_grad<kF64>(A, kGRdtRho, c, g_r);
  adj_add_grad<kF64>(A, kGAu1, c, g_ae);
}

// ---- anisotropic relaxation engine, 2D and 3D -----------------------------------------------
// The relaxation adjoint with one map set per derivative axis: the point-wise algebra of
// adj_prs_point / adj_vel_point with axis a's maps, and one gradient map per (map, axis).
// Gradient slots: 0 dt/rho, 1 dt*K, 2 + 5 a + j the pressure-gradient maps of axis a, 2 + 5 ND
// + 5 a + j the velocity-divergence maps, j = 1/kappa, a1, b1, a2, b2.

template <bool kF64, int ND, bool kBeta = false>
__device__ __forceinline__ void adja_prs_point(const AdjArgs& A, int64_t c, const float lp,
                                               const float (&d)[ND]) {
  const int64_t fs = A.fs;
  const float dtk = __ldg(A.m.dt_k + c);
  const float b2dt = kBeta ? __ldg(A.m.beta2dt + c) : 0.f;
  const float pn = kBeta ? __ldg(S_p(A.Sn, fs) + c) : 0.f;
  const float k = kBeta ? fmaf(b2dt, pn, dtk) : dtk;   // the forward's coefficient of div
  float div = 0.f;
#pragma unroll
  for (int a = 0; a < ND; ++a) {
    const float ikx = __ldg(A.m.inv_kx[a] + c);
    const float ax[2] = {__ldg(A.m.ax[a][0] + c), __ldg(A.m.ax[a][1] + c)};
    const float bx[2] = {__ldg(A.m.bx[a][0] + c), __ldg(A.m.bx[a][1] + c)};
    const float n1 = __ldg(S_phiN<ND>(A.Sn1, fs, a, 0) + c), n2 = __ldg(S_phiN<ND>(A.Sn1, fs, a, 1) + c);
    div += fmaf(d[a], ikx, n1) + n2;
    float lam_d = -k * ikx * lp;
    float g_ax[2], g_bx[2];
#pragma unroll
    for (int nu = 0; nu < 2; ++nu) {
      const float L = A.lam_phi[a][nu][c] - k * lp;
      lam_d = fmaf(ax[nu], L, lam_d);
      g_ax[nu] = L * d[a];
      g_bx[nu] = L * __ldg(S_phiN<ND>(A.Sn, fs, a, nu) + c);
      A.lam_phi[a][nu][c] = bx[nu] * L;
    }
    A.lam_d[a][c] = lam_d;
    const int q = 2 + 5 * ND + 5 * a;
    adj_add_grad<kF64>(A, q, c, -(k * lp * d[a]));
    adj_add_grad<kF64>(A, q + 1, c, g_ax[0]);
    adj_add_grad<kF64>(A, q + 2, c, g_bx[0]);
    adj_add_grad<kF64>(A, q + 3, c, g_ax[1]);
    adj_add_grad<kF64>(A, q + 4, c, g_bx[1]);
  }
  adj_add_grad<kF64>(A, kGDtK, c, -(div * lp));
  if constexpr (kBeta) {
    A.lam_p[c] = lp - b2dt * div * lp;
    adj_add_grad<kF64>(A, A.beta_slot, c, -(pn * div * lp));
  }
}

template <bool kF64, int ND>
__device__ __forceinline__ void adja_vel_point(const AdjArgs& A, int64_t c, const float (&dT)[ND],
                                               const float (&gr)[ND]) {
  const int64_t fs = A.fs;
  const float r = __ldg(A.m.rdt_rho + c);
  float g_r = 0.f;
#pragma unroll
  for (int a = 0; a < ND; ++a) {
    const float iku = __ldg(A.m.inv_ku[a] + c);
    const float au[2] = {__ldg(A.m.au[a][0] + c), __ldg(A.m.au[a][1] + c)};
    const float bu[2] = {__ldg(A.m.bu[a][0] + c), __ldg(A.m.bu[a][1] + c)};
    const float lv = A.lam_v[a][c] + dT[a];
    const float p1 = __ldg(S_psiN<ND>(A.Sn1, fs, a, 0) + c), p2 = __ldg(S_psiN<ND>(A.Sn1, fs, a, 1) + c);
    float lam_g = -r * iku * lv;
    float g_au[2], g_bu[2];
#pragma unroll
    for (int nu = 0; nu < 2; ++nu) {
      const float M = A.lam_psi[a][nu][c] - r * lv;
      lam_g = fmaf(au[nu], M, lam_g);
      g_au[nu] = M * gr[a];
      g_bu[nu] = M * __ldg(S_psiN<ND>(A.Sn, fs, a, nu) + c);
      A.lam_psi[a][nu][c] = bu[nu] * M;
    }
    g_r -= lv * (fmaf(gr[a], iku, p1) + p2);
    A.lam_v[a][c] = lv;
    A.lam_g[a][c] = lam_g;
    const int q = 2 + 5 * a;
    adj_add_grad<kF64>(A, q, c, -(r * gr[a] * lv));
    adj_add_grad<kF64>(A, q + 1, c, g_au[0]);
    adj_add_grad<kF64>(A, q + 2, c, g_bu[0]);
    adj_add_grad<kF64>(A, q + 3, c, g_au[1]);
    adj_add_grad<kF64>(A, q + 4, c, g_bu[1]);
  }
  adj_add_grad<kF64>(A, kGRdtRho, c, g_r);
}

template <int ND, bool kF64, bool kS, bool kBeta = false>
__global__ void __launch_bounds__(256) adja_prs(const AdjArgs A) {
  extern __shared__ float s_taps[];
  const TapSrc<kS> T = stage_taps<kS>(A, s_taps);
  int64_t c;
  if (!adjn_cell<ND>(A.g, &c)) return;
  float d[ND];
#pragma unroll
  for (int a = 0; a < ND; ++a) d[a] = divn_at<ND>(A.m, T, S_v(A.Sn1, A.fs, a), c, A.g, a);
  adja_prs_point<kF64, ND, kBeta>(A, c, A.lam_p[c], d);
}

template <int ND, bool kF64, bool kS>
__global__ void __launch_bounds__(256) adja_vel(const AdjArgs A) {
  extern __shared__ float s_taps[];
  const TapSrc<kS> T = stage_taps<kS>(A, s_taps);
  int64_t c;
  if (!adjn_cell<ND>(A.g, &c)) return;
  float dT[ND], gr[ND];
#pragma unroll
  for (int a = 0; a < ND; ++a) {
    dT[a] = divn_T_at<ND>(A.m, T, A.lam_d[a], c, A.g, a);
    gr[a] = gradn_at<ND>(A.m, T, S_p(A.Sn, A.fs), c, A.g, a);
  }
  adja_vel_point<kF64, ND>(A, c, dT, gr);
}

}  // namespace fwgb
