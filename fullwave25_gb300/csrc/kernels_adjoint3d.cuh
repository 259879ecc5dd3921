// Discrete adjoint of the 3D time step (isotropic relaxation engine): the reverse step of
// kernels_adjoint2d.cuh with three derivative axes; and, further down, the reverse steps of the
// exponential-attenuation and anisotropic relaxation engines in 2D and 3D. Every pressure
// adjoint has a kBeta variant for the nonlinear term. One thread per body cell (blocks of
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

template <bool kF64, bool kS, bool kBeta = false>
__global__ void __launch_bounds__(256) adj3d_prs(const AdjArgs A) {
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
__global__ void __launch_bounds__(256) adj3d_vel(const AdjArgs A) {
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
