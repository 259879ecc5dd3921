// Discrete adjoint of the 2D time step, for gradients of the sensor-trace misfit
// J = 1/2 sum_n || p^{n+1}[outc] - d_n ||^2 with respect to the engine's coefficient maps. The
// steps below are those of the linear isotropic engine (beta = 0); the nonlinear term is the
// kBeta variant of the pressure adjoint (adj_prs_point).
//
// Reverse of step n uses the stored forward states S_n (before the step) and S_{n+1} (after):
//   assemble  lam_p += sum_a D_a^T lam_g_a                      (from step n+1's velocity adjoint)
//   io        lam_p[outc] += r_n ; lam_p[icczero] = 0 ; lam_p[icc] = 0 (n < nTic)
//   pressure  d_a = D'_a v^{n+1/2};  L_nu = lam_phi_nu - k lam_p;
//             lam_d_a = sum_nu ax_nu L_nu - k ikx lam_p;  lam_phi_nu = bx_nu L_nu
//   velocity  lam_v_a += D'_a^T lam_d_a;  g_a = D_a p^n;  M_nu = lam_psi_nu - r lam_v_a;
//             lam_g_a = sum_nu au_nu M_nu - r iku lam_v_a;  lam_psi_nu = bu_nu M_nu
// Gradient contributions are summed over time in FP64, one array per coefficient map.
// The transposes D^T are gathers: output cell q collects the terms of every body cell c whose
// stencil touches q, each weighted by c's own taps.
#pragma once
#include <type_traits>
#include "engine_common.cuh"
#include "kernels_direct.cuh"
#include "tma.cuh"

namespace fwgb {

enum AdjGrad {
  kGRdtRho = 0, kGDtK, kGInvKu, kGInvKx, kGAu1, kGBu1, kGAu2, kGBu2, kGAx1, kGBx1, kGAx2, kGBx2,
  kNumGrad
};
// The anisotropic engine has one map set per derivative axis: 2 + 10 ND gradient maps (dt/rho,
// dt*K, then per axis 1/kappa, a1, b1, a2, b2 of the pressure-gradient maps, then the same of the
// velocity-divergence maps), at most 32 in 3D.
constexpr int kMaxGrad = 33;

struct AdjArgs {
  Grid g;
  Maps m;
  const float* Sn;      // stored state before step n: 11 (2D) / 16 (3D) padded fields, state order
  const float* Sn1;     // stored state after step n
  int64_t fs;           // field stride (padded cells)
  float* lam_p;         // per derivative axis (2 in 2D, 3 in 3D):
  float* lam_v[3];
  float* lam_psi[3][2];
  float* lam_phi[3][2];
  float* lam_d[3];
  float* lam_g[3];
  int ndmap;                 // tap sets in m.taps
  double* grad[kMaxGrad];    // FP64 time sums (kNumGrad maps; anisotropic engine: 2 + 10 ND;
                             // plus one for 2 dt beta when beta is not zero)
  float* g32[kMaxGrad];      // FP32 partial sums of the current segment (segmented mode)
  int n_grad;                // gradient maps in use
  int beta_slot;             // gradient map of 2 dt beta (the last one), or -1
  int* status;               // device status word (bounded waits, alignment)
};

// stored-state field indices in ND dimensions: p, v[ND], psi[a][nu] = 1 + ND + 2a + nu,
// phi[a][nu] = 1 + 3 ND + 2a + nu (2D: psi 3 + 2a + nu, phi 7 + 2a + nu)
__device__ __forceinline__ const float* S_p(const float* S, int64_t) { return S; }
__device__ __forceinline__ const float* S_v(const float* S, int64_t fs, int a) { return S + (1 + a) * fs; }
template <int ND>
__device__ __forceinline__ const float* S_psiN(const float* S, int64_t fs, int a, int nu) {
  return S + (1 + ND + 2 * a + nu) * fs;
}
template <int ND>
__device__ __forceinline__ const float* S_phiN(const float* S, int64_t fs, int a, int nu) {
  return S + (1 + 3 * ND + 2 * a + nu) * fs;
}

// Tap table access: from a shared-memory copy of the table (kS, when it fits) or through the
// read-only path. The transposed stencils read one tap of every neighbour, so the table is read
// ~40 times per cell: the shared copy turns each of those into one L1-latency access.
template <bool kS>
struct TapSrc {
  const float* t;
  __device__ __forceinline__ float tap(int dc, int idx) const {
    if constexpr (kS) return t[dc * kTapStride + idx];
    else return __ldg(t + (size_t)dc * kTapStride + idx);
  }
  __device__ __forceinline__ void load(int dc, float (&c)[8], float& co) const {
    if constexpr (kS) {
      const float* r = t + dc * kTapStride;
#pragma unroll
      for (int k = 0; k < 8; ++k) c[k] = r[k];
      co = r[8];
    } else {
      load_taps(t, dc, c, co);
    }
  }
};

// Copy the tap table into shared memory (all threads of the block; before any early return).
template <bool kS>
__device__ __forceinline__ TapSrc<kS> stage_taps(const AdjArgs& A, float* s_taps) {
  if constexpr (kS) {
    const int n = A.ndmap * kTapStride;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x, nthr = blockDim.x * blockDim.y;
    for (int i = tid; i < n; i += nthr) s_taps[i] = __ldg(A.m.taps + i);
    __syncthreads();
    return TapSrc<kS>{s_taps};
  } else {
    return TapSrc<kS>{A.m.taps};
  }
}

template <bool kS>
__device__ __forceinline__ float tap_of(const Maps& m, const TapSrc<kS>& T, int64_t c, int idx) {
  return T.tap(__ldg(m.dcmap + c), idx);
}

// D_a f at c (the velocity-kernel stencil), same operation order as the forward kernels
template <bool kS>
__device__ __forceinline__ float grad_at(const Maps& m, const TapSrc<kS>& T, const float* f,
                                         int64_t c, int64_t se, int64_t sf, float inv_h) {
  float cm[8], co;
  T.load(__ldg(m.dcmap + c), cm, co);
  float g = 0.f;
#pragma unroll
  for (int k = 1; k <= 8; ++k) g = fmaf(cm[k - 1], __ldg(f + c + k * se) - __ldg(f + c - (k - 1) * se), g);
  g = fmaf(co, (__ldg(f + c + se + sf) - __ldg(f + c + sf)) + (__ldg(f + c + se - sf) - __ldg(f + c - sf)), g);
  return g * inv_h;
}

// D'_a v at c (the pressure-kernel stencil)
template <bool kS>
__device__ __forceinline__ float div_at(const Maps& m, const TapSrc<kS>& T, const float* v,
                                        int64_t c, int64_t se, int64_t sf, float inv_h) {
  float cm[8], co;
  T.load(__ldg(m.dcmap + c), cm, co);
  float d = 0.f;
#pragma unroll
  for (int k = 1; k <= 8; ++k) d = fmaf(cm[k - 1], __ldg(v + c + (k - 1) * se) - __ldg(v + c - k * se), d);
  d = fmaf(co, (__ldg(v + c + sf) - __ldg(v + c - se + sf)) + (__ldg(v + c - sf) - __ldg(v + c - se - sf)), d);
  return d * inv_h;
}

// (D_a^T u)(q): u is zero outside the body
template <bool kS>
__device__ __forceinline__ float grad_T_at(const Maps& m, const TapSrc<kS>& T, const float* u,
                                           int64_t q, int64_t se, int64_t sf, float inv_h) {
  float acc = 0.f;
#pragma unroll
  for (int k = 1; k <= 8; ++k) {
    const int64_t c1 = q - k * se, c2 = q + (k - 1) * se;
    acc += tap_of(m, T, c1, k - 1) * __ldg(u + c1) - tap_of(m, T, c2, k - 1) * __ldg(u + c2);
  }
#pragma unroll
  for (int s = -1; s <= 1; s += 2) {
    const int64_t c1 = q - se - s * sf, c2 = q - s * sf;
    acc += tap_of(m, T, c1, 8) * __ldg(u + c1) - tap_of(m, T, c2, 8) * __ldg(u + c2);
  }
  return acc * inv_h;
}

// (D'_a^T u)(q)
template <bool kS>
__device__ __forceinline__ float div_T_at(const Maps& m, const TapSrc<kS>& T, const float* u,
                                          int64_t q, int64_t se, int64_t sf, float inv_h) {
  float acc = 0.f;
#pragma unroll
  for (int k = 1; k <= 8; ++k) {
    const int64_t c1 = q - (k - 1) * se, c2 = q + k * se;
    acc += tap_of(m, T, c1, k - 1) * __ldg(u + c1) - tap_of(m, T, c2, k - 1) * __ldg(u + c2);
  }
#pragma unroll
  for (int s = -1; s <= 1; s += 2) {
    const int64_t c1 = q - s * sf, c2 = q + se - s * sf;
    acc += tap_of(m, T, c1, 8) * __ldg(u + c1) - tap_of(m, T, c2, 8) * __ldg(u + c2);
  }
  return acc * inv_h;
}

__device__ __forceinline__ bool adj_cell(const Grid& g, int64_t* c) {
  const int j = kGhost + blockIdx.x * blockDim.x + threadIdx.x;
  const int i = kGhost + blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= g.nx - kGhost || j >= g.ny - kGhost) return false;
  *c = (int64_t)i * g.sx + j;
  return true;
}

// lam_p += sum_a D_a^T lam_g_a
template <bool kS>
__global__ void __launch_bounds__(256) adj2d_assemble(const AdjArgs A) {
  extern __shared__ float s_taps[];
  const TapSrc<kS> T = stage_taps<kS>(A, s_taps);
  int64_t q;
  if (!adj_cell(A.g, &q)) return;
  const float add = grad_T_at(A.m, T, A.lam_g[0], q, A.g.sx, 1, A.g.inv_h[0]) +
                    grad_T_at(A.m, T, A.lam_g[1], q, 1, A.g.sx, A.g.inv_h[1]);
  A.lam_p[q] += add;
}

// record adjoint and projections for step n
static __global__ void adj2d_io(const AdjArgs A, const Lists L, const float* residual, int n,
                         int n_src, int n_zero, int n_rec) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int stride = gridDim.x * blockDim.x;
  if (n % L.mod_t == 0) {
    const float* row = residual + (size_t)(n / L.mod_t) * L.ncoordsout;
    for (int e = t; e < n_rec; e += stride) atomicAdd(A.lam_p + L.rec_cell[e], row[L.rec_k[e]]);
  }
}

static __global__ void adj2d_zero(const AdjArgs A, const Lists L, int n, int n_src, int n_zero) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int stride = gridDim.x * blockDim.x;
  for (int e = t; e < n_zero; e += stride) A.lam_p[L.zero_cell[e]] = 0.f;
  if (n < L.nt_ic)
    for (int e = t; e < n_src; e += stride) A.lam_p[L.src_cell[e]] = 0.f;
}

// Gradient accumulation: kF64 = every step's contributions formed and added in FP64 (GB300's FP64
// pipe is the bottleneck then); otherwise contributions are formed in FP32 (the precision of the
// adjoint fields themselves) and summed per checkpoint segment in FP32 partials, which
// adj2d_merge adds into the FP64 time sums at the end of every segment.
// Pressure adjoint of body cell c (ND axes), given its assembled lam_p and the divergence
// components d[a] = D'_a v^{n+1/2} at c. kBeta (nonlinear engine): the forward update is
// p' = p - (dt K + 2 dt beta p) div, so the coefficient of div is that sum at p = p^n, lam_p
// passes to p^n times (1 - 2 dt beta div), and 2 dt beta gets the gradient -p^n div lam_p.
template <bool kF64, int ND, bool kBeta = false>
__device__ __forceinline__ void adj_prs_point(const AdjArgs& A, int64_t c, const float lp,
                                              const float (&d)[ND]) {
  using acc_t = typename std::conditional<kF64, double, float>::type;
  const int64_t fs = A.fs;
  const float dtk = __ldg(A.m.dt_k + c), ikx = __ldg(A.m.inv_kx[0] + c);
  const float b2dt = kBeta ? __ldg(A.m.beta2dt + c) : 0.f;
  const float pn = kBeta ? __ldg(S_p(A.Sn, fs) + c) : 0.f;
  const float k = kBeta ? fmaf(b2dt, pn, dtk) : dtk;   // the forward's coefficient of div
  const float ax[2] = {__ldg(A.m.ax[0][0] + c), __ldg(A.m.ax[0][1] + c)};
  const float bx[2] = {__ldg(A.m.bx[0][0] + c), __ldg(A.m.bx[0][1] + c)};
  acc_t g_dtk = 0, g_ikx = 0, g_ax[2] = {0, 0}, g_bx[2] = {0, 0};
  float div = 0.f;
#pragma unroll
  for (int a = 0; a < ND; ++a) {
    const float n1 = __ldg(S_phiN<ND>(A.Sn1, fs, a, 0) + c), n2 = __ldg(S_phiN<ND>(A.Sn1, fs, a, 1) + c);
    div += fmaf(d[a], ikx, n1) + n2;
    float lam_d = -k * ikx * lp;
#pragma unroll
    for (int nu = 0; nu < 2; ++nu) {
      const float L = A.lam_phi[a][nu][c] - k * lp;
      lam_d = fmaf(ax[nu], L, lam_d);
      g_ax[nu] += (acc_t)L * d[a];
      g_bx[nu] += (acc_t)L * __ldg(S_phiN<ND>(A.Sn, fs, a, nu) + c);
      A.lam_phi[a][nu][c] = bx[nu] * L;
    }
    g_ikx -= (acc_t)k * lp * d[a];
    A.lam_d[a][c] = lam_d;
  }
  g_dtk -= (acc_t)div * lp;
  if constexpr (kBeta) {
    A.lam_p[c] = lp - b2dt * div * lp;
    if constexpr (kF64) A.grad[A.beta_slot][c] -= (double)pn * div * lp;
    else A.g32[A.beta_slot][c] -= pn * div * lp;
  }
  if constexpr (kF64) {
    A.grad[kGDtK][c] += g_dtk;
    A.grad[kGInvKx][c] += g_ikx;
    A.grad[kGAx1][c] += g_ax[0];
    A.grad[kGAx2][c] += g_ax[1];
    A.grad[kGBx1][c] += g_bx[0];
    A.grad[kGBx2][c] += g_bx[1];
  } else {
    A.g32[kGDtK][c] += g_dtk;
    A.g32[kGInvKx][c] += g_ikx;
    A.g32[kGAx1][c] += g_ax[0];
    A.g32[kGAx2][c] += g_ax[1];
    A.g32[kGBx1][c] += g_bx[0];
    A.g32[kGBx2][c] += g_bx[1];
  }
}

// Pressure adjoint of 2D body cell c, given its assembled lam_p.
template <bool kF64, bool kS, bool kBeta = false>
__device__ __forceinline__ void adj_prs_cell(const AdjArgs& A, const TapSrc<kS>& T, int64_t c,
                                             const float lp) {
  const Grid& g = A.g;
  const float d[2] = {div_at(A.m, T, S_v(A.Sn1, A.fs, 0), c, g.sx, 1, g.inv_h[0]),
                      div_at(A.m, T, S_v(A.Sn1, A.fs, 1), c, 1, g.sx, g.inv_h[1])};
  adj_prs_point<kF64, 2, kBeta>(A, c, lp, d);
}

template <bool kF64, bool kS, bool kBeta = false>
__global__ void __launch_bounds__(256) adj2d_prs(const AdjArgs A) {
  extern __shared__ float s_taps[];
  const TapSrc<kS> T = stage_taps<kS>(A, s_taps);
  int64_t c;
  if (!adj_cell(A.g, &c)) return;
  adj_prs_cell<kF64, kS, kBeta>(A, T, c, A.lam_p[c]);
}

// Velocity adjoint of body cell c (ND axes), given (D'_a^T lam_d_a)(c) and the pressure
// gradient components gr[a] = D_a p^n at c.
template <bool kF64, int ND>
__device__ __forceinline__ void adj_vel_point(const AdjArgs& A, int64_t c, const float (&dT)[ND],
                                              const float (&gr)[ND]) {
  using acc_t = typename std::conditional<kF64, double, float>::type;
  const int64_t fs = A.fs;
  const float r = __ldg(A.m.rdt_rho + c), iku = __ldg(A.m.inv_ku[0] + c);
  const float au[2] = {__ldg(A.m.au[0][0] + c), __ldg(A.m.au[0][1] + c)};
  const float bu[2] = {__ldg(A.m.bu[0][0] + c), __ldg(A.m.bu[0][1] + c)};
  acc_t g_r = 0, g_iku = 0, g_au[2] = {0, 0}, g_bu[2] = {0, 0};
#pragma unroll
  for (int a = 0; a < ND; ++a) {
    const float lv = A.lam_v[a][c] + dT[a];
    const float p1 = __ldg(S_psiN<ND>(A.Sn1, fs, a, 0) + c), p2 = __ldg(S_psiN<ND>(A.Sn1, fs, a, 1) + c);
    float lam_g = -r * iku * lv;
#pragma unroll
    for (int nu = 0; nu < 2; ++nu) {
      const float M = A.lam_psi[a][nu][c] - r * lv;
      lam_g = fmaf(au[nu], M, lam_g);
      g_au[nu] += (acc_t)M * gr[a];
      g_bu[nu] += (acc_t)M * __ldg(S_psiN<ND>(A.Sn, fs, a, nu) + c);
      A.lam_psi[a][nu][c] = bu[nu] * M;
    }
    g_r -= (acc_t)lv * (fmaf(gr[a], iku, p1) + p2);
    g_iku -= (acc_t)r * gr[a] * lv;
    A.lam_v[a][c] = lv;
    A.lam_g[a][c] = lam_g;
  }
  if constexpr (kF64) {
    A.grad[kGRdtRho][c] += g_r;
    A.grad[kGInvKu][c] += g_iku;
    A.grad[kGAu1][c] += g_au[0];
    A.grad[kGAu2][c] += g_au[1];
    A.grad[kGBu1][c] += g_bu[0];
    A.grad[kGBu2][c] += g_bu[1];
  } else {
    A.g32[kGRdtRho][c] += g_r;
    A.g32[kGInvKu][c] += g_iku;
    A.g32[kGAu1][c] += g_au[0];
    A.g32[kGAu2][c] += g_au[1];
    A.g32[kGBu1][c] += g_bu[0];
    A.g32[kGBu2][c] += g_bu[1];
  }
}

// Velocity adjoint of 2D body cell c, given (D'_a^T lam_d_a)(c) for both axes.
template <bool kF64, bool kS>
__device__ __forceinline__ void adj_vel_cell(const AdjArgs& A, const TapSrc<kS>& T, int64_t c,
                                             const float (&dT)[2]) {
  const Grid& g = A.g;
  const float gr[2] = {grad_at(A.m, T, S_p(A.Sn, A.fs), c, g.sx, 1, g.inv_h[0]),
                       grad_at(A.m, T, S_p(A.Sn, A.fs), c, 1, g.sx, g.inv_h[1])};
  adj_vel_point<kF64, 2>(A, c, dT, gr);
}

template <bool kF64, bool kS>
__global__ void __launch_bounds__(256) adj2d_vel(const AdjArgs A) {
  extern __shared__ float s_taps[];
  const TapSrc<kS> T = stage_taps<kS>(A, s_taps);
  int64_t c;
  if (!adj_cell(A.g, &c)) return;
  const Grid& g = A.g;
  const float dT[2] = {div_T_at(A.m, T, A.lam_d[0], c, g.sx, 1, g.inv_h[0]),
                       div_T_at(A.m, T, A.lam_d[1], c, 1, g.sx, g.inv_h[1])};
  adj_vel_cell<kF64, kS>(A, T, c, dT);
}

// ---- tiled reverse step: the transposed stencils read shared-memory tiles ----------------------
// Block = one 32 (y) x 8 (x) tile of body cells (the list tiles), origin (i0, j0). Fields are
// staged with the halo the transposed stencils need (zero / tap index 0 outside the array: the
// adjoint fields are zero there, so those terms vanish).
template <int R, int C, class Tv, class Ts>
__device__ __forceinline__ void stage_tile(Tv (&dst)[R][C], const Ts* src, const Grid& g,
                                           int row0, int col0, int tid) {
  for (int e = tid; e < R * C; e += kD2TY * kD2TX) {
    const int r = e / C, cc = e % C;
    const int gr = row0 + r, gc = col0 + cc;
    dst[r][cc] = (gr >= 0 && gr < g.nx && gc >= 0 && gc < (int)g.sx) ? src[(int64_t)gr * g.sx + gc]
                                                                      : Tv(0);
  }
}

// Assemble + record adjoint + projections + pressure adjoint in one launch: lam_p of the tile's
// cells is assembled from the staged lam_g tiles (same operation order as adj2d_assemble), the
// tile's sensor residuals are added and its air / source cells zeroed in shared memory (same
// order as adj2d_io, adj2d_zero), then the pressure adjoint runs on it. Ghost-cell list entries
// (sensors or sources placed in the ghost layer) are skipped: their lam_p is never read.
template <bool kF64, bool kS>
__global__ void __launch_bounds__(256) adj2d_prs_fused(const AdjArgs A, const Lists L,
                                                       const float* residual, int n) {
  extern __shared__ float s_taps[];
  __shared__ float GX[23][34], GY[10][47], LP[kD2TX][kD2TY];
  __shared__ int DC[23][47];
  const TapSrc<kS> T = stage_taps<kS>(A, s_taps);
  const Grid& g = A.g;
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * kD2TY + tx;
  const int i0 = kGhost + blockIdx.y * kD2TX, j0 = kGhost + blockIdx.x * kD2TY;
  stage_tile(GX, A.lam_g[0], g, i0 - 8, j0 - 1, tid);
  stage_tile(GY, A.lam_g[1], g, i0 - 1, j0 - 8, tid);
  stage_tile(DC, A.m.dcmap, g, i0 - 8, j0 - 8, tid);
  __syncthreads();
  const int i = i0 + ty, j = j0 + tx;
  const bool active = i < g.nx - kGhost && j < g.ny - kGhost;
  const int64_t c = (int64_t)i * g.sx + j;
  if (active) {
    // (D_x^T lam_g_x)(c): se = one row, sf = one column (grad_T_at)
    float ax = 0.f;
#pragma unroll
    for (int k = 1; k <= 8; ++k) {
      const int r1 = ty - k + 8, r2 = ty + k - 1 + 8, cu = tx + 1, cd = tx + 8;
      ax += T.tap(DC[r1][cd], k - 1) * GX[r1][cu] - T.tap(DC[r2][cd], k - 1) * GX[r2][cu];
    }
#pragma unroll
    for (int s = -1; s <= 1; s += 2) {
      ax += T.tap(DC[ty + 7][tx + 8 - s], 8) * GX[ty + 7][tx + 1 - s] -
            T.tap(DC[ty + 8][tx + 8 - s], 8) * GX[ty + 8][tx + 1 - s];
    }
    ax *= g.inv_h[0];
    // (D_y^T lam_g_y)(c): se = one column, sf = one row
    float ay = 0.f;
#pragma unroll
    for (int k = 1; k <= 8; ++k) {
      ay += T.tap(DC[ty + 8][tx + 8 - k], k - 1) * GY[ty + 1][tx + 8 - k] -
            T.tap(DC[ty + 8][tx + 7 + k], k - 1) * GY[ty + 1][tx + 7 + k];
    }
#pragma unroll
    for (int s = -1; s <= 1; s += 2) {
      ay += T.tap(DC[ty + 8 - s][tx + 7], 8) * GY[ty + 1 - s][tx + 7] -
            T.tap(DC[ty + 8 - s][tx + 8], 8) * GY[ty + 1 - s][tx + 8];
    }
    ay *= g.inv_h[1];
    const float add = ax + ay;
    LP[ty][tx] = A.lam_p[c] + add;
  }
  __syncthreads();
  const int tile = blockIdx.y * gridDim.x + blockIdx.x;
  auto local = [&](int64_t cell, int* li, int* lj) {
    const int ci = (int)(cell / g.sx), cj = (int)(cell % g.sx);
    *li = ci - i0;
    *lj = cj - j0;
    return ci >= kGhost && ci < g.nx - kGhost && cj >= kGhost && cj < g.ny - kGhost &&
           *li >= 0 && *li < kD2TX && *lj >= 0 && *lj < kD2TY;
  };
  if (n % L.mod_t == 0) {
    const float* row = residual + (size_t)(n / L.mod_t) * L.ncoordsout;
    for (int e = L.rec_ptr[tile] + tid; e < L.rec_ptr[tile + 1]; e += kD2TY * kD2TX) {
      int li, lj;
      if (local(L.rec_cell[e], &li, &lj)) atomicAdd(&LP[li][lj], row[L.rec_k[e]]);
    }
  }
  __syncthreads();
  for (int e = L.zero_ptr[tile] + tid; e < L.zero_ptr[tile + 1]; e += kD2TY * kD2TX) {
    int li, lj;
    if (local(L.zero_cell[e], &li, &lj)) LP[li][lj] = 0.f;
  }
  if (n < L.nt_ic) {
    for (int e = L.src_ptr[tile] + tid; e < L.src_ptr[tile + 1]; e += kD2TY * kD2TX) {
      int li, lj;
      if (local(L.src_cell[e], &li, &lj)) LP[li][lj] = 0.f;
    }
  }
  __syncthreads();
  if (!active) return;
  const float lp = LP[ty][tx];
  A.lam_p[c] = lp;
  adj_prs_cell<kF64, kS>(A, T, c, lp);
}

// Velocity adjoint with the transposed divergence read from staged lam_d tiles (div_T_at order).
template <bool kF64, bool kS>
__global__ void __launch_bounds__(256) adj2d_vel_tiled(const AdjArgs A) {
  extern __shared__ float s_taps[];
  __shared__ float DX[23][34], DY[10][47];
  __shared__ int DC[23][47];
  const TapSrc<kS> T = stage_taps<kS>(A, s_taps);
  const Grid& g = A.g;
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * kD2TY + tx;
  const int i0 = kGhost + blockIdx.y * kD2TX, j0 = kGhost + blockIdx.x * kD2TY;
  stage_tile(DX, A.lam_d[0], g, i0 - 7, j0 - 1, tid);
  stage_tile(DY, A.lam_d[1], g, i0 - 1, j0 - 7, tid);
  stage_tile(DC, A.m.dcmap, g, i0 - 7, j0 - 7, tid);
  __syncthreads();
  const int i = i0 + ty, j = j0 + tx;
  if (i >= g.nx - kGhost || j >= g.ny - kGhost) return;
  const int64_t c = (int64_t)i * g.sx + j;
  // (D'_x^T lam_d_x)(c): se = one row, sf = one column
  float dx = 0.f;
#pragma unroll
  for (int k = 1; k <= 8; ++k) {
    const int r1 = ty - k + 8, r2 = ty + k + 7;
    dx += T.tap(DC[r1][tx + 7], k - 1) * DX[r1][tx + 1] - T.tap(DC[r2][tx + 7], k - 1) * DX[r2][tx + 1];
  }
#pragma unroll
  for (int s = -1; s <= 1; s += 2) {
    dx += T.tap(DC[ty + 7][tx + 7 - s], 8) * DX[ty + 7][tx + 1 - s] -
          T.tap(DC[ty + 8][tx + 7 - s], 8) * DX[ty + 8][tx + 1 - s];
  }
  dx *= g.inv_h[0];
  // (D'_y^T lam_d_y)(c): se = one column, sf = one row
  float dy = 0.f;
#pragma unroll
  for (int k = 1; k <= 8; ++k) {
    dy += T.tap(DC[ty + 7][tx + 8 - k], k - 1) * DY[ty + 1][tx + 8 - k] -
          T.tap(DC[ty + 7][tx + 7 + k], k - 1) * DY[ty + 1][tx + 7 + k];
  }
#pragma unroll
  for (int s = -1; s <= 1; s += 2) {
    dy += T.tap(DC[ty + 7 - s][tx + 7], 8) * DY[ty + 1 - s][tx + 7] -
          T.tap(DC[ty + 7 - s][tx + 8], 8) * DY[ty + 1 - s][tx + 8];
  }
  dy *= g.inv_h[1];
  const float dT[2] = {dx, dy};
  adj_vel_cell<kF64, kS>(A, T, c, dT);
}

// End of a segment: FP64 time sums += FP32 segment partials; partials reset (body cells).
static __global__ void __launch_bounds__(256) adj2d_merge(const AdjArgs A) {
  int64_t c;
  if (!adj_cell(A.g, &c)) return;
  for (int q = 0; q < A.n_grad; ++q) {
    A.grad[q][c] += (double)A.g32[q][c];
    A.g32[q][c] = 0.f;
  }
}

static __global__ void set_step_counter(int* step, int value) { *step = value; }

// ---- TMA-staged reverse step ------------------------------------------------------------------
// Every operand of a block's 32 (y) x 8 (x) tile is brought into shared memory at block start by
// one thread: TMA boxes over the adjoint-field stack, the coefficient-map stack, the two stored
// states and the tap-index map, and a bulk copy of the tap table, all completing on one mbarrier
// (bounded wait). A block thus has its whole input (about 36 KB) in flight at once instead of a
// few dependent loads per thread, which is what limits the tiled kernels above (long-scoreboard
// stalls at full occupancy, a fifth of the DRAM bandwidth). The arithmetic is that of
// adj2d_prs_fused / adj2d_vel_tiled, term for term in the same order.
//
// The adjoint-field allocation holds, per padded cell array: lam_p, lam_v (2), lam_psi (4),
// lam_phi (4), lam_d (2), lam_g (2), then the FP32 gradient partials in coefficient-map order
// (velocity maps rdt_rho inv_ku au1 bu1 au2 bu2, pressure maps dt_k inv_kx ax1 bx1 ax2 bx2), so
// that each kernel's point-wise operands are runs of consecutive fields.
constexpr int kAdjFields = 15;                 // adjoint fields before the gradient partials
constexpr int kAdjStack = kAdjFields + kNumGrad;
constexpr int kAdjLamP = 0, kAdjLamV = 1, kAdjLamPsi = 3, kAdjLamPhi = 7, kAdjLamD = 11,
              kAdjLamG = 13;
constexpr int kAdjMapVel = 0, kAdjMapPrs = 6;  // first coefficient map of each kernel's run of 6
constexpr int kStPsi = 3, kStPhi = 7;          // first psi / phi field of a stored 2D state

struct AdjMaps {
  CUtensorMap lam1, lam4, lam6;     // adjoint stack (pitch, nx, kAdjStack): boxes {32, 8, f}
  CUtensorMap halo_x, halo_y;       // adjoint stack: boxes {40, 24, 1} and {48, 10, 1}
  CUtensorMap maps6;                // coefficient-map stack: box {32, 8, 6}
  CUtensorMap st4, st_vx, st_vy, st_p;  // stored states (pitch, nx, 11, slots): {32, 8, 4, 1},
                                        // {40, 24, 1, 1}, {48, 10, 1, 1}, {48, 24, 1, 1}
  CUtensorMap dc;                   // tap-index map (pitch, nx): box {48, 24}
};

// Halo tiles: x-halo boxes start at (i0 - 8, j0 - 4) (40 wide, 24 rows), y-halo boxes at
// (i0 - 1, j0 - 8) (48 wide, 10 rows), full boxes at (i0 - 8, j0 - 8) (48 x 24). Box starts
// along y are multiples of 4 floats (16 bytes): j0 = 8 + 32 blockIdx.x.
constexpr int kHXW = 40, kHXR = 24, kHYW = 48, kHYR = 10, kHFW = 48, kHFR = 24;
constexpr int kPrsPW = 21, kVelPW = 22;    // point-wise planes of each kernel

struct AdjPrsSmem {
  float gx[kHXR][kHXW];                 // lam_g_x
  float gy[kHYR][kHYW];                 // lam_g_y
  float vx[kHXR][kHXW];                 // v_x of S_{n+1}
  float vy[kHYR][kHYW];                 // v_y of S_{n+1}
  uint16_t dc[kHFR][kHFW];
  // point-wise: 0 lam_p | 1-4 lam_phi | 5-10 dt_k inv_kx ax1 bx1 ax2 bx2 | 11-14 phi of S_n |
  // 15-20 gradient partials of the pressure maps (phi of S_{n+1} is recomputed, not staged)
  float pw[kPrsPW][kD2TX][kD2TY];
  float lp[kD2TX][kD2TY];
  uint64_t bar;
};
struct AdjVelSmem {
  float dx[kHXR][kHXW];                 // lam_d_x
  float dy[kHYR][kHYW];                 // lam_d_y
  float p[kHFR][kHFW];                  // p of S_n
  uint16_t dc[kHFR][kHFW];
  // point-wise: 0-1 lam_v | 2-5 lam_psi | 6-11 rdt_rho inv_ku au1 bu1 au2 bu2 | 12-15 psi of
  // S_n | 16-21 gradient partials of the velocity maps (psi of S_{n+1} is recomputed)
  float pw[kVelPW][kD2TX][kD2TY];
  uint64_t bar;
};
constexpr uint32_t kPrsTx = sizeof(float) * (2 * kHXR * kHXW + 2 * kHYR * kHYW +
                                             kPrsPW * kD2TX * kD2TY) +
                            sizeof(uint16_t) * kHFR * kHFW;
constexpr uint32_t kVelTx = sizeof(float) * (kHXR * kHXW + kHYR * kHYW + kHFR * kHFW +
                                             kVelPW * kD2TX * kD2TY) +
                            sizeof(uint16_t) * kHFR * kHFW;
__host__ __device__ constexpr size_t adj_tap_offset(size_t smem_struct) {
  return (smem_struct + 127) / 128 * 128;
}
static_assert(offsetof(AdjPrsSmem, gy) % 128 == 0 && offsetof(AdjPrsSmem, vx) % 128 == 0 &&
                  offsetof(AdjPrsSmem, vy) % 128 == 0 && offsetof(AdjPrsSmem, dc) % 128 == 0 &&
                  offsetof(AdjPrsSmem, pw) % 128 == 0,
              "TMA destinations must be 128-byte aligned");
static_assert(offsetof(AdjVelSmem, dy) % 128 == 0 && offsetof(AdjVelSmem, p) % 128 == 0 &&
                  offsetof(AdjVelSmem, dc) % 128 == 0 && offsetof(AdjVelSmem, pw) % 128 == 0,
              "TMA destinations must be 128-byte aligned");

// Shared-memory bytes of the TMA reverse-step kernels for a tap table of ndmap sets.
inline size_t adj_prs_tma_smem(int ndmap) {
  return adj_tap_offset(sizeof(AdjPrsSmem)) + (size_t)ndmap * kTapStride * sizeof(float);
}
inline size_t adj_vel_tma_smem(int ndmap) {
  return adj_tap_offset(sizeof(AdjVelSmem)) + (size_t)ndmap * kTapStride * sizeof(float);
}

// Block prologue: alignment guard, barrier init, one thread issues the loads. Returns false when
// the block must stop (misaligned shared memory: reported, nothing issued).
template <class SmemT>
__device__ __forceinline__ bool adj_tma_begin(SmemT& S, const unsigned char* base, int* status,
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

// Reverse step, launch 1 (adj2d_prs_fused with TMA-staged operands). `slot` = store slot of S_n.
template <int kUnused = 0>
__global__ void __launch_bounds__(256, 5) adj2d_prs_tma(const AdjArgs A, const Lists L,
                                                        const float* residual, int n, int slot,
                                                        const __grid_constant__ AdjMaps M) {
  extern __shared__ __align__(128) unsigned char adj_smem[];
  AdjPrsSmem& S = *reinterpret_cast<AdjPrsSmem*>(adj_smem);
  float* taps = reinterpret_cast<float*>(adj_smem + adj_tap_offset(sizeof(AdjPrsSmem)));
  const Grid& g = A.g;
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * kD2TY + tx;
  const int i0 = kGhost + blockIdx.y * kD2TX, j0 = kGhost + blockIdx.x * kD2TY;
  const uint32_t tap_bytes = (uint32_t)A.ndmap * kTapStride * sizeof(float);
  if (!adj_tma_begin(S, adj_smem, A.status, tid, kPrsTx + tap_bytes)) return;
  if (tid == 0) {
    tma_load_3d(S.gx, &M.halo_x, &S.bar, j0 - 4, i0 - 8, kAdjLamG);
    tma_load_3d(S.gy, &M.halo_y, &S.bar, j0 - 8, i0 - 1, kAdjLamG + 1);
    tma_load_4d(S.vx, &M.st_vx, &S.bar, j0 - 4, i0 - 8, 1, slot + 1);
    tma_load_4d(S.vy, &M.st_vy, &S.bar, j0 - 8, i0 - 1, 2, slot + 1);
    tma_load_2d(S.dc, &M.dc, &S.bar, j0 - 8, i0 - 8);
    tma_load_3d(S.pw[0], &M.lam1, &S.bar, j0, i0, kAdjLamP);
    tma_load_3d(S.pw[1], &M.lam4, &S.bar, j0, i0, kAdjLamPhi);
    tma_load_3d(S.pw[5], &M.maps6, &S.bar, j0, i0, kAdjMapPrs);
    tma_load_4d(S.pw[11], &M.st4, &S.bar, j0, i0, kStPhi, slot);
    tma_load_3d(S.pw[15], &M.lam6, &S.bar, j0, i0, kAdjFields + kAdjMapPrs);
    bulk_load(taps, A.m.taps, tap_bytes, &S.bar);
  }
  __syncthreads();   // barrier initialised before anyone polls it
  mbar_wait_bounded(&S.bar, 0, A.status);
  const TapSrc<true> T{taps};
  const int i = i0 + ty, j = j0 + tx;
  const bool active = i < g.nx - kGhost && j < g.ny - kGhost;
  const int64_t c = (int64_t)i * g.sx + j;
  if (active) {
    // (D_x^T lam_g_x)(c)
    float ax = 0.f;
#pragma unroll
    for (int k = 1; k <= 8; ++k) {
      const int r1 = ty - k + 8, r2 = ty + k - 1 + 8, cu = tx + 4, cd = tx + 8;
      ax += T.tap(S.dc[r1][cd], k - 1) * S.gx[r1][cu] - T.tap(S.dc[r2][cd], k - 1) * S.gx[r2][cu];
    }
#pragma unroll
    for (int s = -1; s <= 1; s += 2) {
      ax += T.tap(S.dc[ty + 7][tx + 8 - s], 8) * S.gx[ty + 7][tx + 4 - s] -
            T.tap(S.dc[ty + 8][tx + 8 - s], 8) * S.gx[ty + 8][tx + 4 - s];
    }
    ax *= g.inv_h[0];
    // (D_y^T lam_g_y)(c)
    float ay = 0.f;
#pragma unroll
    for (int k = 1; k <= 8; ++k) {
      ay += T.tap(S.dc[ty + 8][tx + 8 - k], k - 1) * S.gy[ty + 1][tx + 8 - k] -
            T.tap(S.dc[ty + 8][tx + 7 + k], k - 1) * S.gy[ty + 1][tx + 7 + k];
    }
#pragma unroll
    for (int s = -1; s <= 1; s += 2) {
      ay += T.tap(S.dc[ty + 8 - s][tx + 7], 8) * S.gy[ty + 1 - s][tx + 7] -
            T.tap(S.dc[ty + 8 - s][tx + 8], 8) * S.gy[ty + 1 - s][tx + 8];
    }
    ay *= g.inv_h[1];
    const float add = ax + ay;
    S.lp[ty][tx] = S.pw[0][ty][tx] + add;
  }
  __syncthreads();
  const int tile = blockIdx.y * gridDim.x + blockIdx.x;
  auto local = [&](int64_t cell, int* li, int* lj) {
    const int ci = (int)(cell / g.sx), cj = (int)(cell % g.sx);
    *li = ci - i0;
    *lj = cj - j0;
    return ci >= kGhost && ci < g.nx - kGhost && cj >= kGhost && cj < g.ny - kGhost &&
           *li >= 0 && *li < kD2TX && *lj >= 0 && *lj < kD2TY;
  };
  if (n % L.mod_t == 0) {
    const float* row = residual + (size_t)(n / L.mod_t) * L.ncoordsout;
    for (int e = L.rec_ptr[tile] + tid; e < L.rec_ptr[tile + 1]; e += kD2TY * kD2TX) {
      int li, lj;
      if (local(L.rec_cell[e], &li, &lj)) atomicAdd(&S.lp[li][lj], row[L.rec_k[e]]);
    }
  }
  __syncthreads();
  for (int e = L.zero_ptr[tile] + tid; e < L.zero_ptr[tile + 1]; e += kD2TY * kD2TX) {
    int li, lj;
    if (local(L.zero_cell[e], &li, &lj)) S.lp[li][lj] = 0.f;
  }
  if (n < L.nt_ic) {
    for (int e = L.src_ptr[tile] + tid; e < L.src_ptr[tile + 1]; e += kD2TY * kD2TX) {
      int li, lj;
      if (local(L.src_cell[e], &li, &lj)) S.lp[li][lj] = 0.f;
    }
  }
  __syncthreads();
  if (!active) return;
  const float lp = S.lp[ty][tx];
  A.lam_p[c] = lp;
  // pressure adjoint (adj_prs_cell, FP32 contributions)
  auto P = [&](int q) { return S.pw[q][ty][tx]; };
  const float k = P(5), ikx = P(6);
  const float axm[2] = {P(7), P(9)};
  const float bxm[2] = {P(8), P(10)};
  float g_dtk = 0, g_ikx = 0, g_ax[2] = {0, 0}, g_bx[2] = {0, 0};
  float div = 0.f;
  float cm[8], co;
  T.load(S.dc[ty + 8][tx + 8], cm, co);
#pragma unroll
  for (int a = 0; a < 2; ++a) {
    // D'_a v^{n+1/2} at c (div_at order)
    float d = 0.f;
    if (a == 0) {
#pragma unroll
      for (int kk = 1; kk <= 8; ++kk)
        d = fmaf(cm[kk - 1], S.vx[ty + 8 + kk - 1][tx + 4] - S.vx[ty + 8 - kk][tx + 4], d);
      d = fmaf(co, (S.vx[ty + 8][tx + 5] - S.vx[ty + 7][tx + 5]) +
                       (S.vx[ty + 8][tx + 3] - S.vx[ty + 7][tx + 3]), d);
    } else {
#pragma unroll
      for (int kk = 1; kk <= 8; ++kk)
        d = fmaf(cm[kk - 1], S.vy[ty + 1][tx + 8 + kk - 1] - S.vy[ty + 1][tx + 8 - kk], d);
      d = fmaf(co, (S.vy[ty + 2][tx + 8] - S.vy[ty + 2][tx + 7]) +
                       (S.vy[ty][tx + 8] - S.vy[ty][tx + 7]), d);
    }
    d = d * g.inv_h[a];
    // phi of S_{n+1}: the forward update of the memory variables (CellPrsT), bit for bit
    const float n1 = fmaf(bxm[0], P(11 + 2 * a), axm[0] * d);
    const float n2 = fmaf(bxm[1], P(12 + 2 * a), axm[1] * d);
    div += fmaf(d, ikx, n1) + n2;
    float lam_d = -k * ikx * lp;
#pragma unroll
    for (int nu = 0; nu < 2; ++nu) {
      const float Lv = P(1 + 2 * a + nu) - k * lp;
      lam_d = fmaf(axm[nu], Lv, lam_d);
      g_ax[nu] += Lv * d;
      g_bx[nu] += Lv * P(11 + 2 * a + nu);
      A.lam_phi[a][nu][c] = bxm[nu] * Lv;
    }
    g_ikx -= k * lp * d;
    A.lam_d[a][c] = lam_d;
  }
  g_dtk -= div * lp;
  A.g32[kGDtK][c] = P(15) + g_dtk;
  A.g32[kGInvKx][c] = P(16) + g_ikx;
  A.g32[kGAx1][c] = P(17) + g_ax[0];
  A.g32[kGBx1][c] = P(18) + g_bx[0];
  A.g32[kGAx2][c] = P(19) + g_ax[1];
  A.g32[kGBx2][c] = P(20) + g_bx[1];
}

// Reverse step, launch 2 (adj2d_vel_tiled with TMA-staged operands).
template <int kUnused = 0>
__global__ void __launch_bounds__(256, 5) adj2d_vel_tma(const AdjArgs A, int slot,
                                                        const __grid_constant__ AdjMaps M) {
  extern __shared__ __align__(128) unsigned char adj_smem[];
  AdjVelSmem& S = *reinterpret_cast<AdjVelSmem*>(adj_smem);
  float* taps = reinterpret_cast<float*>(adj_smem + adj_tap_offset(sizeof(AdjVelSmem)));
  const Grid& g = A.g;
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * kD2TY + tx;
  const int i0 = kGhost + blockIdx.y * kD2TX, j0 = kGhost + blockIdx.x * kD2TY;
  const uint32_t tap_bytes = (uint32_t)A.ndmap * kTapStride * sizeof(float);
  if (!adj_tma_begin(S, adj_smem, A.status, tid, kVelTx + tap_bytes)) return;
  if (tid == 0) {
    tma_load_3d(S.dx, &M.halo_x, &S.bar, j0 - 4, i0 - 8, kAdjLamD);
    tma_load_3d(S.dy, &M.halo_y, &S.bar, j0 - 8, i0 - 1, kAdjLamD + 1);
    tma_load_4d(S.p, &M.st_p, &S.bar, j0 - 8, i0 - 8, 0, slot);
    tma_load_2d(S.dc, &M.dc, &S.bar, j0 - 8, i0 - 8);
    tma_load_3d(S.pw[0], &M.lam6, &S.bar, j0, i0, kAdjLamV);
    tma_load_3d(S.pw[6], &M.maps6, &S.bar, j0, i0, kAdjMapVel);
    tma_load_4d(S.pw[12], &M.st4, &S.bar, j0, i0, kStPsi, slot);
    tma_load_3d(S.pw[16], &M.lam6, &S.bar, j0, i0, kAdjFields + kAdjMapVel);
    bulk_load(taps, A.m.taps, tap_bytes, &S.bar);
  }
  __syncthreads();
  mbar_wait_bounded(&S.bar, 0, A.status);
  const int i = i0 + ty, j = j0 + tx;
  if (i >= g.nx - kGhost || j >= g.ny - kGhost) return;
  const int64_t c = (int64_t)i * g.sx + j;
  const TapSrc<true> T{taps};
  // (D'_x^T lam_d_x)(c)
  float dx = 0.f;
#pragma unroll
  for (int k = 1; k <= 8; ++k) {
    const int r1 = ty - k + 9, r2 = ty + k + 8;
    dx += T.tap(S.dc[r1][tx + 8], k - 1) * S.dx[r1][tx + 4] -
          T.tap(S.dc[r2][tx + 8], k - 1) * S.dx[r2][tx + 4];
  }
#pragma unroll
  for (int s = -1; s <= 1; s += 2) {
    dx += T.tap(S.dc[ty + 8][tx + 8 - s], 8) * S.dx[ty + 8][tx + 4 - s] -
          T.tap(S.dc[ty + 9][tx + 8 - s], 8) * S.dx[ty + 9][tx + 4 - s];
  }
  dx *= g.inv_h[0];
  // (D'_y^T lam_d_y)(c)
  float dy = 0.f;
#pragma unroll
  for (int k = 1; k <= 8; ++k) {
    dy += T.tap(S.dc[ty + 8][tx + 9 - k], k - 1) * S.dy[ty + 1][tx + 9 - k] -
          T.tap(S.dc[ty + 8][tx + 8 + k], k - 1) * S.dy[ty + 1][tx + 8 + k];
  }
#pragma unroll
  for (int s = -1; s <= 1; s += 2) {
    dy += T.tap(S.dc[ty + 8 - s][tx + 8], 8) * S.dy[ty + 1 - s][tx + 8] -
          T.tap(S.dc[ty + 8 - s][tx + 9], 8) * S.dy[ty + 1 - s][tx + 9];
  }
  dy *= g.inv_h[1];
  const float dT[2] = {dx, dy};
  // velocity adjoint (adj_vel_cell, FP32 contributions)
  auto P = [&](int q) { return S.pw[q][ty][tx]; };
  const float r = P(6), iku = P(7);
  const float aum[2] = {P(8), P(10)};
  const float bum[2] = {P(9), P(11)};
  float g_r = 0, g_iku = 0, g_au[2] = {0, 0}, g_bu[2] = {0, 0};
  float cm[8], co;
  T.load(S.dc[ty + 8][tx + 8], cm, co);
#pragma unroll
  for (int a = 0; a < 2; ++a) {
    const float lv = P(a) + dT[a];
    // D_a p^n at c (grad_at order)
    float gr = 0.f;
    if (a == 0) {
#pragma unroll
      for (int kk = 1; kk <= 8; ++kk)
        gr = fmaf(cm[kk - 1], S.p[ty + 8 + kk][tx + 8] - S.p[ty + 9 - kk][tx + 8], gr);
      gr = fmaf(co, (S.p[ty + 9][tx + 9] - S.p[ty + 8][tx + 9]) +
                        (S.p[ty + 9][tx + 7] - S.p[ty + 8][tx + 7]), gr);
    } else {
#pragma unroll
      for (int kk = 1; kk <= 8; ++kk)
        gr = fmaf(cm[kk - 1], S.p[ty + 8][tx + 8 + kk] - S.p[ty + 8][tx + 9 - kk], gr);
      gr = fmaf(co, (S.p[ty + 9][tx + 9] - S.p[ty + 9][tx + 8]) +
                        (S.p[ty + 7][tx + 9] - S.p[ty + 7][tx + 8]), gr);
    }
    gr = gr * g.inv_h[a];
    // psi of S_{n+1}: the forward update of the memory variables (CellVelT), bit for bit
    const float p1 = fmaf(bum[0], P(12 + 2 * a), aum[0] * gr);
    const float p2 = fmaf(bum[1], P(13 + 2 * a), aum[1] * gr);
    float lam_g = -r * iku * lv;
#pragma unroll
    for (int nu = 0; nu < 2; ++nu) {
      const float Mv = P(2 + 2 * a + nu) - r * lv;
      lam_g = fmaf(aum[nu], Mv, lam_g);
      g_au[nu] += Mv * gr;
      g_bu[nu] += Mv * P(12 + 2 * a + nu);
      A.lam_psi[a][nu][c] = bum[nu] * Mv;
    }
    g_r -= lv * (fmaf(gr, iku, p1) + p2);
    g_iku -= r * gr * lv;
    A.lam_v[a][c] = lv;
    A.lam_g[a][c] = lam_g;
  }
  A.g32[kGRdtRho][c] = P(16) + g_r;
  A.g32[kGInvKu][c] = P(17) + g_iku;
  A.g32[kGAu1][c] = P(18) + g_au[0];
  A.g32[kGBu1][c] = P(19) + g_bu[0];
  A.g32[kGAu2][c] = P(20) + g_au[1];
  A.g32[kGBu2][c] = P(21) + g_bu[1];
}

}  // namespace fwgb
