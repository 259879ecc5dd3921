// Shared definitions of the FDTD engine: device-side parameter blocks and small helpers.
//
// Memory layout in HBM (one handle = one simulation):
//   every field and map is a separate float32 array in C order (the tap-set index map dcmap:
//   uint16, at most 65535 tap sets) with the last axis padded to a multiple of 32 elements, so
//   that every float row of the contiguous axis starts on a 128-byte boundary (a uint16 row on a
//   64-byte one); padding and the 8-cell ghost layer hold zeros and are
//   never updated. Cell (i, j[, k]) lives at ((i * ny + j) * pitch + k) in 3D and
//   (i * pitch + j) in 2D.
//   state  (read + written every step): p, v[ndim], psi[ndim][2] (pressure-gradient memory
//          variables), phi[ndim][2] (velocity-divergence memory variables)
//   maps   (read every step):  dt/rho, dt*K, 1/kappau, 1/kappax, a/b for u1 u2 x1 x2, dcmap,
//          and 2*dt*beta only when beta is not identically zero
//   taps   [ndmap][12] float32: axial taps c1..c8, off-axis tap, 3 zeros
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace fwgb {

constexpr int kGhost = 8;          // taps per side = ghost cells per side
constexpr int kTapStride = 12;     // floats per tap set

struct Lists {
  // Per-tile compressed lists (tile = the block of kernel B that owns the cell).
  const int32_t* src_ptr;   // [n_tiles + 1]
  const int64_t* src_cell;  // padded linear index
  const int32_t* src_k;     // source index (row of icmat)
  const int32_t* zero_ptr;
  const int64_t* zero_cell;
  const int32_t* rec_ptr;
  const int64_t* rec_cell;
  const int32_t* rec_k;     // sensor index (column of the traces)
  const float* icmat_t;     // [nt_ic][ncoords]
  float* traces;            // [n_out][ncoordsout], or [n_out][n_groups] with sensor groups
  const int32_t* rec_group; // per record entry: output column (sensor groups), or nullptr
  const float* rec_w;       // per record entry: weight of the sample in its group
  int32_t ncoords, ncoordsout, nt_ic, mod_t;
};

struct Grid {
  int32_t nx, ny, nz;        // nz = 1 in 2D
  int64_t sx, sy;            // strides (elements) of axis x and y; the last axis has stride 1
  float inv_h[3];            // 1/dx, 1/dy, 1/dz
};

struct Fields {
  float* p;
  float* v[3];
  float* psi[3][2];
  float* phi[3][2];
};

struct Maps {
  const float* rdt_rho;      // dt / rho
  const float* dt_k;         // dt * K
  const float* beta2dt;      // 2 dt beta, or nullptr when beta == 0 everywhere
  // relaxation coefficients per derivative axis; the isotropic engine points every axis at the
  // same arrays (u maps for the pressure gradient, x maps for the velocity divergence)
  const float* inv_ku[3];    // 1 / kappa{u,w,v}
  const float* inv_kx[3];    // 1 / kappa{x,y,z}
  const float* au[3][2];
  const float* bu[3][2];
  const float* ax[3][2];
  const float* bx[3][2];
  const float* a_exp;        // exponential-attenuation engine: amplitude kept per field update
  const uint16_t* dcmap;     // tap-set index per cell (16-bit: at most 65535 tap sets)
  const float* taps;         // [ndmap][12]
};

struct StepArgs {
  Grid g;
  Fields f;
  Maps m;
  Lists l;
  int* step;                 // device step counter: velocity kernel of step n sets it to n+1
};

// Programmatic dependent launch: every time-step kernel is launched allowed to start while the
// previous kernel of the stream drains. It first waits for that kernel (and so, transitively,
// every earlier one) to complete and its writes to be visible, then lets the next kernel launch:
// the launch latency and the next kernel's block scheduling overlap this kernel's last wave.
// Without the launch attribute both instructions are no-ops.
__device__ __forceinline__ void pdl_entry() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Derived coefficient maps, formed once from the caller's maps (the same float32 operations for
// every entry point that prepares them): dt/rho, dt*K, 2*dt*beta and 1/kappa, with a zero map
// entry (ghost cells of a map the caller left at zero) kept at zero.
__device__ __forceinline__ float derive_rdt_rho(float dt, float rho) { return rho != 0.f ? dt / rho : 0.f; }
__device__ __forceinline__ float derive_dt_k(float dt, float k) { return dt * k; }
__device__ __forceinline__ float derive_beta2dt(float dt, float beta) { return 2.f * dt * beta; }
__device__ __forceinline__ float derive_inverse(float kappa) { return kappa != 0.f ? 1.f / kappa : 0.f; }

__device__ __forceinline__ void load_taps(const float* taps, int dc, float (&c)[8], float& co) {
  const float4* t = reinterpret_cast<const float4*>(taps + (size_t)dc * kTapStride);
  float4 a = __ldg(t), b = __ldg(t + 1), e = __ldg(t + 2);
  c[0] = a.x; c[1] = a.y; c[2] = a.z; c[3] = a.w;
  c[4] = b.x; c[5] = b.y; c[6] = b.z; c[7] = b.w;
  co = e.x;
}

// Point-wise operands of one cell for the velocity update, loaded together (all loads issued
// before any use) and written back together. NDIM velocity components; kAniso: one set of
// relaxation coefficients per axis (NA = NDIM sets), else one set shared by every axis.
template <int NDIM, bool kAniso = false>
struct CellVelT {
  static constexpr int NA = kAniso ? NDIM : 1;
  int dc;
  float rr, iku[NA], a1[NA], b1[NA], a2[NA], b2[NA];
  float v[NDIM], s1[NDIM], s2[NDIM];
  __device__ __forceinline__ void load(const StepArgs& A, int64_t c) {
    dc = __ldg(A.m.dcmap + c);
    rr = __ldg(A.m.rdt_rho + c);
#pragma unroll
    for (int a = 0; a < NA; ++a) {
      iku[a] = __ldg(A.m.inv_ku[a] + c);
      a1[a] = __ldg(A.m.au[a][0] + c);
      b1[a] = __ldg(A.m.bu[a][0] + c);
      a2[a] = __ldg(A.m.au[a][1] + c);
      b2[a] = __ldg(A.m.bu[a][1] + c);
    }
#pragma unroll
    for (int a = 0; a < NDIM; ++a) {
      v[a] = A.f.v[a][c];
      s1[a] = A.f.psi[a][0][c];
      s2[a] = A.f.psi[a][1][c];
    }
  }
  // psi_nu <- b_nu psi_nu + a_nu g ;  v <- v - dt/rho (g / kappau + psi_1 + psi_2)
  __device__ __forceinline__ void update_store(const StepArgs& A, int64_t c, const float* g) {
#pragma unroll
    for (int a = 0; a < NDIM; ++a) {
      const int q = kAniso ? a : 0;
      const float n1 = fmaf(b1[q], s1[a], a1[q] * g[a]);
      const float n2 = fmaf(b2[q], s2[a], a2[q] * g[a]);
      A.f.psi[a][0][c] = n1;
      A.f.psi[a][1][c] = n2;
      A.f.v[a][c] = fmaf(-rr, fmaf(g[a], iku[q], n1) + n2, v[a]);
    }
  }
};

template <int NDIM, bool kBeta, bool kAniso = false>
struct CellPrsT {
  static constexpr int NA = kAniso ? NDIM : 1;
  int dc;
  float dtk, b2dt, pc, ikx[NA], a1[NA], b1[NA], a2[NA], b2[NA];
  float f1[NDIM], f2[NDIM];
  __device__ __forceinline__ void load(const StepArgs& A, int64_t c) {
    dc = __ldg(A.m.dcmap + c);
    dtk = __ldg(A.m.dt_k + c);
    b2dt = kBeta ? __ldg(A.m.beta2dt + c) : 0.f;
#pragma unroll
    for (int a = 0; a < NA; ++a) {
      ikx[a] = __ldg(A.m.inv_kx[a] + c);
      a1[a] = __ldg(A.m.ax[a][0] + c);
      b1[a] = __ldg(A.m.bx[a][0] + c);
      a2[a] = __ldg(A.m.ax[a][1] + c);
      b2[a] = __ldg(A.m.bx[a][1] + c);
    }
    pc = A.f.p[c];
#pragma unroll
    for (int a = 0; a < NDIM; ++a) {
      f1[a] = A.f.phi[a][0][c];
      f2[a] = A.f.phi[a][1][c];
    }
  }
  // phi_nu <- b_nu phi_nu + a_nu d ;  p <- p - dt (K + 2 beta p) sum (d / kappax + phi_1 + phi_2)
  __device__ __forceinline__ void update_store(const StepArgs& A, int64_t c, const float* d) {
    float div = 0.f;
#pragma unroll
    for (int a = 0; a < NDIM; ++a) {
      const int q = kAniso ? a : 0;
      const float n1 = fmaf(b1[q], f1[a], a1[q] * d[a]);
      const float n2 = fmaf(b2[q], f2[a], a2[q] * d[a]);
      A.f.phi[a][0][c] = n1;
      A.f.phi[a][1][c] = n2;
      div += fmaf(d[a], ikx[q], n1) + n2;
    }
    const float coef = kBeta ? fmaf(b2dt, pc, dtk) : dtk;
    A.f.p[c] = fmaf(-coef, div, pc);
  }
};

// Exponential-attenuation engine (no memory variables, kappa = 1):
//   v <- a_exp (v - dt/rho g);   p <- a_exp (p - dt (K + 2 beta p) sum_a d_a)
template <int NDIM>
struct CellVelExpT {
  int dc;
  float rr, ae, v[NDIM];
  __device__ __forceinline__ void load(const StepArgs& A, int64_t c) {
    dc = __ldg(A.m.dcmap + c);
    rr = __ldg(A.m.rdt_rho + c);
    ae = __ldg(A.m.a_exp + c);
#pragma unroll
    for (int a = 0; a < NDIM; ++a) v[a] = A.f.v[a][c];
  }
  __device__ __forceinline__ void update_store(const StepArgs& A, int64_t c, const float* g) {
#pragma unroll
    for (int a = 0; a < NDIM; ++a) A.f.v[a][c] = ae * fmaf(-rr, g[a], v[a]);
  }
};

template <int NDIM, bool kBeta>
struct CellPrsExpT {
  int dc;
  float dtk, b2dt, ae, pc;
  __device__ __forceinline__ void load(const StepArgs& A, int64_t c) {
    dc = __ldg(A.m.dcmap + c);
    dtk = __ldg(A.m.dt_k + c);
    b2dt = kBeta ? __ldg(A.m.beta2dt + c) : 0.f;
    ae = __ldg(A.m.a_exp + c);
    pc = A.f.p[c];
  }
  __device__ __forceinline__ void update_store(const StepArgs& A, int64_t c, const float* d) {
    float div = 0.f;
#pragma unroll
    for (int a = 0; a < NDIM; ++a) div += d[a];
    const float coef = kBeta ? fmaf(b2dt, pc, dtk) : dtk;
    A.f.p[c] = ae * fmaf(-coef, div, pc);
  }
};

// Source injection, air zeroing and sensor recording for the cells owned by a block. The per-tile
// lists are indexed tile = tx * n_ty + ty; a block owns the tiles [tx0, tx1) x [ty0, ty1), whose
// entries are contiguous per tx. Called by every thread of the pressure kernel after its pressure
// writes; `tid`/`nthr` span the block. Order per cell: source, air, record.
// `n` is the time step being completed (-1: take it from the device step counter).
__device__ __forceinline__ void span_epilogue(const StepArgs& A, float* p, int tx0, int tx1,
                                              int ty0, int ty1, int n_ty, int tid, int nthr,
                                              int n = -1) {
  const Lists& L = A.l;
  if (n < 0) n = *A.step - 1;
  __syncthreads();
  if (n < L.nt_ic) {
    const float* col = L.icmat_t + (size_t)n * L.ncoords;
    for (int tx = tx0; tx < tx1; ++tx)
      for (int e = L.src_ptr[tx * n_ty + ty0] + tid; e < L.src_ptr[tx * n_ty + ty1]; e += nthr)
        p[L.src_cell[e]] = col[L.src_k[e]];
  }
  __syncthreads();
  for (int tx = tx0; tx < tx1; ++tx)
    for (int e = L.zero_ptr[tx * n_ty + ty0] + tid; e < L.zero_ptr[tx * n_ty + ty1]; e += nthr)
      p[L.zero_cell[e]] = 0.f;
  __syncthreads();
  if (n % L.mod_t == 0) {
    float* row = L.traces + (size_t)(n / L.mod_t) * L.ncoordsout;
    for (int tx = tx0; tx < tx1; ++tx) {
      const int b = L.rec_ptr[tx * n_ty + ty0], end = L.rec_ptr[tx * n_ty + ty1];
      if (L.rec_group) {  // weighted sums per sensor group (e.g. transducer elements)
        for (int e = b + tid; e < end; e += nthr)
          if (L.rec_group[e] >= 0) atomicAdd(row + L.rec_group[e], L.rec_w[e] * p[L.rec_cell[e]]);
      } else {
        for (int e = b + tid; e < end; e += nthr) row[L.rec_k[e]] = p[L.rec_cell[e]];
      }
    }
  }
}

// The epilogue of one tile (the direct kernels: one block per tile).
__device__ __forceinline__ void tile_epilogue(const StepArgs& A, float* p, int tile, int tid,
                                              int nthr, int n = -1) {
  span_epilogue(A, p, tile, tile + 1, 0, 1, 1, tid, nthr, n);
}

}  // namespace fwgb
