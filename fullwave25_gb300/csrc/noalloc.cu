// fw_run_noalloc: a 2D forward solve that allocates no memory at all.
//
// Who needs it: callers that cannot call cudaMalloc once they are running, for example a host
// application whose device memory is handed out only by its own pool, a process that must not
// grow its device footprint after start-up, or a caller that only holds device buffers given to
// it by someone else. They pass device pointers to the inputs and to the output; this entry point
// keeps everything else (the wavefield, the memory variables, the derived coefficient maps, the
// tap table and its bookkeeping) in one file-scope device array instead of allocating it.
//
// The array `g_noalloc_scratch` is FWGB_NOALLOC_SCRATCH_BYTES (48 MiB) in every GPU context that
// loads this library, held until the process exits. 2D only. One call uses, 256-byte aligned:
//   a status block (256 B) | 11 state fields | 5 derived maps (dt/rho, dt*K, 1/kappau, 1/kappax,
//   2*dt*beta) | 16-bit tap indices | tap table [ndmap][12] | empty per-tile lists | one byte per
//   source (does this entry drive its cell: the last entry listed for a cell does)
// i.e. 66 bytes per grid cell plus 48 bytes per tap set, about 760,000 cells at most.
//
// The time step runs the engine's own 2D cell update and stencil (vel2d_body / prs2d_body with
// CellVelT / CellPrsT), so its traces equal fw_create + fw_set_fields + fw_run bit for bit.
// Before any time step, one kernel checks every source, sensor and air coordinate and every
// tap index against the grid; the call reads that verdict back (a stream synchronisation) and
// returns FW_ERR_ARGUMENT without stepping if anything lies outside, so no kernel ever touches
// a bad index.
//
// Every call shares the array and leaves its last contents there; each call clears the parts
// that must start at zero. Calls that overlap on the GPU (different streams, or different host
// threads on one device) race on the array: serialise them.
#include <cuda_runtime.h>

#include <climits>
#include <cstdarg>
#include <cstdio>
#include <cstring>

#include "../../include/fwgb.h"
#include "kernels_direct.cuh"

void fwgb_set_global_error(const char* msg);  // engine.cu: text returned by fw_last_error(NULL)

namespace {

using fwgb::kGhost;
using fwgb::kTapStride;

constexpr size_t kScratchBytes = FWGB_NOALLOC_SCRATCH_BYTES;
constexpr int kFields2D = 11;  // p, vx, vy, psi[2][2], phi[2][2]
constexpr int kDerived = 5;    // dt/rho, dt*K, 1/kappau, 1/kappax, 2*dt*beta

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// Status block at the start of the array (int32 words).
enum : int {
  kStBits = 0,      // bit 0: icc, 1: outc, 2: icczero, 3: dcmap out of range
  kStBeta = 1,      // 1 when some cell has beta != 0
  kStFirstIcc = 2,  // smallest offending entry per array (INT_MAX: none)
  kStFirstOutc = 3,
  kStFirstZero = 4,
  kStFirstDc = 5,
  kStStep = 6,      // step counter word of the argument block (the kernels are given n)
  kStWords = 8
};

int fail(int code, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
int fail(int code, const char* fmt, ...) {
  char body[400], buf[512];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(body, sizeof body, fmt, ap);
  va_end(ap);
  std::snprintf(buf, sizeof buf, "fw_run_noalloc: %s", body);
  fwgb_set_global_error(buf);
  return code;
}

size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

// Byte offsets of one call's regions inside the array.
struct Layout {
  size_t state, derived, dc16, taps, tiles, keep, end;
  Layout(size_t cells, int ndmap, int ntiles, int ncoords) {
    state = 256;
    derived = align256(state + cells * kFields2D * sizeof(float));
    dc16 = align256(derived + cells * kDerived * sizeof(float));
    taps = align256(dc16 + cells * sizeof(uint16_t));
    tiles = align256(taps + (size_t)ndmap * kTapStride * sizeof(float));
    keep = align256(tiles + (size_t)(ntiles + 1) * sizeof(int32_t));
    end = keep + (size_t)ncoords;
  }
};

__global__ void na_init_status(int* st) {
  if (threadIdx.x < kStWords) st[threadIdx.x] = (threadIdx.x >= kStFirstIcc && threadIdx.x <= kStFirstDc) ? INT_MAX : 0;
}

__device__ __forceinline__ bool in_grid(const int32_t* c, int k, int nx, int ny) {
  const int x = c[2 * k], y = c[2 * k + 1];
  return x >= 0 && x < nx && y >= 0 && y < ny;
}

// Checks every coordinate and tap index (reads only the caller's arrays) and notes whether beta
// is nonzero anywhere.
__global__ void na_validate(int* st, int nx, int ny, int ndmap, const int32_t* icc, int ncoords,
                            const int32_t* outc, int nout, const int32_t* zero, int nzero,
                            const int32_t* dcmap, const float* beta, int64_t cells) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t n_all = max(max(cells, (int64_t)ncoords), (int64_t)max(nout, nzero));
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_all; i += stride) {
    if (i < cells) {
      const int dc = dcmap[i];
      if (dc < 0 || dc >= ndmap) {
        atomicOr(st + kStBits, 8);
        atomicMin(st + kStFirstDc, (int)i);
      }
      if (beta[i] != 0.f) st[kStBeta] = 1;
    }
    if (i < ncoords && !in_grid(icc, (int)i, nx, ny)) {
      atomicOr(st + kStBits, 1);
      atomicMin(st + kStFirstIcc, (int)i);
    }
    if (i < nout && !in_grid(outc, (int)i, nx, ny)) {
      atomicOr(st + kStBits, 2);
      atomicMin(st + kStFirstOutc, (int)i);
    }
    if (i < nzero && !in_grid(zero, (int)i, nx, ny)) {
      atomicOr(st + kStBits, 4);
      atomicMin(st + kStFirstZero, (int)i);
    }
  }
}

// The last source entry listed for a cell drives it (as the engine's source lists): `owner`
// (cells int32, preset to -1) takes the largest entry index per cell, then each entry learns
// whether it is that one. Coordinates were validated before.
__global__ void na_owner(int* owner, int ny, const int32_t* icc, int ncoords) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < ncoords; k += gridDim.x * blockDim.x)
    atomicMax(owner + (int64_t)icc[2 * k] * ny + icc[2 * k + 1], k);
}

__global__ void na_keep(const int* owner, unsigned char* keep, int ny, const int32_t* icc,
                        int ncoords) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < ncoords; k += gridDim.x * blockDim.x)
    keep[k] = owner[(int64_t)icc[2 * k] * ny + icc[2 * k + 1]] == k;
}

// Derived maps and 16-bit tap indices (tap indices validated before).
__global__ void na_prep_maps(float* rdt, float* dtk, float* iku, float* ikx, float* b2dt,
                             uint16_t* dc16, const float* rho, const float* K, const float* kappau,
                             const float* kappax, const float* beta, const int32_t* dcmap,
                             int64_t cells, float dt) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < cells;
       c += (int64_t)gridDim.x * blockDim.x) {
    rdt[c] = fwgb::derive_rdt_rho(dt, rho[c]);
    dtk[c] = fwgb::derive_dt_k(dt, K[c]);
    iku[c] = fwgb::derive_inverse(kappau[c]);
    ikx[c] = fwgb::derive_inverse(kappax[c]);
    b2dt[c] = fwgb::derive_beta2dt(dt, beta[c]);
    dc16[c] = (uint16_t)dcmap[c];
  }
}

// dmap [9][2][ndmap] -> taps [ndmap][12]: axial taps c1..c8, the off-axis tap, three zeros.
__global__ void na_prep_taps(float* taps, const float* dmap, int ndmap) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < ndmap; e += gridDim.x * blockDim.x) {
    float* t = taps + (size_t)e * kTapStride;
#pragma unroll
    for (int m = 1; m <= 8; ++m) t[m - 1] = dmap[(size_t)(m * 2) * ndmap + e];
    t[8] = dmap[(size_t)3 * ndmap + e];
    t[9] = t[10] = t[11] = 0.f;
  }
}

__global__ void __launch_bounds__(256) na_vel2d(const fwgb::StepArgs A) {
  fwgb::vel2d_body<fwgb::CellVelT<2, false>>(A, blockIdx.x, blockIdx.y);
}

// The per-tile lists of A are empty: the tile epilogue does nothing; na_io below applies the
// sources, air cells and sensors of step n after every tile has been updated.
template <bool kBeta>
__global__ void __launch_bounds__(256) na_prs2d(const fwgb::StepArgs A, int n) {
  fwgb::prs2d_body<fwgb::CellPrsT<2, kBeta, false>>(A, blockIdx.x, blockIdx.y,
                                                    blockIdx.y * gridDim.x + blockIdx.x, n);
}

// Sources (only the entry that drives its cell), then air cells, then sensors, for step n: one
// block, the three phases ordered by block barriers.
__global__ void __launch_bounds__(1024) na_io(float* p, int ny, int n, const int32_t* icc,
                                             const unsigned char* keep, int ncoords,
                                             const float* icmat, int nt_ic,
                                             const int32_t* icczero, int nzero,
                                             const int32_t* outc, int nout, int mod_t,
                                             float* traces) {
  if (n < nt_ic)
    for (int k = threadIdx.x; k < ncoords; k += blockDim.x)
      if (keep[k]) p[(int64_t)icc[2 * k] * ny + icc[2 * k + 1]] = icmat[(size_t)k * nt_ic + n];
  __syncthreads();
  for (int k = threadIdx.x; k < nzero; k += blockDim.x)
    p[(int64_t)icczero[2 * k] * ny + icczero[2 * k + 1]] = 0.f;
  __syncthreads();
  if (n % mod_t == 0) {
    float* row = traces + (size_t)(n / mod_t) * nout;
    for (int k = threadIdx.x; k < nout; k += blockDim.x)
      row[k] = p[(int64_t)outc[2 * k] * ny + outc[2 * k + 1]];
  }
}

#define NA_CUDA(call)                                                         \
  do {                                                                        \
    cudaError_t e_ = (call);                                                  \
    if (e_ != cudaSuccess) return fail(FW_ERR_CUDA, "%s", cudaGetErrorString(e_)); \
  } while (0)

}  // namespace

extern "C" FWGB_API int fw_run_noalloc(const fw_desc* d, const fw_fields* f, void* stream,
                                       float* traces) {
  if (!d || !f || !traces) return fail(FW_ERR_ARGUMENT, "desc, fields and traces must not be NULL");
  if (d->ndim != 2) return fail(FW_ERR_UNSUPPORTED, "only 2D grids are supported");
  if (d->isotropic != 1 || d->n_relax != 2)
    return fail(FW_ERR_UNSUPPORTED, "only the isotropic two-mechanism engine is supported");
  if (!f->on_device) return fail(FW_ERR_ARGUMENT, "fields must be device pointers (on_device = 1)");
  if (d->nx <= 2 * kGhost || d->ny <= 2 * kGhost || d->nt < 0 || d->mod_t < 1 || d->ndmap < 1 ||
      d->ndmap > 65535 || d->ncoords < 0 || d->ncoordsout < 0 || d->ncoordszero < 0 ||
      d->nt_ic < 0 || !(d->dt > 0.f) || !(d->dx > 0.f) || !(d->dy > 0.f))
    return fail(FW_ERR_ARGUMENT, "invalid grid size, spacing, step count, tap-set count or coordinate count");
  const size_t cells = (size_t)d->nx * d->ny;
  const int body_x = d->nx - 2 * kGhost, body_y = d->ny - 2 * kGhost;
  const dim3 grid((body_y + fwgb::kD2TY - 1) / fwgb::kD2TY, (body_x + fwgb::kD2TX - 1) / fwgb::kD2TX),
      block(fwgb::kD2TY, fwgb::kD2TX);
  const int ntiles = (int)(grid.x * grid.y);
  const Layout lay(cells, d->ndmap, ntiles, d->ncoords);
  if (lay.end > kScratchBytes)
    return fail(FW_ERR_ARGUMENT,
                "grid %d x %d (%d tap sets, %d sources) needs %zu bytes of scratch; the maximum is "
                "%zu bytes (about %zu cells at 66 bytes per cell)", d->nx, d->ny, d->ndmap,
                d->ncoords, lay.end, kScratchBytes, (kScratchBytes - 4096) / 66);
  const float* req[] = {f->dmap, f->rho, f->K, f->beta, f->kappax, f->kappau, f->apmlu1,
                        f->bpmlu1, f->apmlu2, f->bpmlu2, f->apmlx1, f->bpmlx1, f->apmlx2, f->bpmlx2};
  for (const float* q : req)
    if (!q) return fail(FW_ERR_ARGUMENT, "a required map pointer is NULL");
  if (!f->dcmap || (d->ncoords && (!f->icc || (d->nt_ic && !f->icmat))) ||
      (d->ncoordsout && !f->outc) || (d->ncoordszero && !f->icczero))
    return fail(FW_ERR_ARGUMENT, "a required index or signal pointer is NULL");

  // The array's device address in the current device's context, looked up on every call (a
  // cached address would dangle after the context is torn down and recreated).
  void* sym = nullptr;
  NA_CUDA(cudaGetSymbolAddress(&sym, g_noalloc_scratch));
  unsigned char* base = static_cast<unsigned char*>(sym);
  int* st = reinterpret_cast<int*>(base);
  cudaStream_t s = static_cast<cudaStream_t>(stream);

  // -- validate every index before anything reads or writes through one ------------------------
  na_init_status<<<1, 32, 0, s>>>(st);
  na_validate<<<1024, 256, 0, s>>>(st, d->nx, d->ny, d->ndmap, f->icc, d->ncoords, f->outc,
                                   d->ncoordsout, f->icczero, d->ncoordszero, f->dcmap, f->beta,
                                   (int64_t)cells);
  NA_CUDA(cudaGetLastError());
  int hs[kStWords];
  NA_CUDA(cudaMemcpyAsync(hs, st, sizeof hs, cudaMemcpyDeviceToHost, s));
  NA_CUDA(cudaStreamSynchronize(s));
  if (hs[kStBits] & 1) return fail(FW_ERR_ARGUMENT, "icc[%d] lies outside the 2-D grid", hs[kStFirstIcc]);
  if (hs[kStBits] & 2) return fail(FW_ERR_ARGUMENT, "outc[%d] lies outside the 2-D grid", hs[kStFirstOutc]);
  if (hs[kStBits] & 4)
    return fail(FW_ERR_ARGUMENT, "icczero[%d] lies outside the 2-D grid", hs[kStFirstZero]);
  if (hs[kStBits] & 8) {
    int32_t v = 0;
    NA_CUDA(cudaMemcpy(&v, f->dcmap + hs[kStFirstDc], sizeof v, cudaMemcpyDeviceToHost));
    return fail(FW_ERR_ARGUMENT, "dcmap[%d] = %d outside [0, %d)", hs[kStFirstDc], v, d->ndmap);
  }
  const bool has_beta = hs[kStBeta] != 0;

  // -- the driving entry of every source cell, then the state cleared ----------------------------
  float* state = reinterpret_cast<float*>(base + lay.state);
  unsigned char* keep = base + lay.keep;
  if (d->ncoords) {
    int* owner = reinterpret_cast<int*>(state);  // scratch use of the state region before it is cleared
    NA_CUDA(cudaMemsetAsync(owner, 0xFF, cells * sizeof(int), s));
    na_owner<<<64, 256, 0, s>>>(owner, d->ny, f->icc, d->ncoords);
    na_keep<<<64, 256, 0, s>>>(owner, keep, d->ny, f->icc, d->ncoords);
  }
  NA_CUDA(cudaMemsetAsync(state, 0, cells * kFields2D * sizeof(float), s));
  NA_CUDA(cudaMemsetAsync(base + lay.tiles, 0, (size_t)(ntiles + 1) * sizeof(int32_t), s));

  // -- derived maps, tap indices and tap table ---------------------------------------------------
  float* der = reinterpret_cast<float*>(base + lay.derived);
  float* rdt = der;
  float* dtk = der + cells;
  float* iku = der + 2 * cells;
  float* ikx = der + 3 * cells;
  float* b2dt = der + 4 * cells;
  uint16_t* dc16 = reinterpret_cast<uint16_t*>(base + lay.dc16);
  float* taps = reinterpret_cast<float*>(base + lay.taps);
  na_prep_maps<<<1024, 256, 0, s>>>(rdt, dtk, iku, ikx, b2dt, dc16, f->rho, f->K, f->kappau,
                                    f->kappax, f->beta, f->dcmap, (int64_t)cells, d->dt);
  na_prep_taps<<<(d->ndmap + 255) / 256, 256, 0, s>>>(taps, f->dmap, d->ndmap);
  NA_CUDA(cudaGetLastError());

  // -- the engine's argument block over the scratch regions ---------------------------------------
  fwgb::StepArgs A{};
  A.g.nx = d->nx;
  A.g.ny = d->ny;
  A.g.nz = 1;
  A.g.sx = d->ny;
  A.g.sy = 1;
  A.g.inv_h[0] = 1.f / d->dx;
  A.g.inv_h[1] = 1.f / d->dy;
  A.g.inv_h[2] = 0.f;
  float* fld[kFields2D];
  for (int q = 0; q < kFields2D; ++q) fld[q] = state + (size_t)q * cells;
  A.f.p = fld[0];
  A.f.v[0] = fld[1];
  A.f.v[1] = fld[2];
  A.f.psi[0][0] = fld[3]; A.f.psi[0][1] = fld[4]; A.f.psi[1][0] = fld[5]; A.f.psi[1][1] = fld[6];
  A.f.phi[0][0] = fld[7]; A.f.phi[0][1] = fld[8]; A.f.phi[1][0] = fld[9]; A.f.phi[1][1] = fld[10];
  A.m.rdt_rho = rdt;
  A.m.dt_k = dtk;
  A.m.beta2dt = has_beta ? b2dt : nullptr;
  for (int a = 0; a < 3; ++a) {
    A.m.inv_ku[a] = iku;
    A.m.inv_kx[a] = ikx;
    A.m.au[a][0] = f->apmlu1; A.m.au[a][1] = f->apmlu2;
    A.m.bu[a][0] = f->bpmlu1; A.m.bu[a][1] = f->bpmlu2;
    A.m.ax[a][0] = f->apmlx1; A.m.ax[a][1] = f->apmlx2;
    A.m.bx[a][0] = f->bpmlx1; A.m.bx[a][1] = f->bpmlx2;
  }
  A.m.dcmap = dc16;
  A.m.taps = taps;
  const int32_t* empty = reinterpret_cast<const int32_t*>(base + lay.tiles);
  A.l.src_ptr = A.l.zero_ptr = A.l.rec_ptr = empty;
  A.l.traces = traces;
  A.l.mod_t = 1;
  A.step = st + kStStep;

  for (int n = 0; n < d->nt; ++n) {
    na_vel2d<<<grid, block, 0, s>>>(A);
    if (has_beta) na_prs2d<true><<<grid, block, 0, s>>>(A, n);
    else na_prs2d<false><<<grid, block, 0, s>>>(A, n);
    na_io<<<1, 1024, 0, s>>>(A.f.p, d->ny, n, f->icc, keep, d->ncoords, f->icmat, d->nt_ic,
                             f->icczero, d->ncoordszero, f->outc, d->ncoordsout, d->mod_t, traces);
  }
  NA_CUDA(cudaGetLastError());
  return FW_OK;
}
