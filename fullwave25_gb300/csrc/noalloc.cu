// fw_run_noalloc: a 2D forward solve that allocates no memory at all.
//
// Who needs it: callers that cannot call cudaMalloc once they are running, for example a host
// application whose device memory is handed out only by its own pool, a process that must not
// grow its device footprint after start-up, or a caller that only holds device buffers given to
// it by someone else. They pass device pointers to the inputs and to the output; this entry point
// keeps the wavefield (pressure, velocities and memory variables) in one file-scope device array
// instead of allocating it.
//
// The array `g_noalloc_scratch` is FWGB_NOALLOC_SCRATCH_BYTES (32 MiB) in every GPU context that
// loads this library, held until the process exits. 2D only: 11 float32 fields per cell, so grids
// up to 762,600 cells (e.g. the 944 x 688 PML-extended plain 2D workload). Every call shares the
// array and leaves its last contents there; each call zeroes the part it uses before stepping.
// Calls that overlap on the GPU (different streams, or different host threads on one device)
// race on the array: serialise them.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/fwgb.h"

void fwgb_set_global_error(const char* msg);  // engine.cu: text returned by fw_last_error(NULL)

namespace {

constexpr size_t kScratchBytes = FWGB_NOALLOC_SCRATCH_BYTES;
constexpr int kGhost = 8;
constexpr int kFields2D = 11;  // p, vx, vy, psi[2][2], phi[2][2]

static __device__ __align__(256) float g_noalloc_scratch[kScratchBytes / sizeof(float)];

int fail(int code, const char* msg) {
  char buf[512];
  std::snprintf(buf, sizeof buf, "fw_run_noalloc: %s", msg);
  fwgb_set_global_error(buf);
  return code;
}

// Device address of the scratch array, looked up once per device with that device current.
float* scratch_address(int device, cudaError_t* err) {
  static std::mutex mu;
  static float* addr[64] = {};
  static bool done[64] = {};
  if (device < 0 || device >= 64) {
    *err = cudaErrorInvalidDevice;
    return nullptr;
  }
  std::lock_guard<std::mutex> lock(mu);
  if (!done[device]) {
    void* p = nullptr;
    *err = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (*err != cudaSuccess) return nullptr;
    addr[device] = static_cast<float*>(p);
    done[device] = true;
  }
  *err = cudaSuccess;
  return addr[device];
}

struct NaArgs {
  int nx, ny;
  float inv_dx, inv_dy, dt;
  int ndmap, has_beta;
  const float *dmap, *rho, *K, *beta, *kappax, *kappau;
  const float *au1, *bu1, *au2, *bu2, *ax1, *bx1, *ax2, *bx2;
  const int32_t* dcmap;
  float *p, *vx, *vy, *psi[2][2], *phi[2][2];
};

__device__ __forceinline__ void taps_of(const NaArgs& A, int dc, float (&c)[8], float& co) {
#pragma unroll
  for (int m = 1; m <= 8; ++m) c[m - 1] = __ldg(A.dmap + (size_t)(m * 2) * A.ndmap + dc);
  co = __ldg(A.dmap + (size_t)3 * A.ndmap + dc);
}

// Velocity update; the same arithmetic as the engine's 2D velocity kernel, with dt/rho and
// 1/kappau formed from the caller's raw maps (the same float32 operations the engine uses when
// it prepares its derived maps).
__global__ void __launch_bounds__(256) na_vel2d(const NaArgs A) {
  const int j = kGhost + blockIdx.x * 32 + threadIdx.x;
  const int i = kGhost + blockIdx.y * 8 + threadIdx.y;
  if (i >= A.nx - kGhost || j >= A.ny - kGhost) return;
  const int64_t sx = A.ny, c = (int64_t)i * sx + j;
  const float* __restrict__ p = A.p;
  float cm[8], co;
  taps_of(A, __ldg(A.dcmap + c), cm, co);
  float gx = 0.f, gy = 0.f;
#pragma unroll
  for (int m = 1; m <= 8; ++m) {
    gx = fmaf(cm[m - 1], p[c + m * sx] - p[c - (m - 1) * sx], gx);
    gy = fmaf(cm[m - 1], p[c + m] - p[c - (m - 1)], gy);
  }
  gx = fmaf(co, (p[c + sx + 1] - p[c + 1]) + (p[c + sx - 1] - p[c - 1]), gx);
  gy = fmaf(co, (p[c + 1 + sx] - p[c + sx]) + (p[c + 1 - sx] - p[c - sx]), gy);
  gx = gx * A.inv_dx;
  gy = gy * A.inv_dy;
  const float r = __ldg(A.rho + c), ku = __ldg(A.kappau + c);
  const float rr = r != 0.f ? A.dt / r : 0.f;
  const float iku = ku != 0.f ? 1.f / ku : 0.f;
  const float a1 = __ldg(A.au1 + c), b1 = __ldg(A.bu1 + c);
  const float a2 = __ldg(A.au2 + c), b2 = __ldg(A.bu2 + c);
  float s1 = fmaf(b1, A.psi[0][0][c], a1 * gx), s2 = fmaf(b2, A.psi[0][1][c], a2 * gx);
  A.psi[0][0][c] = s1;
  A.psi[0][1][c] = s2;
  A.vx[c] = fmaf(-rr, fmaf(gx, iku, s1) + s2, A.vx[c]);
  s1 = fmaf(b1, A.psi[1][0][c], a1 * gy);
  s2 = fmaf(b2, A.psi[1][1][c], a2 * gy);
  A.psi[1][0][c] = s1;
  A.psi[1][1][c] = s2;
  A.vy[c] = fmaf(-rr, fmaf(gy, iku, s1) + s2, A.vy[c]);
}

__global__ void __launch_bounds__(256) na_prs2d(const NaArgs A) {
  const int j = kGhost + blockIdx.x * 32 + threadIdx.x;
  const int i = kGhost + blockIdx.y * 8 + threadIdx.y;
  if (i >= A.nx - kGhost || j >= A.ny - kGhost) return;
  const int64_t sx = A.ny, c = (int64_t)i * sx + j;
  const float* __restrict__ vx = A.vx;
  const float* __restrict__ vy = A.vy;
  float cm[8], co;
  taps_of(A, __ldg(A.dcmap + c), cm, co);
  float dx = 0.f, dy = 0.f;
#pragma unroll
  for (int m = 1; m <= 8; ++m) {
    dx = fmaf(cm[m - 1], vx[c + (m - 1) * sx] - vx[c - m * sx], dx);
    dy = fmaf(cm[m - 1], vy[c + (m - 1)] - vy[c - m], dy);
  }
  dx = fmaf(co, (vx[c + 1] - vx[c - sx + 1]) + (vx[c - 1] - vx[c - sx - 1]), dx);
  dy = fmaf(co, (vy[c + sx] - vy[c + sx - 1]) + (vy[c - sx] - vy[c - sx - 1]), dy);
  dx *= A.inv_dx;
  dy *= A.inv_dy;
  const float kx = __ldg(A.kappax + c);
  const float ikx = kx != 0.f ? 1.f / kx : 0.f;
  const float a1 = __ldg(A.ax1 + c), b1 = __ldg(A.bx1 + c);
  const float a2 = __ldg(A.ax2 + c), b2 = __ldg(A.bx2 + c);
  const float fx1 = fmaf(b1, A.phi[0][0][c], a1 * dx), fx2 = fmaf(b2, A.phi[0][1][c], a2 * dx);
  const float fy1 = fmaf(b1, A.phi[1][0][c], a1 * dy), fy2 = fmaf(b2, A.phi[1][1][c], a2 * dy);
  A.phi[0][0][c] = fx1;
  A.phi[0][1][c] = fx2;
  A.phi[1][0][c] = fy1;
  A.phi[1][1][c] = fy2;
  const float div = (fmaf(dx, ikx, fx1) + fx2) + (fmaf(dy, ikx, fy1) + fy2);
  const float pc = A.p[c];
  float coef = A.dt * __ldg(A.K + c);
  if (A.has_beta) coef = fmaf(2.f * A.dt * __ldg(A.beta + c), pc, coef);
  A.p[c] = fmaf(-coef, div, pc);
}

// Sources, then air cells, then sensors, for step n: one block so the three phases are ordered
// by block barriers. Source coordinates must be distinct (as map_to_coords produces them).
__global__ void __launch_bounds__(1024) na_io(float* p, int ny, int n, const int32_t* icc,
                                             int ncoords, const float* icmat, int nt_ic,
                                             const int32_t* icczero, int nzero,
                                             const int32_t* outc, int nout, int mod_t,
                                             float* traces) {
  if (n < nt_ic)
    for (int k = threadIdx.x; k < ncoords; k += blockDim.x)
      p[(int64_t)icc[2 * k] * ny + icc[2 * k + 1]] = icmat[(size_t)k * nt_ic + n];
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

}  // namespace

extern "C" FWGB_API int fw_run_noalloc(const fw_desc* d, const fw_fields* f, void* stream,
                                       float* traces) {
  if (!d || !f || !traces) return fail(FW_ERR_ARGUMENT, "desc, fields and traces must not be NULL");
  if (d->ndim != 2) return fail(FW_ERR_UNSUPPORTED, "only 2D grids are supported");
  if (d->isotropic != 1 || d->n_relax != 2)
    return fail(FW_ERR_UNSUPPORTED, "only the isotropic two-mechanism engine is supported");
  if (!f->on_device) return fail(FW_ERR_ARGUMENT, "fields must be device pointers (on_device = 1)");
  if (d->nx <= 2 * kGhost || d->ny <= 2 * kGhost || d->nt < 0 || d->mod_t < 1 || d->ndmap < 1 ||
      d->ncoords < 0 || d->ncoordsout < 0 || d->ncoordszero < 0 || d->nt_ic < 0 || !(d->dt > 0.f))
    return fail(FW_ERR_ARGUMENT, "invalid grid size, step count or coordinate count");
  const size_t cells = (size_t)d->nx * d->ny;
  const size_t need = cells * kFields2D * sizeof(float);
  if (need > kScratchBytes) {
    char msg[256];
    std::snprintf(msg, sizeof msg,
                  "grid %d x %d needs %zu bytes of wavefield scratch; the maximum is %zu bytes "
                  "(%zu cells)", d->nx, d->ny, need, kScratchBytes,
                  kScratchBytes / (kFields2D * sizeof(float)));
    return fail(FW_ERR_ARGUMENT, msg);
  }
  const float* req[] = {f->dmap, f->rho, f->K, f->beta, f->kappax, f->kappau, f->apmlu1,
                        f->bpmlu1, f->apmlu2, f->bpmlu2, f->apmlx1, f->bpmlx1, f->apmlx2, f->bpmlx2};
  for (const float* q : req)
    if (!q) return fail(FW_ERR_ARGUMENT, "a required map pointer is NULL");
  if (!f->dcmap || (d->ncoords && (!f->icc || (d->nt_ic && !f->icmat))) ||
      (d->ncoordsout && !f->outc) || (d->ncoordszero && !f->icczero))
    return fail(FW_ERR_ARGUMENT, "a required index or signal pointer is NULL");
  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess) return fail(FW_ERR_CUDA, "cudaGetDevice failed");
  cudaError_t e = cudaSuccess;
  float* base = scratch_address(device, &e);
  if (!base) return fail(FW_ERR_CUDA, cudaGetErrorString(e));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // the wavefield and memory variables start at zero
  e = cudaMemsetAsync(base, 0, need, s);
  if (e != cudaSuccess) return fail(FW_ERR_CUDA, cudaGetErrorString(e));
  NaArgs A{};
  A.nx = d->nx;
  A.ny = d->ny;
  A.inv_dx = 1.f / d->dx;
  A.inv_dy = 1.f / d->dy;
  A.dt = d->dt;
  A.ndmap = d->ndmap;
  A.has_beta = 1;  // beta is read; a zero map gives the linear update exactly
  A.dmap = f->dmap; A.rho = f->rho; A.K = f->K; A.beta = f->beta;
  A.kappax = f->kappax; A.kappau = f->kappau;
  A.au1 = f->apmlu1; A.bu1 = f->bpmlu1; A.au2 = f->apmlu2; A.bu2 = f->bpmlu2;
  A.ax1 = f->apmlx1; A.bx1 = f->bpmlx1; A.ax2 = f->apmlx2; A.bx2 = f->bpmlx2;
  A.dcmap = f->dcmap;
  float* fld[kFields2D];
  for (int q = 0; q < kFields2D; ++q) fld[q] = base + (size_t)q * cells;
  A.p = fld[0]; A.vx = fld[1]; A.vy = fld[2];
  A.psi[0][0] = fld[3]; A.psi[0][1] = fld[4]; A.psi[1][0] = fld[5]; A.psi[1][1] = fld[6];
  A.phi[0][0] = fld[7]; A.phi[0][1] = fld[8]; A.phi[1][0] = fld[9]; A.phi[1][1] = fld[10];
  const dim3 grid((d->ny - 2 * kGhost + 31) / 32, (d->nx - 2 * kGhost + 7) / 8), block(32, 8);
  for (int n = 0; n < d->nt; ++n) {
    na_vel2d<<<grid, block, 0, s>>>(A);
    na_prs2d<<<grid, block, 0, s>>>(A);
    na_io<<<1, 1024, 0, s>>>(A.p, d->ny, n, f->icc, d->ncoords, f->icmat, d->nt_ic, f->icczero,
                             d->ncoordszero, f->outc, d->ncoordsout, d->mod_t, traces);
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return fail(FW_ERR_CUDA, cudaGetErrorString(e));
  return FW_OK;
}
