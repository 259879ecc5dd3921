// Host side of the FDTD engine: the C ABI declared in include/fwgb.h.
//
// One handle owns the device memory of one simulation: padded state and map arrays, the tap
// table, per-tile source/air/sensor lists and the trace buffer. Time steps are issued as two
// kernels per step (velocity, then pressure + tile epilogue); blocks of steps are captured once
// into a CUDA graph and replayed, so the per-step host cost is one graph launch per block.
// Kernel launches and tensor maps: launch.cu; the group engine: group.cu; the adjoint: adjoint.cu.
#include "engine_host.cuh"

using namespace fwgbh;

namespace {

thread_local std::string g_create_error = "no error";

}  // namespace

// Handle-less error text shared with the other translation units of the library.
void fwgb_set_global_error(const char* msg) { g_create_error = msg; }

namespace fwgbh {

int fail(fw_handle* h, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (h) h->err = buf; else g_create_error = buf;
  return code;
}

const char* last_global_error() { return g_create_error.c_str(); }
void set_global_error(const std::string& msg) { g_create_error = msg; }

int check_device_status(fw_handle* h, cudaStream_t s) {
  int st = 0;
  FW_CUDA(h, cudaMemcpyAsync(&st, h->step + 1, sizeof(int), cudaMemcpyDeviceToHost, s));
  FW_CUDA(h, cudaStreamSynchronize(s));
  if (st) return fail(h, FW_ERR_DEVICE, "a kernel reported device status 0x%x (bounded wait timed out)", st);
  return FW_OK;
}

}  // namespace fwgbh

namespace {

// Tiling of the per-tile source/air/sensor lists, which is also the direct kernels' block tiling
// (and in 3D the plane-march kernels'). 2D march blocks own whole rectangles of these tiles.
Tiling make_tiling(const fw_handle* h) {
  Tiling t{};
  if (h->ndim == 2) {
    t.t[0] = kD2TX; t.t[1] = kD2TY; t.t[2] = 1;
  } else if (h->variant == kMarch) {
    t.t[0] = h->march_xc; t.t[1] = kMTY; t.t[2] = kMTZ;
  } else {
    t.t[0] = kD3TX; t.t[1] = kD3TY; t.t[2] = kD3TZ;
  }
  const int64_t ext[3] = {h->nx, h->ny, h->nz};
  for (int a = 0; a < 3; ++a) {
    if (a == 2 && h->ndim == 2) { t.n[a] = 1; continue; }
    const int64_t body = ext[a] - 2 * kGhost;
    t.n[a] = (int)((body + t.t[a] - 1) / t.t[a]);
  }
  return t;
}

// Tile (block of the pressure kernel) that owns cell (i, j, k). Ghost cells belong to the tile
// of the nearest body cell, so that sources or sensors placed there are still served.
int tile_of(const fw_handle* h, int64_t i, int64_t j, int64_t k) {
  const Tiling& t = h->tiling;
  auto idx = [&](int64_t v, int64_t n, int a) {
    v = std::min(std::max(v, (int64_t)kGhost), n - kGhost - 1) - kGhost;
    return (int)(v / t.t[a]);
  };
  const int tx = idx(i, h->nx, 0), ty = idx(j, h->ny, 1);
  const int tz = h->ndim == 3 ? idx(k, h->nz, 2) : 0;
  return (tx * t.n[1] + ty) * t.n[2] + tz;
}

int64_t padded_index(const fw_handle* h, int64_t i, int64_t j, int64_t k) {
  return h->ndim == 2 ? i * h->pitch + j : (i * h->ny + j) * h->pitch + k;
}

__global__ void transform_maps(float* rho_to_rdt, float* k_to_dtk, float* beta_to_2dt,
                               int64_t n, float dt) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n;
       c += (int64_t)gridDim.x * blockDim.x) {
    rho_to_rdt[c] = fwgb::derive_rdt_rho(dt, rho_to_rdt[c]);
    k_to_dtk[c] = fwgb::derive_dt_k(dt, k_to_dtk[c]);
    beta_to_2dt[c] = fwgb::derive_beta2dt(dt, beta_to_2dt[c]);
  }
}

__global__ void invert_map(float* kappa_to_inv, int64_t n) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n;
       c += (int64_t)gridDim.x * blockDim.x)
    kappa_to_inv[c] = fwgb::derive_inverse(kappa_to_inv[c]);
}

__global__ void transpose_icmat(const float* src, float* dst, int ncoords, int nt_ic) {
  // src [ncoords][nt_ic] -> dst [nt_ic][ncoords]
  __shared__ float tile[32][33];
  const int n0 = blockIdx.x * 32, k0 = blockIdx.y * 32;
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int k = k0 + r, n = n0 + threadIdx.x;
    if (k < ncoords && n < nt_ic) tile[r][threadIdx.x] = src[(size_t)k * nt_ic + n];
  }
  __syncthreads();
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int n = n0 + r, k = k0 + threadIdx.x;
    if (k < ncoords && n < nt_ic) dst[(size_t)n * ncoords + k] = tile[threadIdx.x][r];
  }
}

__global__ void any_nonzero(const float* a, int64_t n, int* flag) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n;
       c += (int64_t)gridDim.x * blockDim.x)
    if (a[c] != 0.f) { *flag = 1; return; }
}

// Copy a dense C-order grid array (host or device) into a padded device array.
int upload_grid(fw_handle* h, void* dst, const void* src, size_t elem, bool on_device,
                cudaStream_t s) {
  const int64_t last = h->ndim == 2 ? h->ny : h->nz;
  const int64_t rows = h->ndim == 2 ? h->nx : h->nx * h->ny;
  FW_CUDA(h, cudaMemcpy2DAsync(dst, h->pitch * elem, src, last * elem, last * elem, rows,
                               on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s));
  return FW_OK;
}

// Self-test kernels for the bounded waits: each waits on something nothing will complete.
__global__ void selftest_mbar_timeout(int* status) {
  __shared__ alignas(8) uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_barrier_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) mbar_wait_bounded(&bar, 0, status);   // no arrival: gives up
}

__global__ void selftest_grid_barrier_timeout(unsigned* bar, int* status) {
  // one block, while the barrier counts two: the generation never advances
  grid_barrier(bar, status, 2u);
}

int check_desc(const fw_desc* d) {
  if (!d) return fail(nullptr, FW_ERR_ARGUMENT, "desc is NULL");
  if (d->ndim != 2 && d->ndim != 3) return fail(nullptr, FW_ERR_ARGUMENT, "ndim must be 2 or 3, got %d", d->ndim);
  const int nz = d->ndim == 3 ? d->nz : 1;
  if (d->nx <= 2 * kGhost || d->ny <= 2 * kGhost || (d->ndim == 3 && nz <= 2 * kGhost))
    return fail(nullptr, FW_ERR_ARGUMENT, "every axis needs more than %d cells (got %d x %d x %d)",
                2 * kGhost, d->nx, d->ny, nz);
  if (d->nt < 0 || d->nt_ic < 0 || d->mod_t < 1 || d->ncoords < 0 || d->ncoordsout < 0 ||
      d->ncoordszero < 0 || d->ndmap < 1)
    return fail(nullptr, FW_ERR_ARGUMENT, "negative count or modT/ndmap < 1");
  if (d->ndmap > 65535)   // the engine keeps the tap-set index of a cell in 16 bits
    return fail(nullptr, FW_ERR_ARGUMENT, "ndmap = %d: at most 65535 tap sets", d->ndmap);
  if (!(d->dt > 0.f) || !(d->dx > 0.f) || !(d->dy > 0.f) || (d->ndim == 3 && !(d->dz > 0.f)))
    return fail(nullptr, FW_ERR_ARGUMENT, "grid spacing and time step must be positive");
  if (d->isotropic != 0 && d->isotropic != 1)
    return fail(nullptr, FW_ERR_ARGUMENT, "isotropic must be 0 or 1 (got %d)", d->isotropic);
  if (d->n_relax != 2 && d->n_relax != 0)
    return fail(nullptr, FW_ERR_UNSUPPORTED,
                "n_relax must be 2 (relaxation engine) or 0 (exponential attenuation), got %d",
                d->n_relax);
  if (d->n_relax == 0 && d->isotropic != 1)
    return fail(nullptr, FW_ERR_ARGUMENT, "the exponential-attenuation engine has no per-axis maps");
  return FW_OK;
}

}  // namespace

extern "C" {

int fw_abi_version(void) { return FWGB_ABI_VERSION; }

int fw_create(const fw_desc* desc, fw_handle** out) {
  if (!out) return fail(nullptr, FW_ERR_ARGUMENT, "out is NULL");
  *out = nullptr;
  int st = check_desc(desc);
  if (st) return st;
  fw_handle* h = new (std::nothrow) fw_handle();
  if (!h) return fail(nullptr, FW_ERR_OOM, "host allocation failed");
  h->d = *desc;
  h->ndim = desc->ndim;
  h->nx = desc->nx;
  h->ny = desc->ny;
  h->nz = desc->ndim == 3 ? desc->nz : 1;
  h->aniso = desc->isotropic == 0;
  h->exp = desc->n_relax == 0;
  h->pitch = round_up(h->ndim == 2 ? h->ny : h->nz, 32);
  h->ncells_padded = h->ndim == 2 ? h->nx * h->pitch : h->nx * h->ny * h->pitch;
  h->n_out = (desc->nt + desc->mod_t - 1) / desc->mod_t;
  h->n_cols = desc->ncoordsout;
  {
    const char* v = std::getenv("FWGB_VARIANT");
    h->variant = (h->ndim == 3 && !(v && std::strcmp(v, "direct") == 0)) ? kMarch : kDirect;
    if (h->variant == kMarch) {
      // isotropic relaxation engine: point-wise operands staged by TMA as well, unless
      // FWGB_STREAM3D=0. Streaming blocks march 32 planes with a two-stage point-wise ring (the
      // next plane's operands in flight while a plane is computed); FWGB_XC3D=64 marches 64
      // planes and FWGB_PS3D=3 then deepens the ring to three stages. Measured on the plain 3D
      // workload (Gcell/s): 32 planes 33.74, 64 planes 33.37 (3 stages 31.36), 16 planes
      // 33.30, 128 planes 32.34.
      const char* sv = std::getenv("FWGB_STREAM3D");
      const char* ps = std::getenv("FWGB_PS3D");
      const char* xc = std::getenv("FWGB_XC3D");
      h->stream3d = !h->aniso && !h->exp && !(sv && std::strcmp(sv, "0") == 0);
      h->ps3d = (ps && std::strcmp(ps, "3") == 0) ? 3 : 2;
      const bool x64 = (xc && std::strcmp(xc, "64") == 0) || h->ps3d == 3;
      if (h->stream3d && !x64) h->march_xc = kStreamXC;
    }
  }
  h->tiling = make_tiling(h);
  auto alloc = [&](void** p, size_t bytes) -> int {
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return fail(nullptr, e == cudaErrorMemoryAllocation ? FW_ERR_OOM : FW_ERR_CUDA,
                  "cudaMalloc(%zu bytes) failed: %s", bytes, cudaGetErrorString(e));
    }
    h->bytes += bytes;
    return FW_OK;
  };
  const size_t cells = (size_t)h->ncells_padded;
  if ((st = alloc((void**)&h->state, cells * n_state(h->ndim) * sizeof(float))) ||
      (st = alloc((void**)&h->maps, cells * n_maps(h) * sizeof(float))) ||
      (st = alloc((void**)&h->dcmap, cells * sizeof(uint16_t))) ||
      (st = alloc((void**)&h->taps, (size_t)desc->ndmap * kTapStride * sizeof(float))) ||
      (st = alloc((void**)&h->icmat_t, (size_t)desc->ncoords * desc->nt_ic * sizeof(float))) ||
      (st = alloc((void**)&h->traces, (size_t)h->n_out * desc->ncoordsout * sizeof(float))) ||
      (st = alloc((void**)&h->step, sizeof(int) * 4))) {
    fw_destroy(h);
    return st;
  }
  if (cudaStreamCreateWithFlags(&h->capture_stream, cudaStreamNonBlocking) != cudaSuccess) {
    fw_destroy(h);
    return fail(nullptr, FW_ERR_CUDA, "stream creation failed");
  }
  // zero everything once: ghost cells, padding and memory variables start at zero
  if (cudaMemset(h->state, 0, cells * n_state(h->ndim) * sizeof(float)) != cudaSuccess ||
      cudaMemset(h->maps, 0, cells * n_maps(h) * sizeof(float)) != cudaSuccess ||
      cudaMemset(h->dcmap, 0, cells * sizeof(uint16_t)) != cudaSuccess ||
      cudaMemset(h->step, 0, sizeof(int) * 4) != cudaSuccess) {
    fw_destroy(h);
    return fail(nullptr, FW_ERR_CUDA, "initial cudaMemset failed");
  }
  // argument block
  StepArgs& A = h->args;
  A.g.nx = (int)h->nx; A.g.ny = (int)h->ny; A.g.nz = (int)h->nz;
  A.g.sx = h->ndim == 2 ? h->pitch : h->ny * h->pitch;
  A.g.sy = h->ndim == 2 ? 1 : h->pitch;
  A.g.inv_h[0] = 1.f / desc->dx;
  A.g.inv_h[1] = 1.f / desc->dy;
  A.g.inv_h[2] = h->ndim == 3 ? 1.f / desc->dz : 0.f;
  set_state_pointers(h, &A, h->state);
  A.m.rdt_rho = map_field(h, kMRdtRho);
  A.m.dt_k = map_field(h, kMDtK);
  A.m.beta2dt = map_field(h, kMBeta2dt);
  for (int a = 0; a < 3; ++a) {
    const bool own = h->aniso && a >= 1 && a < h->ndim;
    A.m.inv_ku[a] = own ? map_field(h, axis_map(a, 0)) : map_field(h, kMInvKu);
    A.m.au[a][0] = own ? map_field(h, axis_map(a, 1)) : map_field(h, kMAu1);
    A.m.bu[a][0] = own ? map_field(h, axis_map(a, 2)) : map_field(h, kMBu1);
    A.m.au[a][1] = own ? map_field(h, axis_map(a, 3)) : map_field(h, kMAu2);
    A.m.bu[a][1] = own ? map_field(h, axis_map(a, 4)) : map_field(h, kMBu2);
    A.m.inv_kx[a] = own ? map_field(h, axis_map(a, 5)) : map_field(h, kMInvKx);
    A.m.ax[a][0] = own ? map_field(h, axis_map(a, 6)) : map_field(h, kMAx1);
    A.m.bx[a][0] = own ? map_field(h, axis_map(a, 7)) : map_field(h, kMBx1);
    A.m.ax[a][1] = own ? map_field(h, axis_map(a, 8)) : map_field(h, kMAx2);
    A.m.bx[a][1] = own ? map_field(h, axis_map(a, 9)) : map_field(h, kMBx2);
  }
  A.m.a_exp = map_field(h, kMAu1);  // exponential engine: a_exp in the first relaxation slot
  A.m.dcmap = h->dcmap;
  A.m.taps = h->taps;
  A.l.icmat_t = h->icmat_t;
  A.l.traces = h->traces;
  A.l.ncoords = desc->ncoords;
  A.l.ncoordsout = desc->ncoordsout;
  A.l.nt_ic = desc->nt_ic;
  A.l.mod_t = desc->mod_t;
  A.step = h->step;
  if (h->ndim == 2) {
    // isotropic relaxation engine: the row-march shapes stage the point-wise operands by TMA too,
    // unless FWGB_STREAM2D=0
    const char* s2 = std::getenv("FWGB_STREAM2D");
    h->stream2d = !h->aniso && !h->exp && !(s2 && std::strcmp(s2, "0") == 0);
    // 2D kernel shape: forced by FWGB_VARIANT=direct or FWGB_SHAPE2D=<k>, else the direct kernels
    // until the autotuner (first advance from step 0) has measured the shapes for this grid
    const char* v = std::getenv("FWGB_VARIANT");
    const char* sh = std::getenv("FWGB_SHAPE2D");
    int k = 0;
    if (v && std::strcmp(v, "direct") == 0) {
      h->shape_fixed = true;
    } else if (sh && *sh) {
      k = std::atoi(sh);
      if (k < 0 || k >= kNumShapes2D) {
        fw_destroy(h);
        return fail(nullptr, FW_ERR_ARGUMENT, "FWGB_SHAPE2D=%s outside [0, %d)", sh, kNumShapes2D);
      }
      h->shape_fixed = true;
    } else if (v && std::strcmp(v, "march") == 0) {
      k = 4;
      h->shape_fixed = true;
    }
    if ((st = set_shape2d(h, k))) {
      g_create_error = h->err;
      fw_destroy(h);
      return st;
    }
  }
  if (h->variant == kMarch && h->ndim == 3) {
    if ((st = encode_field_map(h, &h->tmaps.p, A.f.p, kPW, kPH)) ||
        (st = encode_field_map(h, &h->tmaps.vx, A.f.v[0], kXW, kXH)) ||
        (st = encode_field_map(h, &h->tmaps.vy, A.f.v[1], kYW, kYH)) ||
        (st = encode_field_map(h, &h->tmaps.vz, A.f.v[2], kZW, kZH)) ||
        (h->stream3d && ((st = encode_stream_maps(h)) || (st = prepare_stream3d(h))))) {
      g_create_error = h->err;
      fw_destroy(h);
      return st;
    }
  }
  *out = h;
  return FW_OK;
}

}  // extern "C"

namespace {

int set_fields_impl(fw_handle* h, const fw_fields* f, const fw_fields_aniso* an,
                    const float* a_exp) {
  if (!h) return fail(nullptr, FW_ERR_ARGUMENT, "handle is NULL");
  if (!f) return fail(h, FW_ERR_ARGUMENT, "fields is NULL");
  if (h->exp != (a_exp != nullptr))
    return fail(h, FW_ERR_ARGUMENT, h->exp ? "an exponential-attenuation handle (n_relax = 0) needs "
                                             "fw_set_fields_exp"
                                           : "a_exp given to a relaxation handle");
  if (h->aniso && !an)
    return fail(h, FW_ERR_ARGUMENT, "an anisotropic handle (isotropic = 0) needs fw_set_fields_aniso");
  if (!h->aniso && an)
    return fail(h, FW_ERR_ARGUMENT, "per-direction maps given to an isotropic handle");
  const fw_desc& d = h->d;
  const float* need[] = {f->d, f->dmap, f->c, f->rho, f->K, f->beta};
  for (const float* p : need)
    if (!p) return fail(h, FW_ERR_ARGUMENT, "a required map or table pointer is NULL");
  const float* need_relax[] = {f->kappax, f->kappau, f->apmlu1, f->bpmlu1, f->apmlx1, f->bpmlx1,
                               f->apmlu2, f->bpmlu2, f->apmlx2, f->bpmlx2};
  if (!h->exp)
    for (const float* p : need_relax)
      if (!p) return fail(h, FW_ERR_ARGUMENT, "a required relaxation map pointer is NULL");
  if (!f->dcmap) return fail(h, FW_ERR_ARGUMENT, "dcmap is NULL");
  if ((d.ncoords && (!f->icc || (d.nt_ic && !f->icmat))) || (d.ncoordsout && !f->outc) ||
      (d.ncoordszero && !f->icczero))
    return fail(h, FW_ERR_ARGUMENT, "coordinate or icmat pointer is NULL");
  const bool dev = f->on_device != 0;
  cudaStream_t s = h->capture_stream;
  // captured graphs hold the old list pointers and kernel choice: rebuild them on next use
  if (h->graph) {
    cudaGraphExecDestroy(h->graph);
    h->graph = nullptr;
    h->graph_steps = 0;
  }
  const size_t dense = (size_t)h->nx * h->ny * h->nz;
  const int nd = h->ndim;

  // -- coordinates (validated on the host) and per-tile lists ---------------------------------
  auto fetch_i32 = [&](const int32_t* src, size_t n, std::vector<int32_t>& out) -> int {
    out.resize(n);
    if (!n) return FW_OK;
    FW_CUDA(h, cudaMemcpy(out.data(), src, n * sizeof(int32_t),
                          dev ? cudaMemcpyDeviceToHost : cudaMemcpyHostToHost));
    return FW_OK;
  };
  std::vector<int32_t> icc, outc, zero, dcm;
  int st;
  if ((st = fetch_i32(f->icc, (size_t)d.ncoords * nd, icc)) ||
      (st = fetch_i32(f->outc, (size_t)d.ncoordsout * nd, outc)) ||
      (st = fetch_i32(f->icczero, (size_t)d.ncoordszero * nd, zero)) ||
      (st = fetch_i32(f->dcmap, dense, dcm)))
    return st;
  for (size_t c = 0; c < dense; ++c)
    if (dcm[c] < 0 || dcm[c] >= d.ndmap)
      return fail(h, FW_ERR_ARGUMENT, "dcmap[%zu] = %d outside [0, %d)", c, dcm[c], d.ndmap);
  const int64_t ext[3] = {h->nx, h->ny, h->nz};
  auto cell_of = [&](const std::vector<int32_t>& v, size_t e, int64_t* cell, int* tile) -> bool {
    int64_t q[3] = {0, 0, 0};
    for (int a = 0; a < nd; ++a) {
      q[a] = v[e * nd + a];
      if (q[a] < 0 || q[a] >= ext[a]) return false;
    }
    *cell = padded_index(h, q[0], q[1], q[2]);
    *tile = tile_of(h, q[0], q[1], q[2]);
    return true;
  };
  const int ntiles = h->tiling.count();
  struct Entry { int tile; int64_t cell; int32_t k; };
  auto build = [&](const std::vector<int32_t>& v, int n, const char* name, bool dedupe_last,
                   std::vector<Entry>& out) -> int {
    out.clear();
    out.reserve(n);
    for (int e = 0; e < n; ++e) {
      Entry en{0, 0, e};
      if (!cell_of(v, (size_t)e, &en.cell, &en.tile))
        return fail(h, FW_ERR_ARGUMENT, "%s[%d] lies outside the %d-D grid", name, e, nd);
      out.push_back(en);
    }
    if (dedupe_last) {  // a cell listed twice is driven by its last entry
      std::vector<Entry> tmp = out;
      std::stable_sort(tmp.begin(), tmp.end(), [](const Entry& a, const Entry& b) { return a.cell < b.cell; });
      out.clear();
      for (size_t e = 0; e < tmp.size(); ++e)
        if (e + 1 == tmp.size() || tmp[e + 1].cell != tmp[e].cell) out.push_back(tmp[e]);
    }
    std::stable_sort(out.begin(), out.end(), [](const Entry& a, const Entry& b) {
      return a.tile != b.tile ? a.tile < b.tile : a.k < b.k;
    });
    return FW_OK;
  };
  std::vector<Entry> es, ez, eo;
  if ((st = build(icc, d.ncoords, "icc", true, es)) ||
      (st = build(zero, d.ncoordszero, "icczero", true, ez)) ||
      (st = build(outc, d.ncoordsout, "outc", false, eo)))
    return st;
  // pressure written in the ghost layer (sources or air cells there): it then persists across
  // steps, which the out-of-place adjoint recomputation does not carry over
  auto in_ghost = [&](const std::vector<int32_t>& v, int n) {
    for (int e = 0; e < n; ++e)
      for (int a = 0; a < nd; ++a)
        if (v[(size_t)e * nd + a] < kGhost || v[(size_t)e * nd + a] >= ext[a] - kGhost) return true;
    return false;
  };
  h->ghost_writes = in_ghost(icc, d.ncoords) || in_ghost(zero, d.ncoordszero);
  // layout: src_ptr, zero_ptr, rec_ptr (int32, ntiles+1 each), src_k, rec_k (int32),
  //         then src_cell, zero_cell, rec_cell (int64, 8-byte aligned)
  const size_t n_i32 = 3 * (size_t)(ntiles + 1) + es.size() + eo.size();
  const size_t off64 = round_up((int64_t)(n_i32 * 4), 16);
  const size_t n_i64 = es.size() + ez.size() + eo.size();
  std::vector<unsigned char> blob(off64 + n_i64 * 8 + 16, 0);
  int32_t* i32 = reinterpret_cast<int32_t*>(blob.data());
  int64_t* i64 = reinterpret_cast<int64_t*>(blob.data() + off64);
  auto fill_ptr = [&](const std::vector<Entry>& v, int32_t* ptr) {
    std::fill(ptr, ptr + ntiles + 1, 0);
    for (const Entry& e : v) ptr[e.tile + 1]++;
    for (int t = 0; t < ntiles; ++t) ptr[t + 1] += ptr[t];
  };
  int32_t* src_ptr = i32;
  int32_t* zero_ptr = src_ptr + ntiles + 1;
  int32_t* rec_ptr = zero_ptr + ntiles + 1;
  int32_t* src_k = rec_ptr + ntiles + 1;
  int32_t* rec_k = src_k + es.size();
  fill_ptr(es, src_ptr);
  fill_ptr(ez, zero_ptr);
  fill_ptr(eo, rec_ptr);
  int64_t* src_cell = i64;
  int64_t* zero_cell = src_cell + es.size();
  int64_t* rec_cell = zero_cell + ez.size();
  for (size_t e = 0; e < es.size(); ++e) { src_k[e] = es[e].k; src_cell[e] = es[e].cell; }
  for (size_t e = 0; e < ez.size(); ++e) zero_cell[e] = ez[e].cell;
  for (size_t e = 0; e < eo.size(); ++e) { rec_k[e] = eo[e].k; rec_cell[e] = eo[e].cell; }
  h->rec_k_host.assign(rec_k, rec_k + eo.size());
  if (h->groups) {  // new sensor lists: previous groups no longer apply
    cudaFree(h->groups);
    h->groups = nullptr;
    h->args.l.rec_group = nullptr;
    h->args.l.rec_w = nullptr;
    if (h->n_cols != d.ncoordsout) {
      cudaFree(h->traces);
      h->traces = nullptr;
      FW_CUDA(h, cudaMalloc(&h->traces, (size_t)h->n_out * std::max(d.ncoordsout, 1) * sizeof(float)));
      h->args.l.traces = h->traces;
    }
    h->n_cols = d.ncoordsout;
    h->args.l.ncoordsout = d.ncoordsout;
  }
  if (h->lists) { cudaFree(h->lists); h->lists = nullptr; }
  FW_CUDA(h, cudaMalloc(&h->lists, blob.size()));
  FW_CUDA(h, cudaMemcpy(h->lists, blob.data(), blob.size(), cudaMemcpyHostToDevice));
  unsigned char* L = static_cast<unsigned char*>(h->lists);
  const size_t o_src_k = (size_t)(src_k - i32) * 4, o_rec_k = (size_t)(rec_k - i32) * 4;
  h->args.l.src_ptr = reinterpret_cast<int32_t*>(L);
  h->args.l.zero_ptr = reinterpret_cast<int32_t*>(L) + ntiles + 1;
  h->args.l.rec_ptr = reinterpret_cast<int32_t*>(L) + 2 * (ntiles + 1);
  h->args.l.src_k = reinterpret_cast<int32_t*>(L + o_src_k);
  h->args.l.rec_k = reinterpret_cast<int32_t*>(L + o_rec_k);
  h->args.l.src_cell = reinterpret_cast<int64_t*>(L + off64);
  h->args.l.zero_cell = reinterpret_cast<int64_t*>(L + off64) + es.size();
  h->args.l.rec_cell = reinterpret_cast<int64_t*>(L + off64) + es.size() + ez.size();

  // -- maps -------------------------------------------------------------------------------------
  struct { const float* src; int idx; bool relax; } mapsrc[] = {
      {f->rho, kMRdtRho, false}, {f->K, kMDtK, false}, {f->beta, kMBeta2dt, false},
      {f->kappau, kMInvKu, true}, {f->kappax, kMInvKx, true},
      {f->apmlu1, kMAu1, true}, {f->bpmlu1, kMBu1, true}, {f->apmlu2, kMAu2, true},
      {f->bpmlu2, kMBu2, true}, {f->apmlx1, kMAx1, true}, {f->bpmlx1, kMBx1, true},
      {f->apmlx2, kMAx2, true}, {f->bpmlx2, kMBx2, true}};
  for (auto& m : mapsrc) {
    if (h->exp && m.relax) continue;  // no relaxation maps in the exponential engine
    if ((st = upload_grid(h, map_field(h, m.idx), m.src, sizeof(float), dev, s))) return st;
  }
  if (h->exp && (st = upload_grid(h, map_field(h, kMAu1), a_exp, sizeof(float), dev, s)))
    return st;
  std::vector<int> kappa_maps;
  if (!h->exp) kappa_maps = {kMInvKu, kMInvKx};
  if (h->aniso) {
    // axis y: kappaw/apmlw*/bpmlw* (gradient), kappay/apmly*/bpmly* (divergence); axis z: v, z
    const float* per_axis[3][10] = {
        {},
        {an->kappaw, an->apmlw1, an->bpmlw1, an->apmlw2, an->bpmlw2,
         an->kappay, an->apmly1, an->bpmly1, an->apmly2, an->bpmly2},
        {an->kappav, an->apmlv1, an->bpmlv1, an->apmlv2, an->bpmlv2,
         an->kappaz, an->apmlz1, an->bpmlz1, an->apmlz2, an->bpmlz2}};
    for (int a = 1; a < h->ndim; ++a)
      for (int k = 0; k < 10; ++k) {
        if (!per_axis[a][k]) return fail(h, FW_ERR_ARGUMENT, "a per-direction map for axis %d is NULL", a);
        if ((st = upload_grid(h, map_field(h, axis_map(a, k)), per_axis[a][k], sizeof(float), dev, s)))
          return st;
      }
    for (int a = 1; a < h->ndim; ++a) {
      kappa_maps.push_back(axis_map(a, 0));
      kappa_maps.push_back(axis_map(a, 5));
    }
  }
  {  // 16-bit tap-set indices (validated above: 0 <= dcmap < ndmap <= 65535)
    std::vector<uint16_t> dc16(dcm.begin(), dcm.end());
    if ((st = upload_grid(h, h->dcmap, dc16.data(), sizeof(uint16_t), false, s))) return st;
    FW_CUDA(h, cudaStreamSynchronize(s));   // the host copy is freed on return
  }
  transform_maps<<<1024, 256, 0, s>>>(map_field(h, kMRdtRho), map_field(h, kMDtK),
                                      map_field(h, kMBeta2dt), h->ncells_padded, d.dt);
  for (int idx : kappa_maps) invert_map<<<1024, 256, 0, s>>>(map_field(h, idx), h->ncells_padded);
  FW_CUDA(h, cudaGetLastError());
  // beta: use the nonlinear kernel only when some cell has beta != 0
  any_nonzero<<<1024, 256, 0, s>>>(map_field(h, kMBeta2dt), h->ncells_padded, h->step + 2);
  FW_CUDA(h, cudaGetLastError());
  int flag = 0;
  FW_CUDA(h, cudaMemcpyAsync(&flag, h->step + 2, sizeof(int), cudaMemcpyDeviceToHost, s));
  FW_CUDA(h, cudaStreamSynchronize(s));
  h->has_beta = flag != 0;
  h->args.m.beta2dt = h->has_beta ? map_field(h, kMBeta2dt) : nullptr;

  // -- tap table [ndmap][12] ----------------------------------------------------------------------
  std::vector<float> dmap((size_t)18 * d.ndmap), taps((size_t)d.ndmap * kTapStride, 0.f);
  FW_CUDA(h, cudaMemcpy(dmap.data(), f->dmap, dmap.size() * sizeof(float),
                        dev ? cudaMemcpyDeviceToHost : cudaMemcpyHostToHost));
  for (int e = 0; e < d.ndmap; ++e) {
    for (int m = 1; m <= 8; ++m) taps[(size_t)e * kTapStride + m - 1] = dmap[((size_t)m * 2 + 0) * d.ndmap + e];
    taps[(size_t)e * kTapStride + 8] = dmap[((size_t)1 * 2 + 1) * d.ndmap + e];
  }
  FW_CUDA(h, cudaMemcpy(h->taps, taps.data(), taps.size() * sizeof(float), cudaMemcpyHostToDevice));

  // -- source signals -------------------------------------------------------------------------
  h->fields_set = true;
  if (d.ncoords && d.nt_ic) {
    if ((st = fw_set_source_signal(h, f->icmat, f->on_device))) { h->fields_set = false; return st; }
  }
  st = fw_reset(h, s);
  if (st) return st;
  FW_CUDA(h, cudaStreamSynchronize(s));
  return FW_OK;
}

}  // namespace

extern "C" {

int fw_set_fields(fw_handle* h, const fw_fields* f) {
  return set_fields_impl(h, f, nullptr, nullptr);
}

int fw_set_fields_aniso(fw_handle* h, const fw_fields* f, const fw_fields_aniso* an) {
  if (!an) return fail(h, FW_ERR_ARGUMENT, "per-direction maps are NULL");
  return set_fields_impl(h, f, an, nullptr);
}

int fw_set_fields_exp(fw_handle* h, const fw_fields* f, const float* a_exp) {
  if (!a_exp) return fail(h, FW_ERR_ARGUMENT, "a_exp is NULL");
  return set_fields_impl(h, f, nullptr, a_exp);
}

int fw_set_source_signal(fw_handle* h, const float* icmat, int32_t on_device) {
  if (!h) return fail(nullptr, FW_ERR_ARGUMENT, "handle is NULL");
  const fw_desc& d = h->d;
  if (!d.ncoords || !d.nt_ic) return FW_OK;
  if (!icmat) return fail(h, FW_ERR_ARGUMENT, "icmat is NULL");
  const size_t n = (size_t)d.ncoords * d.nt_ic;
  float* staging = nullptr;
  FW_CUDA(h, cudaMalloc(&staging, n * sizeof(float)));
  cudaStream_t s = h->capture_stream;
  cudaError_t e = cudaMemcpyAsync(staging, icmat, n * sizeof(float),
                                  on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) {
    dim3 grid((d.nt_ic + 31) / 32, (d.ncoords + 31) / 32), block(32, 8);
    transpose_icmat<<<grid, block, 0, s>>>(staging, h->icmat_t, d.ncoords, d.nt_ic);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFree(staging);
  if (e != cudaSuccess) return fail(h, FW_ERR_CUDA, "source upload failed: %s", cudaGetErrorString(e));
  return FW_OK;
}

int fw_set_sensor_groups(fw_handle* h, const int32_t* group_of_sensor, const float* weight,
                         int32_t n_groups) {
  if (!h) return fail(nullptr, FW_ERR_ARGUMENT, "handle is NULL");
  if (!h->fields_set) return fail(h, FW_ERR_STATE, "fw_set_fields must be called first");
  if (n_groups < 0 || (n_groups > 0 && (!group_of_sensor || !weight)))
    return fail(h, FW_ERR_ARGUMENT, "bad sensor groups");
  const fw_desc& d = h->d;
  if (h->graph) {
    cudaGraphExecDestroy(h->graph);
    h->graph = nullptr;
    h->graph_steps = 0;
  }
  if (h->groups) {
    cudaFree(h->groups);
    h->groups = nullptr;
  }
  const int32_t cols = n_groups > 0 ? n_groups : d.ncoordsout;
  if (cols != h->n_cols) {
    cudaFree(h->traces);
    h->traces = nullptr;
    FW_CUDA(h, cudaMalloc(&h->traces, (size_t)h->n_out * std::max(cols, 1) * sizeof(float)));
    h->args.l.traces = h->traces;
    h->n_cols = cols;
  }
  h->args.l.ncoordsout = cols;
  h->args.l.rec_group = nullptr;
  h->args.l.rec_w = nullptr;
  if (n_groups > 0) {
    const size_t ne = h->rec_k_host.size();
    std::vector<int32_t> grp(ne);
    std::vector<float> w(ne);
    for (size_t e = 0; e < ne; ++e) {
      const int k = h->rec_k_host[e];
      grp[e] = group_of_sensor[k];
      w[e] = weight[k];
      if (grp[e] >= n_groups) return fail(h, FW_ERR_ARGUMENT, "sensor %d: group %d >= %d", k, grp[e], n_groups);
    }
    FW_CUDA(h, cudaMalloc(&h->groups, ne * 8 + 16));
    int32_t* dg = static_cast<int32_t*>(h->groups);
    float* dw = reinterpret_cast<float*>(dg + ne);
    FW_CUDA(h, cudaMemcpy(dg, grp.data(), ne * 4, cudaMemcpyHostToDevice));
    FW_CUDA(h, cudaMemcpy(dw, w.data(), ne * 4, cudaMemcpyHostToDevice));
    h->args.l.rec_group = dg;
    h->args.l.rec_w = dw;
  }
  int st = fw_reset(h, h->capture_stream);
  if (st) return st;
  FW_CUDA(h, cudaStreamSynchronize(h->capture_stream));
  return FW_OK;
}

int fw_set_source_columns(fw_handle* h, void* stream, const float* cols, int32_t n0,
                          int32_t ncols, int32_t on_device) {
  if (!h) return fail(nullptr, FW_ERR_ARGUMENT, "handle is NULL");
  const fw_desc& d = h->d;
  if (n0 < 0 || ncols < 0 || (int64_t)n0 + ncols > d.nt_ic)
    return fail(h, FW_ERR_ARGUMENT, "source columns [%d, %d) outside [0, %d)", n0, n0 + ncols, d.nt_ic);
  if (!d.ncoords || !ncols) return FW_OK;
  if (!cols) return fail(h, FW_ERR_ARGUMENT, "cols is NULL");
  FW_CUDA(h, cudaMemcpyAsync(h->icmat_t + (size_t)n0 * d.ncoords, cols,
                             (size_t)ncols * d.ncoords * sizeof(float),
                             on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                             static_cast<cudaStream_t>(stream)));
  return FW_OK;
}

int fw_reset(fw_handle* h, void* stream) {
  if (!h) return fail(nullptr, FW_ERR_ARGUMENT, "handle is NULL");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  FW_CUDA(h, cudaMemsetAsync(h->state, 0, (size_t)h->ncells_padded * n_state(h->ndim) * sizeof(float), s));
  FW_CUDA(h, cudaMemsetAsync(h->traces, 0, (size_t)h->n_out * h->n_cols * sizeof(float), s));
  FW_CUDA(h, cudaMemsetAsync(h->step, 0, 2 * sizeof(int), s));
  h->host_step = 0;
  return FW_OK;
}

}  // extern "C"

namespace {

std::mutex g_tune_mutex;
std::map<std::array<int64_t, 6>, int> g_tuned;   // (device, nx, ny, aniso, exp, beta) -> shape

// 2D kernel-shape autotuner. Called on the first advance from step 0, when the state is all zero:
// every shape of kShapes2D runs kTuneSteps steps twice (the second timed with events on the
// caller's stream), the handle is reset after each trial, and the fastest shape is kept. All
// shapes give bit-identical results, so the choice changes speed only. The choice is cached per
// device, grid size and cell physics, so later handles of the same kind skip the trials.
int autotune_2d(fw_handle* h, cudaStream_t s) {
  int dev = 0;
  FW_CUDA(h, cudaGetDevice(&dev));
  const std::array<int64_t, 6> key{dev, h->nx, h->ny, h->aniso, h->exp, h->has_beta};
  {
    std::lock_guard<std::mutex> lk(g_tune_mutex);
    auto it = g_tuned.find(key);
    if (it != g_tuned.end()) {
      h->shape_fixed = true;
      return it->second == h->shape2d ? FW_OK : set_shape2d(h, it->second);
    }
  }
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  FW_CUDA(h, cudaEventCreate(&e0));
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return fail(h, FW_ERR_CUDA, "cudaEventCreate failed");
  }
  int st = FW_OK, best = 0;
  float best_ms = 0.f;
  for (int k = 0; k < kNumShapes2D && st == FW_OK; ++k) {
    float ms = 0.f;
    if ((st = set_shape2d(h, k))) break;
    if (kShapes2D[k].persistent) {
      if ((st = launch_persistent(h, s, 0, kTuneSteps))) break;
      if (cudaEventRecord(e0, s) != cudaSuccess) { st = fail(h, FW_ERR_CUDA, "event record failed"); break; }
      if ((st = launch_persistent(h, s, kTuneSteps, kTuneSteps))) break;
      if (cudaEventRecord(e1, s) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
          cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) {
        st = fail(h, FW_ERR_CUDA, "autotuning trial of 2D shape %d failed: %s", k,
                  cudaGetErrorString(cudaGetLastError()));
        break;
      }
    } else {
      if ((st = build_graph(h, kTuneSteps))) break;
      if (cudaGraphLaunch(h->graph, s) != cudaSuccess || cudaEventRecord(e0, s) != cudaSuccess ||
          cudaGraphLaunch(h->graph, s) != cudaSuccess || cudaEventRecord(e1, s) != cudaSuccess ||
          cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) {
        st = fail(h, FW_ERR_CUDA, "autotuning trial of 2D shape %d failed: %s", k,
                  cudaGetErrorString(cudaGetLastError()));
        break;
      }
    }
    if ((st = check_device_status(h, s)) || (st = fw_reset(h, s))) break;
    if (k == 0 || ms < best_ms) { best_ms = ms; best = k; }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st) return st;
  if ((st = set_shape2d(h, best))) return st;
  h->shape_fixed = true;
  std::lock_guard<std::mutex> lk(g_tune_mutex);
  g_tuned[key] = best;
  return FW_OK;
}

}  // namespace

extern "C" {

int fw_advance(fw_handle* h, void* stream, int32_t n_steps) {
  if (!h) return fail(nullptr, FW_ERR_ARGUMENT, "handle is NULL");
  if (!h->fields_set) return fail(h, FW_ERR_STATE, "fw_set_fields must be called before stepping");
  if (n_steps < 0 || (int64_t)h->host_step + n_steps > h->d.nt)
    return fail(h, FW_ERR_ARGUMENT, "cannot advance %d steps from step %d (nt = %d)", n_steps,
                h->host_step, h->d.nt);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (h->ndim == 2 && !h->shape_fixed && h->host_step == 0 && n_steps > 0) {
    // autotune unless disabled (FWGB_AUTOTUNE=0), too short, or inside a stream capture
    const char* a = std::getenv("FWGB_AUTOTUNE");
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    FW_CUDA(h, cudaStreamIsCapturing(s, &cs));
    if ((a && std::strcmp(a, "0") == 0) || h->d.nt < 2 * kTuneSteps) {
      h->shape_fixed = true;
    } else if (cs == cudaStreamCaptureStatusNone) {
      int st = autotune_2d(h, s);
      if (st) return st;
    }
  }
  if (h->ndim == 2 && kShapes2D[h->shape2d].persistent) {
    // one cooperative launch for all the steps; under a stream capture the direct kernels run
    // instead (same results)
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    FW_CUDA(h, cudaStreamIsCapturing(s, &cs));
    if (cs == cudaStreamCaptureStatusNone) {
      int st = launch_persistent(h, s, h->host_step, n_steps);
      if (st) return st;
      h->host_step += n_steps;
      return FW_OK;
    }
  }
  constexpr int kGraphSteps = 64;
  int left = n_steps;
  if (left >= kGraphSteps) {
    if (h->graph_steps != kGraphSteps) {
      int st = build_graph(h, kGraphSteps);
      if (st) return st;
    }
    while (left >= kGraphSteps) {
      FW_CUDA(h, cudaGraphLaunch(h->graph, s));
      left -= kGraphSteps;
    }
  }
  for (; left > 0; --left) launch_step(h, s);
  FW_CUDA(h, cudaGetLastError());
  h->host_step += n_steps;
  return FW_OK;
}

int fw_run(fw_handle* h, void* stream, float* out, int32_t out_on_device) {
  if (!h) return fail(nullptr, FW_ERR_ARGUMENT, "handle is NULL");
  int st;
  if ((st = fw_reset(h, stream)) || (st = fw_advance(h, stream, h->d.nt))) return st;
  if (out) return fw_read_traces(h, stream, 0, h->n_out, out, out_on_device);
  return check_device_status(h, static_cast<cudaStream_t>(stream));
}

int fw_read_traces(fw_handle* h, void* stream, int32_t row0, int32_t n_rows, float* dst,
                   int32_t on_device) {
  if (!h) return fail(nullptr, FW_ERR_ARGUMENT, "handle is NULL");
  if (row0 < 0 || n_rows < 0 || row0 + n_rows > h->n_out)
    return fail(h, FW_ERR_ARGUMENT, "trace rows [%d, %d) outside [0, %d)", row0, row0 + n_rows, h->n_out);
  if (!dst && n_rows) return fail(h, FW_ERR_ARGUMENT, "dst is NULL");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t n = (size_t)n_rows * h->n_cols;
  if (n) FW_CUDA(h, cudaMemcpyAsync(dst, h->traces + (size_t)row0 * h->n_cols, n * sizeof(float),
                                    on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, s));
  if (!on_device) {
    FW_CUDA(h, cudaStreamSynchronize(s));
    return check_device_status(h, s);
  }
  return FW_OK;
}

int fw_trace_buffer(fw_handle* h, float** dev_ptr) {
  if (!h || !dev_ptr) return fail(h, FW_ERR_ARGUMENT, "NULL argument");
  *dev_ptr = h->traces;
  return FW_OK;
}

int fw_get_field(fw_handle* h, void* stream, int32_t field, float* dst, int32_t on_device) {
  if (!h) return fail(nullptr, FW_ERR_ARGUMENT, "handle is NULL");
  if (field < 0 || field > h->ndim || !dst) return fail(h, FW_ERR_ARGUMENT, "bad field %d or NULL dst", field);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const float* src = field == 0 ? h->args.f.p : h->args.f.v[field - 1];
  const int64_t last = h->ndim == 2 ? h->ny : h->nz;
  const int64_t rows = h->ndim == 2 ? h->nx : h->nx * h->ny;
  FW_CUDA(h, cudaMemcpy2DAsync(dst, last * sizeof(float), src, h->pitch * sizeof(float),
                               last * sizeof(float), rows,
                               on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, s));
  if (!on_device) FW_CUDA(h, cudaStreamSynchronize(s));
  return FW_OK;
}

int fw_current_step(const fw_handle* h, int32_t* step) {
  if (!h || !step) return FW_ERR_ARGUMENT;
  *step = h->host_step;
  return FW_OK;
}

int fw_device_bytes(const fw_handle* h, uint64_t* bytes) {
  if (!h || !bytes) return FW_ERR_ARGUMENT;
  *bytes = h->bytes;
  return FW_OK;
}

int fw_kernel_variant(const fw_handle* h, int32_t* variant) {
  if (!h || !variant) return FW_ERR_ARGUMENT;
  *variant = (h->variant == kMarch && h->stream3d) ? kStream : h->variant;
  return FW_OK;
}

int fw_block_tile(const fw_handle* h, int32_t tile[3]) {
  if (!h || !tile) return FW_ERR_ARGUMENT;
  if (h->ndim == 2 && kShapes2D[h->shape2d].ty > 0) {
    tile[0] = kShapes2D[h->shape2d].xc;
    tile[1] = kShapes2D[h->shape2d].ty;
    tile[2] = 1;
  } else {
    for (int a = 0; a < 3; ++a) tile[a] = h->tiling.t[a];
  }
  return FW_OK;
}

int fw_launches_per_step(const fw_handle* h, int32_t* n) {
  if (!h || !n) return FW_ERR_ARGUMENT;
  *n = 2;
  return FW_OK;
}

int fw_copy_state_rows(fw_handle* dst, int32_t dst_row0, const fw_handle* src, int32_t src_row0,
                       int32_t n_rows, void* stream) {
  if (!dst || !src) return fail(nullptr, FW_ERR_ARGUMENT, "handle is NULL");
  if (dst->ndim != src->ndim || dst->ny != src->ny || dst->nz != src->nz ||
      dst->pitch != src->pitch)
    return fail(dst, FW_ERR_ARGUMENT, "state rows copy between grids of different cross-section");
  if (n_rows < 0 || dst_row0 < 0 || src_row0 < 0 || dst_row0 + n_rows > dst->nx ||
      src_row0 + n_rows > src->nx)
    return fail(dst, FW_ERR_ARGUMENT, "rows [%d, %d) <- [%d, %d) outside the grids (%lld, %lld)",
                dst_row0, dst_row0 + n_rows, src_row0, src_row0 + n_rows, (long long)dst->nx,
                (long long)src->nx);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t row = (size_t)(dst->ndim == 2 ? dst->pitch : dst->ny * dst->pitch);
  for (int f = 0; f < n_state(dst->ndim); ++f) {
    float* d = state_field(dst, f) + row * dst_row0;
    const float* sp = src->state + (size_t)f * src->ncells_padded + row * src_row0;
    FW_CUDA(dst, cudaMemcpyAsync(d, sp, row * n_rows * sizeof(float), cudaMemcpyDeviceToDevice, s));
  }
  return FW_OK;
}

int fw_selftest_waits(int32_t status_out[2]) {
  if (!status_out) return fail(nullptr, FW_ERR_ARGUMENT, "status_out is NULL");
  int* st = nullptr;
  unsigned* bar = nullptr;
  if (cudaMalloc(&st, 2 * sizeof(int)) != cudaSuccess ||
      cudaMalloc(&bar, kBarWords * sizeof(unsigned)) != cudaSuccess) {
    cudaFree(st);
    return fail(nullptr, FW_ERR_OOM, "self-test allocation failed");
  }
  cudaError_t e = cudaMemset(st, 0, 2 * sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(bar, 0, kBarWords * sizeof(unsigned));
  if (e == cudaSuccess) {
    selftest_mbar_timeout<<<1, 32>>>(st);
    selftest_grid_barrier_timeout<<<1, dim3(kD2TY, kD2TX)>>>(bar, st + 1);
    e = cudaDeviceSynchronize();
  }
  int h_st[2] = {0, 0};
  if (e == cudaSuccess) e = cudaMemcpy(h_st, st, sizeof(h_st), cudaMemcpyDeviceToHost);
  cudaFree(st);
  cudaFree(bar);
  if (e != cudaSuccess)
    return fail(nullptr, FW_ERR_CUDA, "self-test failed: %s", cudaGetErrorString(e));
  status_out[0] = h_st[0];
  status_out[1] = h_st[1];
  return FW_OK;
}

int fw_destroy(fw_handle* h) {
  if (!h) return FW_OK;
  {
    void* bufs[] = {h->adj_ckpt, h->adj_store, h->adj_store2, h->adj_lam, h->adj_grad, h->groups};
    for (void* b : bufs)
      if (b) cudaFree(b);
  }
  if (h->graph) cudaGraphExecDestroy(h->graph);
  if (h->capture_stream) cudaStreamDestroy(h->capture_stream);
  void* ptrs[] = {h->state, h->maps, h->dcmap, h->taps, h->icmat_t, h->traces, h->step, h->lists,
                  h->bar};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  delete h;
  return FW_OK;
}

const char* fw_last_error(const fw_handle* h) { return h ? h->err.c_str() : g_create_error.c_str(); }

}  // extern "C"

