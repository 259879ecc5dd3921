// Host side of the discrete adjoint (2D and 3D): checkpointed forward pass and the reverse pass
// with per-segment recomputation (the C ABI's fw_adjoint_forward / fw_adjoint_backward).
#include "engine_host.cuh"
#include "kernels_adjoint_nd.cuh"

using namespace fwgbh;

namespace {

// Gradient maps of a handle: 12 (isotropic relaxation and exponential engines: the AdjGrad
// order), or 2 + 10 ND (anisotropic engine: one relaxation map set per derivative axis); then
// one more, 2 dt beta, when beta is not zero everywhere.
int n_grad_base(const fw_handle* h) { return h->aniso ? 2 + 10 * h->ndim : kNumGrad; }
int n_grad_maps(const fw_handle* h) { return n_grad_base(h) + (h->has_beta ? 1 : 0); }

// The reverse step's launches after lam_p is assembled, for the kernels with thread-loaded
// operands: every engine (isotropic and anisotropic relaxation, exponential attenuation), 2D
// and 3D, linear or nonlinear.
template <int ND, bool kF64, bool kS, bool kBeta>
void launch_reverse_thread(const fw_handle* h, const AdjArgs& A, dim3 g, dim3 b, size_t shm,
                           cudaStream_t s) {
  if (h->exp) {
    adjx_prs<ND, kF64, kS, kBeta><<<g, b, shm, s>>>(A);
    adjx_vel<ND, kF64, kS><<<g, b, shm, s>>>(A);
  } else if (h->aniso) {
    adja_prs<ND, kF64, kS, kBeta><<<g, b, shm, s>>>(A);
    adja_vel<ND, kF64, kS><<<g, b, shm, s>>>(A);
  } else if constexpr (ND == 3) {
    adj3d_prs<kF64, kS, kBeta><<<g, b, shm, s>>>(A);
    adj3d_vel<kF64, kS><<<g, b, shm, s>>>(A);
  } else {
    adj2d_prs<kF64, kS, kBeta><<<g, b, shm, s>>>(A);
    adj2d_vel<kF64, kS><<<g, b, shm, s>>>(A);
  }
}

template <int ND, bool kF64>
void launch_reverse_thread_nd(const fw_handle* h, const AdjArgs& A, bool smem_taps, dim3 g,
                              dim3 b, size_t shm, cudaStream_t s) {
  const int v = (smem_taps ? 2 : 0) + (h->has_beta ? 1 : 0);
  switch (v) {
    case 0: launch_reverse_thread<ND, kF64, false, false>(h, A, g, b, 0, s); break;
    case 1: launch_reverse_thread<ND, kF64, false, true>(h, A, g, b, 0, s); break;
    case 2: launch_reverse_thread<ND, kF64, true, false>(h, A, g, b, shm, s); break;
    default: launch_reverse_thread<ND, kF64, true, true>(h, A, g, b, shm, s); break;
  }
}

// Adjoint-field allocation of an ND handle, per padded cell array: lam_p, lam_v (ND),
// lam_psi (2 ND), lam_phi (2 ND), lam_d (ND), lam_g (ND), then the FP32 gradient partials.
// In 2D this is the layout the TMA reverse-step kernels address by constant field indices.
struct AdjLayout {
  int lam_v, lam_psi, lam_phi, lam_d, lam_g, fields, stack;
  AdjLayout(int nd, int n_grad)
      : lam_v(1), lam_psi(1 + nd), lam_phi(1 + 3 * nd), lam_d(1 + 5 * nd), lam_g(1 + 6 * nd),
        fields(1 + 7 * nd), stack(1 + 7 * nd + n_grad) {}
};
static_assert(1 + 2 == kAdjLamPsi && 1 + 6 == kAdjLamPhi && 1 + 10 == kAdjLamD &&
                  1 + 12 == kAdjLamG && 1 + 14 == kAdjFields,
              "2D adjoint-field layout of the TMA kernels");

static_assert(kAdjMapVel == kMRdtRho && kAdjMapPrs == kMDtK, "map runs of the adjoint kernels");

// Field of each gradient partial (AdjGrad order) in the adjoint allocation: coefficient-map order
// after the adjoint fields, so each TMA kernel reads its six partials as one run.
constexpr int kGradSlot[kNumGrad] = {kMRdtRho, kMDtK, kMInvKu, kMInvKx, kMAu1, kMBu1,
                                     kMAu2,    kMBu2, kMAx1,   kMBx1,   kMAx2, kMBx2};

// Tensor maps of the TMA reverse-step kernels over this handle's adjoint fields, coefficient
// maps, state store (K + 1 slots) and tap-index map.
int encode_adj_maps(fw_handle* h, AdjMaps* M, float* store) {
  const cuuint64_t row = (cuuint64_t)h->pitch * 4, field = (cuuint64_t)h->ncells_padded * 4;
  const cuuint64_t pitch = (cuuint64_t)h->pitch, nx = (cuuint64_t)h->nx;
  const cuuint64_t d_lam[3] = {pitch, nx, (cuuint64_t)kAdjStack};
  const cuuint64_t d_map[3] = {pitch, nx, (cuuint64_t)n_maps(h)};
  const cuuint64_t s3[2] = {row, field};
  const int ns = n_state(h->ndim);
  const cuuint64_t d_st[4] = {pitch, nx, (cuuint64_t)ns, (cuuint64_t)h->adj_every + 1};
  const cuuint64_t s4[3] = {row, field, field * ns};
  const cuuint64_t d_dc[2] = {pitch, nx};
  const cuuint64_t s_dc[1] = {(cuuint64_t)h->pitch * 2};
  const cuuint32_t b1[3] = {kD2TY, kD2TX, 1}, b4[3] = {kD2TY, kD2TX, 4}, b6[3] = {kD2TY, kD2TX, 6};
  const cuuint32_t bhx[3] = {kHXW, kHXR, 1}, bhy[3] = {kHYW, kHYR, 1};
  const cuuint32_t bs4[4] = {kD2TY, kD2TX, 4, 1}, bsx[4] = {kHXW, kHXR, 1, 1};
  const cuuint32_t bsy[4] = {kHYW, kHYR, 1, 1}, bsp[4] = {kHFW, kHFR, 1, 1};
  const cuuint32_t bdc[2] = {kHFW, kHFR};
  int st;
  if ((st = encode_map(h, &M->lam1, h->adj_lam, 3, d_lam, s3, b1)) ||
      (st = encode_map(h, &M->lam4, h->adj_lam, 3, d_lam, s3, b4)) ||
      (st = encode_map(h, &M->lam6, h->adj_lam, 3, d_lam, s3, b6)) ||
      (st = encode_map(h, &M->halo_x, h->adj_lam, 3, d_lam, s3, bhx)) ||
      (st = encode_map(h, &M->halo_y, h->adj_lam, 3, d_lam, s3, bhy)) ||
      (st = encode_map(h, &M->maps6, h->maps, 3, d_map, s3, b6)) ||
      (st = encode_map(h, &M->st4, store, 4, d_st, s4, bs4)) ||
      (st = encode_map(h, &M->st_vx, store, 4, d_st, s4, bsx)) ||
      (st = encode_map(h, &M->st_vy, store, 4, d_st, s4, bsy)) ||
      (st = encode_map(h, &M->st_p, store, 4, d_st, s4, bsp)) ||
      (st = encode_map(h, &M->dc, h->dcmap, 2, d_dc, s_dc, bdc, CU_TENSOR_MAP_DATA_TYPE_UINT16)))
    return st;
  return FW_OK;
}

// Allow the TMA reverse-step kernels the device's whole opt-in shared memory, once per device.
// Handles with different tap-table sizes run concurrently (gradient workers on their own
// streams), so the limit is not set per call: a smaller per-call value set by one thread would
// make another thread's larger launch invalid.
int prepare_adjoint_kernels(fw_handle* h, int dev, int smem_optin) {
  static std::mutex mu;
  static std::vector<int> done;
  std::lock_guard<std::mutex> lk(mu);
  if (std::find(done.begin(), done.end(), dev) != done.end()) return FW_OK;
  FW_CUDA(h, cudaFuncSetAttribute(adj2d_prs_tma<0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  smem_optin));
  FW_CUDA(h, cudaFuncSetAttribute(adj2d_vel_tma<0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  smem_optin));
  done.push_back(dev);
  return FW_OK;
}

// The FP64 gradient sums of the coefficient maps into the caller's dense
// [n][nx][ny] (2D) or [n][nx][ny][nz] (3D) buffer: rows of the last axis, unpadded.
int copy_gradients(fw_handle* h, const AdjArgs& A, double* grad_out, cudaStream_t s) {
  if (!grad_out) return FW_OK;
  const size_t width = h->ndim == 3 ? (size_t)h->nz : (size_t)h->ny;
  const size_t rows = h->ndim == 3 ? (size_t)h->nx * h->ny : (size_t)h->nx;
  for (int q = 0; q < A.n_grad; ++q)
    FW_CUDA(h, cudaMemcpy2DAsync(grad_out + (size_t)q * rows * width, width * sizeof(double),
                                 A.grad[q], h->pitch * sizeof(double), width * sizeof(double),
                                 rows, cudaMemcpyDeviceToDevice, s));
  return FW_OK;
}

// Free the adjoint buffers of h (checkpoints, state store, adjoint fields, gradient sums).
void release_adjoint(fw_handle* h) {
  void* bufs[] = {h->adj_ckpt, h->adj_store, h->adj_store2, h->adj_lam, h->adj_grad};
  for (void* b : bufs)
    if (b) cudaFree(b);
  h->adj_ckpt = h->adj_store = h->adj_store2 = h->adj_lam = nullptr;
  h->adj_grad = nullptr;
  h->bytes -= h->adj_bytes;
  h->adj_bytes = 0;
  h->adj_every = h->adj_nckpt = h->adj_ngrad = 0;
}

}  // namespace

extern "C" {

int fw_adjoint_forward(fw_handle* h, void* stream, int32_t checkpoint_every) {
  if (!h) return fail(nullptr, FW_ERR_ARGUMENT, "handle is NULL");
  if (!h->fields_set) return fail(h, FW_ERR_STATE, "fw_set_fields must be called first");
  if (h->args.l.rec_group)   // the misfit is defined on individual sensor traces
    return fail(h, FW_ERR_UNSUPPORTED, "the adjoint needs individual sensor traces: clear the sensor groups");
  if (checkpoint_every < 1) return fail(h, FW_ERR_ARGUMENT, "checkpoint_every must be >= 1");
  const size_t state_elems = (size_t)h->ncells_padded * n_state(h->ndim);
  const int nckpt = (h->d.nt + checkpoint_every - 1) / checkpoint_every;
  // (re)allocate when the checkpointing or the number of gradient maps (beta set or cleared by
  // fw_set_fields since the last call) changes
  if (checkpoint_every != h->adj_every || nckpt != h->adj_nckpt || n_grad_maps(h) != h->adj_ngrad) {
    release_adjoint(h);
    const size_t b_ckpt = state_elems * std::max(nckpt, 1) * sizeof(float);
    const size_t b_store = state_elems * (checkpoint_every + 1) * sizeof(float);
    // adjoint fields and temporaries (15 in 2D, 22 in 3D), then the FP32 segment partials
    const size_t b_lam = (size_t)h->ncells_padded * AdjLayout(h->ndim, n_grad_maps(h)).stack *
                         sizeof(float);
    const size_t b_grad = (size_t)h->ncells_padded * n_grad_maps(h) * sizeof(double);
    // FWGB_ADJ_OVERLAP=0: one state store, segments recomputed and reversed one after another
    // (always so in 3D, whose recomputation runs in place on the handle's own state)
    const char* ov = std::getenv("FWGB_ADJ_OVERLAP");
    const bool two = h->ndim == 2 && !(ov && std::strcmp(ov, "0") == 0);
    cudaError_t e = cudaMalloc(&h->adj_ckpt, b_ckpt);
    if (e == cudaSuccess) e = cudaMalloc(&h->adj_store, b_store);
    if (e == cudaSuccess && two) e = cudaMalloc(&h->adj_store2, b_store);
    // the out-of-place recomputation never writes the ghost layer of a stored state: keep it zero
    if (e == cudaSuccess) e = cudaMemset(h->adj_store, 0, b_store);
    if (e == cudaSuccess && two) e = cudaMemset(h->adj_store2, 0, b_store);
    if (e == cudaSuccess) e = cudaMalloc(&h->adj_lam, b_lam);
    if (e == cudaSuccess) e = cudaMalloc(&h->adj_grad, b_grad);
    if (e != cudaSuccess) {   // leave no partial allocation behind
      release_adjoint(h);
      return fail(h, e == cudaErrorMemoryAllocation ? FW_ERR_OOM : FW_ERR_CUDA,
                  "adjoint buffers (%zu bytes): %s", b_ckpt + (two ? 2 : 1) * b_store + b_lam + b_grad,
                  cudaGetErrorString(e));
    }
    h->adj_bytes = b_ckpt + (two ? 2 : 1) * b_store + b_lam + b_grad;
    h->bytes += h->adj_bytes;
    h->adj_every = checkpoint_every;
    h->adj_nckpt = nckpt;
    h->adj_ngrad = n_grad_maps(h);
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int st = fw_reset(h, stream);
  if (st) return st;
  for (int seg = 0; seg < nckpt; ++seg) {
    FW_CUDA(h, cudaMemcpyAsync(h->adj_ckpt + state_elems * seg, h->state, state_elems * sizeof(float),
                               cudaMemcpyDeviceToDevice, s));
    const int n = std::min(checkpoint_every, h->d.nt - seg * checkpoint_every);
    if ((st = fw_advance(h, stream, n))) return st;
  }
  return FW_OK;
}

int fw_adjoint_backward(fw_handle* h, void* stream, const float* residual, double* grad_out) {
  if (!h) return fail(nullptr, FW_ERR_ARGUMENT, "handle is NULL");
  if (!h->adj_ckpt || h->host_step != h->d.nt)
    return fail(h, FW_ERR_STATE, "fw_adjoint_forward must run (to nt) before fw_adjoint_backward");
  if (n_grad_maps(h) != h->adj_ngrad)
    return fail(h, FW_ERR_STATE, "the fields changed since fw_adjoint_forward: run it again");
  if (!residual && h->d.ncoordsout) return fail(h, FW_ERR_ARGUMENT, "residual is NULL");
  if (h->args.l.rec_group)
    return fail(h, FW_ERR_UNSUPPORTED, "the adjoint needs individual sensor traces: clear the sensor groups");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int64_t fs = h->ncells_padded;
  const size_t state_elems = (size_t)fs * n_state(h->ndim);
  const int n_grad = n_grad_maps(h);
  const AdjLayout lay(h->ndim, n_grad);
  FW_CUDA(h, cudaMemsetAsync(h->adj_lam, 0, (size_t)fs * lay.stack * sizeof(float), s));
  FW_CUDA(h, cudaMemsetAsync(h->adj_grad, 0, (size_t)fs * n_grad * sizeof(double), s));
  AdjArgs A{};
  A.g = h->args.g;
  A.m = h->args.m;
  A.fs = fs;
  A.lam_p = h->adj_lam;
  for (int a = 0; a < h->ndim; ++a) {
    A.lam_v[a] = h->adj_lam + (lay.lam_v + a) * fs;
    for (int nu = 0; nu < 2; ++nu) {
      A.lam_psi[a][nu] = h->adj_lam + (lay.lam_psi + 2 * a + nu) * fs;
      A.lam_phi[a][nu] = h->adj_lam + (lay.lam_phi + 2 * a + nu) * fs;
    }
    A.lam_d[a] = h->adj_lam + (lay.lam_d + a) * fs;
    A.lam_g[a] = h->adj_lam + (lay.lam_g + a) * fs;
  }
  A.n_grad = n_grad;
  A.beta_slot = h->has_beta ? n_grad_base(h) : -1;
  for (int q = 0; q < n_grad; ++q) {
    A.grad[q] = h->adj_grad + (size_t)q * fs;
    // isotropic maps: partials in coefficient-map order (the TMA kernels read runs of six);
    // 2 dt beta after them (its map slot, kMBeta2dt, is 12)
    const int slot = h->aniso || q >= kNumGrad ? q : kGradSlot[q];
    A.g32[q] = h->adj_lam + (size_t)(lay.fields + slot) * fs;
  }
  A.ndmap = h->d.ndmap;
  A.status = h->step + 1;
  // the tap table goes to shared memory when it fits next to the tiled kernels' static tiles
  // (11 KB) within the default 48 KB per block (up to 682 tap sets)
  const size_t tap_bytes = (size_t)h->d.ndmap * kTapStride * sizeof(float);
  const bool smem_taps = tap_bytes <= 32 * 1024;
  // FWGB_ADJ_FUSED=0: the five-launch reverse step (assemble, record, projections, pressure,
  // velocity) instead of the two tiled launches
  const char* fenv = std::getenv("FWGB_ADJ_FUSED");
  const bool fused = !(fenv && std::strcmp(fenv, "0") == 0) && !h->has_beta;
  const size_t sm = smem_taps ? tap_bytes : 0;
  // FWGB_ADJ_F64_STEPS=1: form and add every step's contributions in FP64 (slow on GB300's FP64
  // pipe; kept to validate the default segmented FP32-partial / FP64-total accumulation)
  const char* f64env = std::getenv("FWGB_ADJ_F64_STEPS");
  const bool f64_steps = f64env && std::strcmp(f64env, "1") == 0;
  // Default reverse step: the TMA-staged kernels (FP32 partials; the tap table goes to shared
  // memory with the tiles when it fits the per-block limit). FWGB_ADJ_TMA=0: the tiled kernels.
  const char* tenv = std::getenv("FWGB_ADJ_TMA");
  int dev = 0, smem_optin = 0;
  FW_CUDA(h, cudaGetDevice(&dev));
  FW_CUDA(h, cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  const size_t smem_prs = adj_prs_tma_smem(h->d.ndmap), smem_vel = adj_vel_tma_smem(h->d.ndmap);
  const bool tma = h->ndim == 2 && !h->exp && !h->aniso && fused && !f64_steps &&
                   !(tenv && std::strcmp(tenv, "0") == 0) &&
                   std::max(smem_prs, smem_vel) <= (size_t)smem_optin;
  // Recomputation: out of place from one stored state into the next (the TMA tile step kernels
  // reading slot n and writing slot n + 1), unless pressure is written in the ghost layer (it
  // persists there in place) or FWGB_ADJ_OOP=0: then a copy of the state into the store before
  // each in-place step.
  const char* oenv = std::getenv("FWGB_ADJ_OOP");
  const bool oop = h->ndim == 2 && !h->exp && !h->aniso && !h->has_beta && !h->ghost_writes &&
                   !(oenv && std::strcmp(oenv, "0") == 0);
  // Overlap (default when a second store exists, with out-of-place recomputation and the TMA
  // reverse step): segment k-1 is recomputed on a second stream into the other store while
  // segment k is reversed on `stream`; events order each store's reuse. Same kernels, same
  // operands: the gradient is bitwise that of the sequential pass.
  const bool overlap = oop && tma && h->adj_store2 != nullptr;
  float* stores[2] = {h->adj_store, overlap ? h->adj_store2 : h->adj_store};
  Tile2Maps MT[2] = {};
  AdjMaps M[2] = {};
  for (int b = 0; b < (overlap ? 2 : 1); ++b) {
    int st = FW_OK;
    if (oop) st = encode_tile2_maps(h, &MT[b], stores[b], h->adj_every + 1);
    if (!st && tma) st = encode_adj_maps(h, &M[b], stores[b]);
    if (st) return st;
  }
  if (tma) {
    int st = prepare_adjoint_kernels(h, dev, smem_optin);
    if (st) return st;
  }
  const Lists& L = h->args.l;
  // list lengths: sources after de-duplication, air cells, sensors
  int32_t counts[3] = {0, 0, 0};
  {
    const int nt_tiles = h->tiling.count();
    FW_CUDA(h, cudaMemcpy(&counts[0], L.src_ptr + nt_tiles, sizeof(int32_t), cudaMemcpyDeviceToHost));
    FW_CUDA(h, cudaMemcpy(&counts[1], L.zero_ptr + nt_tiles, sizeof(int32_t), cudaMemcpyDeviceToHost));
    FW_CUDA(h, cudaMemcpy(&counts[2], L.rec_ptr + nt_tiles, sizeof(int32_t), cudaMemcpyDeviceToHost));
  }
  const dim3 block(32, 8), grid((unsigned)((h->ny - 2 * kGhost + 31) / 32),
                                (unsigned)((h->nx - 2 * kGhost + 7) / 8));
  // 3D: one block per 32 (z) x 8 (y) cells of an x plane
  const dim3 block3(kA3TZ, kA3TY),
      grid3((unsigned)((h->nz - 2 * kGhost + kA3TZ - 1) / kA3TZ),
            (unsigned)((h->ny - 2 * kGhost + kA3TY - 1) / kA3TY), (unsigned)(h->nx - 2 * kGhost));
  const int K = h->adj_every;
  // recompute segment seg from its checkpoint into store b, keeping every state (out of place)
  auto recompute_oop = [&](int seg, int b, cudaStream_t rs) -> int {
    const int n0 = seg * K, n1 = std::min(n0 + K, (int)h->d.nt);
    set_step_counter<<<1, 1, 0, rs>>>(h->step, n0);
    FW_CUDA(h, cudaMemcpyAsync(stores[b], h->adj_ckpt + state_elems * seg,
                               state_elems * sizeof(float), cudaMemcpyDeviceToDevice, rs));
    StepArgs out = h->args;
    for (int n = n0; n < n1; ++n) {
      set_state_pointers(h, &out, stores[b] + state_elems * (n - n0 + 1));
      vel2d_tile<kTileIso, true><<<grid, block, sizeof(VelTileSmem<kTileIso>), rs>>>(
          out, MT[b], n - n0);
      prs2d_tile<kTileIso, false, true><<<grid, block, sizeof(PrsTileSmem<kTileIso, false>),
                                          rs>>>(out, MT[b], n - n0);
    }
    if (seg == 0)   // leave the first segment's recomputation in the handle, as in place
      FW_CUDA(h, cudaMemcpyAsync(h->state, stores[b] + state_elems * (n1 - n0),
                                 state_elems * sizeof(float), cudaMemcpyDeviceToDevice, rs));
    FW_CUDA(h, cudaGetLastError());
    return FW_OK;
  };
  if (overlap) {
    // i-th segment from the end -> store i % 2; the recomputation of segment i + 1 runs on the
    // second stream while segment i is reversed on `stream`
    cudaStream_t rs = nullptr;
    cudaEvent_t ev[5] = {};   // start, recomputed[2], reversed[2]
    auto cleanup = [&]() {
      for (cudaEvent_t e : ev)
        if (e) cudaEventDestroy(e);
      if (rs) cudaStreamDestroy(rs);
    };
    auto run = [&]() -> int {
      FW_CUDA(h, cudaStreamCreateWithFlags(&rs, cudaStreamNonBlocking));
      for (cudaEvent_t& e : ev) FW_CUDA(h, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
      cudaEvent_t ev_start = ev[0], *rec = ev + 1, *rev = ev + 3;
      FW_CUDA(h, cudaEventRecord(ev_start, s));
      FW_CUDA(h, cudaStreamWaitEvent(rs, ev_start, 0));
      const int nseg = h->adj_nckpt;
      int st;
      if ((st = recompute_oop(nseg - 1, 0, rs))) return st;
      FW_CUDA(h, cudaEventRecord(rec[0], rs));
      for (int i = 0; i < nseg; ++i) {
        const int seg = nseg - 1 - i, b = i % 2;
        if (i + 1 < nseg) {
          if (i >= 1) FW_CUDA(h, cudaStreamWaitEvent(rs, rev[(i + 1) % 2], 0));
          if ((st = recompute_oop(seg - 1, (i + 1) % 2, rs))) return st;
          FW_CUDA(h, cudaEventRecord(rec[(i + 1) % 2], rs));
        }
        FW_CUDA(h, cudaStreamWaitEvent(s, rec[b], 0));
        const int n0 = seg * K, n1 = std::min(n0 + K, (int)h->d.nt);
        for (int n = n1 - 1; n >= n0; --n) {
          A.Sn = stores[b] + state_elems * (n - n0);
          A.Sn1 = stores[b] + state_elems * (n - n0 + 1);
          adj2d_prs_tma<0><<<grid, block, smem_prs, s>>>(A, L, residual, n, n - n0, M[b]);
          adj2d_vel_tma<0><<<grid, block, smem_vel, s>>>(A, n - n0, M[b]);
        }
        adj2d_merge<<<grid, block, 0, s>>>(A);
        FW_CUDA(h, cudaGetLastError());
        FW_CUDA(h, cudaEventRecord(rev[b], s));
      }
      return FW_OK;
    };
    const int st = run();
    if (st) {
      cudaStreamSynchronize(s);
      if (rs) cudaStreamSynchronize(rs);
      cleanup();
      return st;
    }
    // every operation of the second stream precedes an event `stream` waited on, so the status
    // check (a synchronisation of `stream`) also covers it
    const int st2 = copy_gradients(h, A, grad_out, s);
    const int st3 = st2 ? st2 : check_device_status(h, s);
    cleanup();
    return st3;
  }
  bool first = true;
  for (int seg = h->adj_nckpt - 1; seg >= 0; --seg) {
    const int n0 = seg * K, n1 = std::min(n0 + K, (int)h->d.nt);
    // recompute the segment from its checkpoint, keeping every state
    if (oop) {
      int st = recompute_oop(seg, 0, s);
      if (st) return st;
    } else {
      set_step_counter<<<1, 1, 0, s>>>(h->step, n0);
      FW_CUDA(h, cudaMemcpyAsync(h->state, h->adj_ckpt + state_elems * seg,
                                 state_elems * sizeof(float), cudaMemcpyDeviceToDevice, s));
      for (int n = n0; n < n1; ++n) {
        FW_CUDA(h, cudaMemcpyAsync(h->adj_store + state_elems * (n - n0), h->state,
                                   state_elems * sizeof(float), cudaMemcpyDeviceToDevice, s));
        launch_step(h, s);
      }
      FW_CUDA(h, cudaMemcpyAsync(h->adj_store + state_elems * (n1 - n0), h->state,
                                 state_elems * sizeof(float), cudaMemcpyDeviceToDevice, s));
    }
    for (int n = n1 - 1; n >= n0; --n) {
      A.Sn = h->adj_store + state_elems * (n - n0);
      A.Sn1 = h->adj_store + state_elems * (n - n0 + 1);
      if (h->ndim == 3 || h->exp || h->aniso || !fused) {   // thread-load kernels, any engine
        const bool d3 = h->ndim == 3;
        const dim3 gx = d3 ? grid3 : grid, bx = d3 ? block3 : block;
        const size_t shm = smem_taps ? sm : 0;
        if (!first) {
          if (d3 && smem_taps) adj3d_assemble<true><<<gx, bx, shm, s>>>(A);
          else if (d3) adj3d_assemble<false><<<gx, bx, 0, s>>>(A);
          else if (smem_taps) adj2d_assemble<true><<<gx, bx, shm, s>>>(A);
          else adj2d_assemble<false><<<gx, bx, 0, s>>>(A);
        }
        first = false;
        if (counts[2]) adj2d_io<<<(counts[2] + 255) / 256, 256, 0, s>>>(A, L, residual, n, 0, 0, counts[2]);
        if (counts[0] || counts[1])
          adj2d_zero<<<(std::max(counts[0], counts[1]) + 255) / 256, 256, 0, s>>>(A, L, n, counts[0], counts[1]);
        if (d3 && f64_steps) launch_reverse_thread_nd<3, true>(h, A, smem_taps, gx, bx, shm, s);
        else if (d3) launch_reverse_thread_nd<3, false>(h, A, smem_taps, gx, bx, shm, s);
        else if (f64_steps) launch_reverse_thread_nd<2, true>(h, A, smem_taps, gx, bx, shm, s);
        else launch_reverse_thread_nd<2, false>(h, A, smem_taps, gx, bx, shm, s);
        continue;
      }
      if (tma) {
        adj2d_prs_tma<0><<<grid, block, smem_prs, s>>>(A, L, residual, n, n - n0, M[0]);
        adj2d_vel_tma<0><<<grid, block, smem_vel, s>>>(A, n - n0, M[0]);
        continue;
      }
      // 2D isotropic linear engine, tiled thread-load form (FWGB_ADJ_TMA=0)
      if (f64_steps && smem_taps) {
        adj2d_prs_fused<true, true><<<grid, block, sm, s>>>(A, L, residual, n);
        adj2d_vel_tiled<true, true><<<grid, block, sm, s>>>(A);
      } else if (f64_steps) {
        adj2d_prs_fused<true, false><<<grid, block, 0, s>>>(A, L, residual, n);
        adj2d_vel_tiled<true, false><<<grid, block, 0, s>>>(A);
      } else if (smem_taps) {
        adj2d_prs_fused<false, true><<<grid, block, sm, s>>>(A, L, residual, n);
        adj2d_vel_tiled<false, true><<<grid, block, sm, s>>>(A);
      } else {
        adj2d_prs_fused<false, false><<<grid, block, 0, s>>>(A, L, residual, n);
        adj2d_vel_tiled<false, false><<<grid, block, 0, s>>>(A);
      }
    }
    if (!f64_steps) {
      if (h->ndim == 3) adj3d_merge<<<grid3, block3, 0, s>>>(A);
      else adj2d_merge<<<grid, block, 0, s>>>(A);
    }
    FW_CUDA(h, cudaGetLastError());
  }
  const int st = copy_gradients(h, A, grad_out, s);
  return st ? st : check_device_status(h, s);
}

}  // extern "C"
