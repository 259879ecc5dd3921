// Step launches of the engine library: the kernel family and shape of a handle -> kernel
// instantiations, the persistent cooperative launch, CUDA-graph capture of blocks of steps, and
// the TMA tensor maps the march kernels read through.
#include "engine_host.cuh"

namespace fwgbh {

// One time step: velocity kernel, then pressure kernel (+ tile epilogue), with the cell physics
// CV/CP (isotropic, anisotropic or exponential attenuation) of the handle.
template <int TY, int XC, class CV, class CP>
void launch_march2d(fw_handle* h, cudaStream_t s) {
  const int body_x = (int)h->nx - 2 * kGhost, body_y = (int)h->ny - 2 * kGhost;
  dim3 grid((body_y + TY - 1) / TY, (body_x + XC - 1) / XC);
  launch_k(vel2d_march<TY, XC, CV>, grid, dim3(TY), 0, s, h->args, h->tmaps2);
  launch_k(prs2d_march<TY, XC, CP>, grid, dim3(TY), 0, s, h->args, h->tmaps2);
}

// Streaming row march (isotropic engine): point-wise operands by TMA as well.
template <int TY, int XC, bool kBeta>
void launch_stream2d_shape(fw_handle* h, cudaStream_t s) {
  const int body_x = (int)h->nx - 2 * kGhost, body_y = (int)h->ny - 2 * kGhost;
  dim3 grid((body_y + TY - 1) / TY, (body_x + XC - 1) / XC);
  launch_k(vel2d_march<TY, XC, CellVelT<2, false>, true, kMRdtRho>, grid, dim3(TY), 0, s,
           h->args, h->tmaps2);
  launch_k(prs2d_march<TY, XC, CellPrsT<2, kBeta, false>, true, kBeta, kMDtK>, grid, dim3(TY), 0,
           s, h->args, h->tmaps2);
}

static_assert(kTileMapVel == kMRdtRho && kTileMapPrs == kMDtK && kTileMapBeta == kMBeta2dt &&
                  kTileMapAexp == kMAu1 && kTileMapGradY == kMaps && kTileMapDivY == kMaps + 5,
              "map slots read by the tile kernels");

// TMA tile kernels (2D, cell physics P): one 32 x 8 tile per block, operands staged by TMA.
template <int P, bool kBeta>
void launch_tile2d(fw_handle* h, cudaStream_t s) {
  const Tiling& t = h->tiling;
  const dim3 block(kD2TY, kD2TX);
  dim3 grid(t.n[1], t.n[0]);
  launch_k(vel2d_tile<P>, grid, block, sizeof(VelTileSmem<P>), s, h->args, h->tmaps_t, 0);
  launch_k(prs2d_tile<P, kBeta>, grid, block, sizeof(PrsTileSmem<P, kBeta>), s, h->args,
           h->tmaps_t, 0);
}

template <bool kBeta>
void launch_stream2d(fw_handle* h, cudaStream_t s) {
  switch (h->shape2d) {
    case 1: launch_stream2d_shape<64, 16, kBeta>(h, s); break;
    case 2: launch_stream2d_shape<64, 32, kBeta>(h, s); break;
    case 3: launch_stream2d_shape<128, 16, kBeta>(h, s); break;
    case 4: launch_stream2d_shape<128, 32, kBeta>(h, s); break;
    case 5: launch_stream2d_shape<128, 64, kBeta>(h, s); break;
    default: break;
  }
}

template <int ND, class CV, class CP, int kMin>
void launch_typed(fw_handle* h, cudaStream_t s) {
  const Tiling& t = h->tiling;
  if constexpr (ND == 2) {
    static_assert(kNumShapes2D == 8, "one case per 2D kernel shape");
    switch (h->shape2d) {
      case 0:
      case kTileShape:      // the tile shape is launched by launch_nd for every physics
      case kPersistentShape: {  // the persistent shape issues the direct kernels when captured
        dim3 grid(t.n[1], t.n[0]), block(kD2TY, kD2TX);
        launch_k(vel2d_direct<CV>, grid, block, 0, s, h->args);
        launch_k(prs2d_direct<CP>, grid, block, 0, s, h->args);
        break;
      }
      case 1: launch_march2d<64, 16, CV, CP>(h, s); break;
      case 2: launch_march2d<64, 32, CV, CP>(h, s); break;
      case 3: launch_march2d<128, 16, CV, CP>(h, s); break;
      case 4: launch_march2d<128, 32, CV, CP>(h, s); break;
      case 5: launch_march2d<128, 64, CV, CP>(h, s); break;
    }
  } else if (h->variant == kMarch) {
    dim3 grid(t.n[2], t.n[1], t.n[0]), block(kMTZ, kMTY);
    const MarchMaps& tm = h->tmaps;
    launch_k(vel3d_march<kMarchXC, CV, kMin>, grid, block, 0, s, h->args, tm.p);
    launch_k(prs3d_march<kMarchXC, CP, kMin>, grid, block, 0, s, h->args, tm.vx, tm.vy, tm.vz);
  } else {
    dim3 grid(t.n[2], t.n[1], t.n[0]), block(kD3TZ, kD3TY, kD3TX);
    launch_k(vel3d_direct<CV>, grid, block, 0, s, h->args);
    launch_k(prs3d_direct<CP>, grid, block, 0, s, h->args);
  }
}

// Streaming 3D kernels (isotropic engine): kPS-stage point-wise ring in dynamic shared memory,
// XC x planes per block.
template <int XC, int kPS, bool kBeta>
void launch_stream3d_ps(fw_handle* h, cudaStream_t s) {
  const Tiling& t = h->tiling;
  dim3 grid(t.n[2], t.n[1], t.n[0]), block(kMTZ, kMTY);
  const MarchMaps& tm = h->tmaps;
  const StreamMaps& sm = h->smaps;
  launch_k(vel3d_stream<XC, kPS, kMRdtRho>, grid, block, vel_stream_smem<kPS>(), s,
           h->args, tm.p, sm.vstate, sm.vmaps, sm.dcmap);
  launch_k(prs3d_stream<XC, kPS, kBeta, kMDtK>, grid, block, prs_stream_smem<kPS, kBeta>(), s,
           h->args, tm.vx, tm.vy, tm.vz, sm.pstate, sm.phi, kBeta ? sm.pmaps7 : sm.pmaps6,
           sm.dcmap);
}

template <bool kBeta>
void launch_stream3d(fw_handle* h, cudaStream_t s) {
  if (h->march_xc == kStreamXC) launch_stream3d_ps<kStreamXC, 2, kBeta>(h, s);
  else if (h->ps3d == 2) launch_stream3d_ps<kMarchXC, 2, kBeta>(h, s);
  else launch_stream3d_ps<kMarchXC, 3, kBeta>(h, s);
}

template <int ND, bool kBeta>
void launch_nd(fw_handle* h, cudaStream_t s) {
  if constexpr (ND == 2) {
    if (kShapes2D[h->shape2d].tile) {
      if (h->exp) launch_tile2d<kTileExp, kBeta>(h, s);
      else if (h->aniso) launch_tile2d<kTileAniso, kBeta>(h, s);
      else launch_tile2d<kTileIso, kBeta>(h, s);
      return;
    }
  }
  if (h->exp) {
    // the exponential engine is issue- and latency-bound (few bytes per cell): 4 blocks per SM
    // (64 registers) hide more latency than 3 (measured 58.7 vs 54.9 Gcell-updates/s, 656^3)
    launch_typed<ND, CellVelExpT<ND>, CellPrsExpT<ND, kBeta>, 4>(h, s);
  } else if (h->aniso) {
    launch_typed<ND, CellVelT<ND, true>, CellPrsT<ND, kBeta, true>, 2>(h, s);
  } else {
    if constexpr (ND == 3) {
      if (h->stream3d && h->variant == kMarch) {
        launch_stream3d<kBeta>(h, s);
        return;
      }
    } else {
      if (h->stream2d && kShapes2D[h->shape2d].ty > 0) {
        launch_stream2d<kBeta>(h, s);
        return;
      }
    }
    launch_typed<ND, CellVelT<ND, false>, CellPrsT<ND, kBeta, false>, 3>(h, s);
  }
}

void launch_step(fw_handle* h, cudaStream_t s) {
  if (h->ndim == 2) {
    if (h->has_beta) launch_nd<2, true>(h, s);
    else launch_nd<2, false>(h, s);
  } else {
    if (h->has_beta) launch_nd<3, true>(h, s);
    else launch_nd<3, false>(h, s);
  }
}

// Persistent 2D kernel: steps n0 .. n0 + n_steps - 1 in one cooperative launch. Each block owns
// an equal share of the 32 x 8 tiles; the grid is at most the co-resident block count.
template <class CV, class CP>
int launch_persistent_typed(fw_handle* h, cudaStream_t s, int n0, int n_steps) {
  auto kern = step2d_persistent<CV, CP>;
  int per_sm = 0, dev = 0, sms = 0;
  FW_CUDA(h, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kD2TY * kD2TX, 0));
  FW_CUDA(h, cudaGetDevice(&dev));
  FW_CUDA(h, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  int n_tiles = h->tiling.count(), n_ty = h->tiling.n[1];
  const int max_blocks = std::min(per_sm * sms, kBarMaxBlocks);
  if (max_blocks < 1) return fail(h, FW_ERR_CUDA, "persistent kernel: no block fits an SM");
  const int per_block = (n_tiles + max_blocks - 1) / max_blocks;
  const int grid = (n_tiles + per_block - 1) / per_block;
  if (!h->bar) FW_CUDA(h, cudaMalloc(&h->bar, kBarWords * sizeof(unsigned)));
  FW_CUDA(h, cudaMemsetAsync(h->bar, 0, kBarWords * sizeof(unsigned), s));
  void* args[] = {&h->args, &h->bar, &n0, &n_steps, &n_tiles, &n_ty};
  FW_CUDA(h, cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(kern), dim3(grid),
                                         dim3(kD2TY, kD2TX), args, 0, s));
  return FW_OK;
}

template <bool kBeta>
int launch_persistent_nd(fw_handle* h, cudaStream_t s, int n0, int n_steps) {
  if (h->exp)
    return launch_persistent_typed<CellVelExpT<2>, CellPrsExpT<2, kBeta>>(h, s, n0, n_steps);
  if (h->aniso)
    return launch_persistent_typed<CellVelT<2, true>, CellPrsT<2, kBeta, true>>(h, s, n0, n_steps);
  return launch_persistent_typed<CellVelT<2, false>, CellPrsT<2, kBeta, false>>(h, s, n0, n_steps);
}

int launch_persistent(fw_handle* h, cudaStream_t s, int n0, int n_steps) {
  if (n_steps <= 0) return FW_OK;
  return h->has_beta ? launch_persistent_nd<true>(h, s, n0, n_steps)
                     : launch_persistent_nd<false>(h, s, n0, n_steps);
}

int build_graph(fw_handle* h, int steps) {
  if (h->graph) {
    cudaGraphExecDestroy(h->graph);
    h->graph = nullptr;
  }
  cudaGraph_t graph = nullptr;
  FW_CUDA(h, cudaStreamBeginCapture(h->capture_stream, cudaStreamCaptureModeThreadLocal));
  for (int n = 0; n < steps; ++n) launch_step(h, h->capture_stream);
  cudaError_t e = cudaStreamEndCapture(h->capture_stream, &graph);
  if (e != cudaSuccess) return fail(h, FW_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(e));
  e = cudaGraphInstantiate(&h->graph, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return fail(h, FW_ERR_CUDA, "graph instantiate failed: %s", cudaGetErrorString(e));
  h->graph_steps = steps;
  return FW_OK;
}

using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                   const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                   const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                   CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// The driver's tensor-map encoder, looked up once per process (thread-safe static
// initialisation: handles are created from several threads, e.g. serving and gradient workers).
EncodeTiledFn tensor_map_encoder() {
  static const EncodeTiledFn fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    const cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                                           cudaEnableDefault, &q);
    return (e == cudaSuccess && p && q == cudaDriverEntryPointSuccess)
               ? reinterpret_cast<EncodeTiledFn>(p)
               : nullptr;
  }();
  return fn;
}

int encode_map(fw_handle* h, CUtensorMap* map, void* base, cuuint32_t rank,
               const cuuint64_t* dims, const cuuint64_t* strides, const cuuint32_t* box,
               CUtensorMapDataType type) {
  const EncodeTiledFn encode = tensor_map_encoder();
  if (!encode)
    return fail(h, FW_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
  const cuuint32_t estr[4] = {1, 1, 1, 1};
  CUresult r = encode(map, type, rank, base, dims, strides, box, estr,
                      CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                      CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(h, FW_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  return FW_OK;
}

// 4D float32 tensor map over a stack of padded 3D fields (the state or the map allocation):
// dims (pitch, ny, nx, n_fields), box (32, 8, 1, f): f consecutive fields of one plane tile.
int encode_stack_map(fw_handle* h, CUtensorMap* map, float* base, int n_fields, uint32_t f) {
  const cuuint64_t dims[4] = {(cuuint64_t)h->pitch, (cuuint64_t)h->ny, (cuuint64_t)h->nx,
                              (cuuint64_t)n_fields};
  const cuuint64_t strides[3] = {(cuuint64_t)h->pitch * 4, (cuuint64_t)(h->pitch * h->ny) * 4,
                                 (cuuint64_t)h->ncells_padded * 4};
  const cuuint32_t box[4] = {(cuuint32_t)kMTZ, (cuuint32_t)kMTY, 1, f};
  return encode_map(h, map, base, 4, dims, strides, box);
}

// Tensor maps of the streaming 3D kernels (state and map stacks, tap-index map).
int encode_stream_maps(fw_handle* h) {
  StreamMaps& m = h->smaps;
  const int ns = n_state(h->ndim), nm = n_maps(h);
  const cuuint64_t dims[3] = {(cuuint64_t)h->pitch, (cuuint64_t)h->ny, (cuuint64_t)h->nx};
  const cuuint64_t dc_strides[2] = {(cuuint64_t)h->pitch * 2, (cuuint64_t)(h->pitch * h->ny) * 2};
  const cuuint32_t box[3] = {(cuuint32_t)kMTZ, (cuuint32_t)kMTY, 1};
  int st;
  if ((st = encode_stack_map(h, &m.vstate, h->state, ns, kVelStateF)) ||
      (st = encode_stack_map(h, &m.vmaps, h->maps, nm, kVelMapF)) ||
      (st = encode_stack_map(h, &m.pstate, h->state, ns, 1)) ||
      (st = encode_stack_map(h, &m.phi, h->state, ns, kPrsPhiF)) ||
      (st = encode_stack_map(h, &m.pmaps6, h->maps, nm, kVelMapF)) ||
      (st = encode_stack_map(h, &m.pmaps7, h->maps, nm, kVelMapF + 1)) ||
      (st = encode_map(h, &m.dcmap, h->dcmap, 3, dims, dc_strides, box,
                       CU_TENSOR_MAP_DATA_TYPE_UINT16)))
    return st;
  return FW_OK;
}

// 3D float32 tensor map over one padded field: dims (pitch, ny, nx), box (bz, by, 1).
int encode_field_map(fw_handle* h, CUtensorMap* map, float* base, uint32_t bz, uint32_t by) {
  const cuuint64_t dims[3] = {(cuuint64_t)h->pitch, (cuuint64_t)h->ny, (cuuint64_t)h->nx};
  const cuuint64_t strides[2] = {(cuuint64_t)h->pitch * 4, (cuuint64_t)(h->pitch * h->ny) * 4};
  const cuuint32_t box[3] = {bz, by, 1};
  return encode_map(h, map, base, 3, dims, strides, box);
}

// 2D float32 tensor map over one padded 2D field: dims (pitch, nx), box (bw, 1) = one row segment.
int encode_row_map(fw_handle* h, CUtensorMap* map, float* base, uint32_t bw) {
  const cuuint64_t dims[2] = {(cuuint64_t)h->pitch, (cuuint64_t)h->nx};
  const cuuint64_t strides[1] = {(cuuint64_t)h->pitch * 4};
  const cuuint32_t box[2] = {bw, 1};
  return encode_map(h, map, base, 2, dims, strides, box);
}

// 3D float32 tensor map over a stack of padded 2D fields: dims (pitch, nx, n_fields), box
// (ty, 1, f): f consecutive fields of one row segment.
int encode_row_stack_map(fw_handle* h, CUtensorMap* map, float* base, int n_fields, uint32_t ty,
                         uint32_t f) {
  const cuuint64_t dims[3] = {(cuuint64_t)h->pitch, (cuuint64_t)h->nx, (cuuint64_t)n_fields};
  const cuuint64_t strides[2] = {(cuuint64_t)h->pitch * 4, (cuuint64_t)h->ncells_padded * 4};
  const cuuint32_t box[3] = {ty, 1, f};
  return encode_map(h, map, base, 3, dims, strides, box);
}

// Every tensor map of the 2D row march for block width ty (the point-wise ones only for the
// isotropic relaxation engine).
int encode_march2_maps(fw_handle* h, uint32_t ty, March2Maps* m) {
  int st;
  if ((st = encode_row_map(h, &m->p, h->args.f.p, ty + 16)) ||
      (st = encode_row_map(h, &m->vx, h->args.f.v[0], ty + 8)) ||
      (st = encode_row_map(h, &m->vy, h->args.f.v[1], ty + 16)))
    return st;
  if (h->aniso || h->exp) return FW_OK;
  const int ns = n_state(h->ndim), nm = n_maps(h);
  const cuuint64_t dims[2] = {(cuuint64_t)h->pitch, (cuuint64_t)h->nx};
  const cuuint64_t dc_strides[1] = {(cuuint64_t)h->pitch * 2};
  const cuuint32_t box[2] = {ty, 1};
  if ((st = encode_row_stack_map(h, &m->vst, h->state, ns, ty, kV2StateF)) ||
      (st = encode_row_stack_map(h, &m->vmp, h->maps, nm, ty, kV2MapF)) ||
      (st = encode_row_stack_map(h, &m->pp, h->state, ns, ty, 1)) ||
      (st = encode_row_stack_map(h, &m->phi, h->state, ns, ty, kP2PhiF)) ||
      (st = encode_row_stack_map(h, &m->pmp6, h->maps, nm, ty, kV2MapF)) ||
      (st = encode_row_stack_map(h, &m->pmp7, h->maps, nm, ty, kV2MapF + 1)) ||
      (st = encode_map(h, &m->dc, h->dcmap, 2, dims, dc_strides, box,
                       CU_TENSOR_MAP_DATA_TYPE_UINT16)))
    return st;
  return FW_OK;
}

// Select 2D kernel shape k: encode the row tensor maps for its width, drop the step graph.
// Tensor maps of the TMA tile kernels: the state stack (pitch, nx, 11) -- or, with slots > 0, a
// store of `slots` states at `store` (pitch, nx, 11, slots) --, the coefficient-map stack and the
// tap-index map.
int encode_tile2_maps(fw_handle* h, Tile2Maps* m, float* store, int slots) {
  const cuuint64_t row = (cuuint64_t)h->pitch * 4, field = (cuuint64_t)h->ncells_padded * 4;
  const cuuint64_t pitch = (cuuint64_t)h->pitch, nx = (cuuint64_t)h->nx;
  const int ns = n_state(h->ndim);
  const cuuint64_t d_st[4] = {pitch, nx, (cuuint64_t)ns, (cuuint64_t)slots};
  const cuuint64_t d_mp[3] = {pitch, nx, (cuuint64_t)n_maps(h)};
  const cuuint64_t str[3] = {row, field, field * ns};
  const cuuint64_t d_dc[2] = {pitch, nx};
  const cuuint64_t dc_str[1] = {(cuuint64_t)h->pitch * 2};
  const cuuint32_t bp[4] = {48, 24, 1, 1}, bx[4] = {40, 24, 1, 1}, by[4] = {48, 10, 1, 1};
  const cuuint32_t b1[4] = {kD2TY, kD2TX, 1, 1}, b2[4] = {kD2TY, kD2TX, 2, 1};
  const cuuint32_t b3[4] = {kD2TY, kD2TX, 3, 1}, b4[4] = {kD2TY, kD2TX, 4, 1};
  const cuuint32_t b5[4] = {kD2TY, kD2TX, 5, 1}, b6[4] = {kD2TY, kD2TX, 6, 1};
  const cuuint32_t bdc[2] = {kD2TY, kD2TX};
  float* base = slots > 0 ? store : h->state;
  const cuuint32_t r = slots > 0 ? 4 : 3;
  int st;
  if ((st = encode_map(h, &m->p_halo, base, r, d_st, str, bp)) ||
      (st = encode_map(h, &m->vx_halo, base, r, d_st, str, bx)) ||
      (st = encode_map(h, &m->vy_halo, base, r, d_st, str, by)) ||
      (st = encode_map(h, &m->st1, base, r, d_st, str, b1)) ||
      (st = encode_map(h, &m->st2, base, r, d_st, str, b2)) ||
      (st = encode_map(h, &m->st4, base, r, d_st, str, b4)) ||
      (st = encode_map(h, &m->st6, base, r, d_st, str, b6)) ||
      (st = encode_map(h, &m->mp1, h->maps, 3, d_mp, str, b1)) ||
      (st = encode_map(h, &m->mp3, h->maps, 3, d_mp, str, b3)) ||
      (st = encode_map(h, &m->mp5, h->maps, 3, d_mp, str, b5)) ||
      (st = encode_map(h, &m->mp6, h->maps, 3, d_mp, str, b6)) ||
      (st = encode_map(h, &m->dc, h->dcmap, 2, d_dc, dc_str, bdc, CU_TENSOR_MAP_DATA_TYPE_UINT16)))
    return st;
  return FW_OK;
}

int set_shape2d(fw_handle* h, int k) {
  if (kShapes2D[k].ty > 0) {
    int st = encode_march2_maps(h, (uint32_t)kShapes2D[k].ty, &h->tmaps2);
    if (st) return st;
  }
  const bool tile = kShapes2D[k].tile;
  if (tile) {
    int st = encode_tile2_maps(h, &h->tmaps_t, nullptr, 0);
    if (st) return st;
  }
  h->shape2d = k;
  h->variant = kShapes2D[k].persistent ? kPersistent : kShapes2D[k].ty > 0 ? kMarch
               : tile ? kTile : kDirect;
  h->graph_steps = 0;   // the next advance captures a graph with the new kernels
  return FW_OK;
}

// Allow the streaming kernels their dynamic shared memory (once per process; before any capture).
template <int XC, int kPS>
cudaError_t stream3d_attributes() {
  cudaError_t e;
  if ((e = cudaFuncSetAttribute(vel3d_stream<XC, kPS, kMRdtRho>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)vel_stream_smem<kPS>())) != cudaSuccess)
    return e;
  if ((e = cudaFuncSetAttribute(prs3d_stream<XC, kPS, false, kMDtK>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)prs_stream_smem<kPS, false>())) != cudaSuccess)
    return e;
  return cudaFuncSetAttribute(prs3d_stream<XC, kPS, true, kMDtK>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)prs_stream_smem<kPS, true>());
}

int prepare_stream3d(fw_handle* h) {
  static std::mutex mu;
  static std::vector<int> done;   // devices whose attributes are set
  int dev = 0;
  FW_CUDA(h, cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(mu);
  if (std::find(done.begin(), done.end(), dev) != done.end()) return FW_OK;
  cudaError_t e = stream3d_attributes<kStreamXC, 2>();
  if (e == cudaSuccess) e = stream3d_attributes<kMarchXC, 2>();
  if (e == cudaSuccess) e = stream3d_attributes<kMarchXC, 3>();
  if (e != cudaSuccess)
    return fail(h, FW_ERR_CUDA, "streaming 3D kernels: cudaFuncSetAttribute failed: %s",
                cudaGetErrorString(e));
  done.push_back(dev);
  return FW_OK;
}

}  // namespace fwgbh
