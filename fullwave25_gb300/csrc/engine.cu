// Host side of the FDTD engine: the C ABI declared in include/fwgb.h.
//
// One handle owns the device memory of one simulation: padded state and map arrays, the tap
// table, per-tile source/air/sensor lists and the trace buffer. Time steps are issued as two
// kernels per step (velocity, then pressure + tile epilogue); blocks of steps are captured once
// into a CUDA graph and replayed, so the per-step host cost is one graph launch per block.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <array>
#include <map>
#include <mutex>
#include <new>
#include <string>
#include <utility>
#include <vector>

#include "../../include/fwgb.h"
#include "engine_common.cuh"
#include "kernels_direct.cuh"
#include "kernels_march3d.cuh"
#include "kernels_march2d.cuh"
#include "kernels_persistent2d.cuh"
#include "kernels_stream3d.cuh"
#include "kernels_adjoint2d.cuh"

using namespace fwgb;

namespace {

thread_local std::string g_create_error = "no error";

}  // namespace

// Handle-less error text shared with the other translation units of the library.
void fwgb_set_global_error(const char* msg) { g_create_error = msg; }

namespace {

constexpr int kMarchXC = 64;   // x planes per block of the 3D register-load plane march
constexpr int kStreamXC = 32;  // x planes per block of the streaming 3D march (default)

// 2D kernel shapes the autotuner chooses from: 0 = direct kernels (one block per 32 y x 8 x tile),
// 1-5 = row-march kernels with TY threads (y columns) walking XC rows (TY + 16 <= 256, the TMA box
// limit; TY a multiple of 32 and XC of 8, whole list tiles per block), 6 = the persistent kernel
// (direct bodies, one cooperative launch per block of steps, grid barriers between phases).
struct Shape2D { int ty, xc; bool persistent; };
constexpr Shape2D kShapes2D[] = {{0, 0, false},   {64, 16, false},  {64, 32, false},
                                 {128, 16, false}, {128, 32, false}, {128, 64, false},
                                 {0, 0, true}};
constexpr int kPersistentShape = 6;
constexpr int kNumShapes2D = sizeof(kShapes2D) / sizeof(kShapes2D[0]);
constexpr int kTuneSteps = 64;   // time steps per autotuning trial (one graph)

enum Variant { kDirect = 0, kMarch = 1, kPersistent = 2, kStream = 3 };

struct Tiling {
  int t[3];   // tile extent along x, y, z (z unused in 2D)
  int n[3];   // tiles along x, y, z
  int count() const { return n[0] * n[1] * n[2]; }
};

}  // namespace

struct fw_handle {
  fw_desc d{};
  int ndim = 0;
  int64_t nx = 0, ny = 0, nz = 1, pitch = 0;  // pitch = padded length of the last axis
  int64_t ncells_padded = 0;
  std::string err = "no error";
  // device memory
  float* state = nullptr;      // n_state padded arrays
  float* maps = nullptr;       // n_maps padded arrays
  int32_t* dcmap = nullptr;
  float* taps = nullptr;
  float* icmat_t = nullptr;    // [nt_ic][ncoords]
  float* traces = nullptr;     // [n_out][ncoordsout]
  int* step = nullptr;
  unsigned* bar = nullptr;     // persistent 2D kernel: grid-barrier words (kBarWords)
  void* lists = nullptr;       // one allocation for all per-tile lists
  std::vector<int32_t> rec_k_host;   // sensor index of each record entry (entry order)
  void* groups = nullptr;      // rec_group (int32) + rec_w (float) per record entry
  int32_t n_cols = 0;          // trace row length: ncoordsout, or n_groups with sensor groups
  size_t bytes = 0;
  bool has_beta = false, fields_set = false;
  bool aniso = false;          // per-axis relaxation maps (the anisotropic engine)
  bool exp = false;            // exponential-attenuation engine (n_relax = 0, map a_exp)
  int n_out = 0;
  int32_t host_step = 0;
  Tiling tiling{};
  StepArgs args{};
  cudaStream_t capture_stream = nullptr;
  cudaGraphExec_t graph = nullptr;
  int graph_steps = 0;
  int variant = kDirect;
  int shape2d = 0;             // index into kShapes2D (2D handles)
  bool shape_fixed = false;    // 2D shape forced (FWGB_SHAPE2D / FWGB_VARIANT) or already tuned
  MarchMaps tmaps{};
  March2Maps tmaps2{};
  bool stream2d = false;       // 2D isotropic row march: point-wise operands staged by TMA too
  StreamMaps smaps{};
  bool stream3d = false;       // 3D isotropic: point-wise operands staged by TMA too
  int ps3d = 2;                // stages of the point-wise ring of the streaming kernels
  int march_xc = kMarchXC;     // x planes per block of the 3D march (streaming: kStreamXC)
  // adjoint (2D): checkpoints every adj_every steps, per-segment state store, adjoint fields
  int adj_every = 0, adj_nckpt = 0;
  float* adj_ckpt = nullptr;     // adj_nckpt states
  float* adj_store = nullptr;    // adj_every + 1 states
  float* adj_lam = nullptr;      // 11 adjoint fields + 4 temporaries
  double* adj_grad = nullptr;    // kNumGrad padded FP64 arrays
  size_t adj_bytes = 0;
};

namespace {

int fail(fw_handle* h, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (h) h->err = buf; else g_create_error = buf;
  return code;
}

#define FW_CUDA(h, call)                                                                   \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess)                                                                 \
      return fail(h, e_ == cudaErrorMemoryAllocation ? FW_ERR_OOM : FW_ERR_CUDA,           \
                  "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
  } while (0)

int64_t round_up(int64_t v, int64_t m) { return (v + m - 1) / m * m; }

int n_state(int ndim) { return 1 + ndim + 4 * ndim; }
// maps, in the order the streaming 3D kernels fetch them (one contiguous run per kernel):
// velocity rdt_rho inv_ku au1 bu1 au2 bu2 | pressure dt_k inv_kx ax1 bx1 ax2 bx2 | beta2dt
// (x axis, or every axis in the isotropic engine); then for the anisotropic engine per further
// axis a >= 1: inv_ku, au1 bu1 au2 bu2, inv_kx, ax1 bx1 ax2 bx2 at 13 + 10 (a - 1) + k
enum MapSlot {
  kMRdtRho = 0, kMInvKu, kMAu1, kMBu1, kMAu2, kMBu2,
  kMDtK, kMInvKx, kMAx1, kMBx1, kMAx2, kMBx2,
  kMBeta2dt
};
constexpr int kMaps = 13;
int n_maps(const fw_handle* h) { return kMaps + (h->aniso ? 10 * (h->ndim - 1) : 0); }
int axis_map(int a, int k) { return kMaps + 10 * (a - 1) + k; }

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
    const float r = rho_to_rdt[c];
    rho_to_rdt[c] = r != 0.f ? dt / r : 0.f;
    k_to_dtk[c] = dt * k_to_dtk[c];
    beta_to_2dt[c] = 2.f * dt * beta_to_2dt[c];
  }
}

__global__ void invert_map(float* kappa_to_inv, int64_t n) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n;
       c += (int64_t)gridDim.x * blockDim.x) {
    const float k = kappa_to_inv[c];
    kappa_to_inv[c] = k != 0.f ? 1.f / k : 0.f;
  }
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

float* state_field(fw_handle* h, int idx) { return h->state + (size_t)idx * h->ncells_padded; }
float* map_field(fw_handle* h, int idx) { return h->maps + (size_t)idx * h->ncells_padded; }

// Copy a dense C-order grid array (host or device) into a padded device array.
int upload_grid(fw_handle* h, void* dst, const void* src, size_t elem, bool on_device,
                cudaStream_t s) {
  const int64_t last = h->ndim == 2 ? h->ny : h->nz;
  const int64_t rows = h->ndim == 2 ? h->nx : h->nx * h->ny;
  FW_CUDA(h, cudaMemcpy2DAsync(dst, h->pitch * elem, src, last * elem, last * elem, rows,
                               on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s));
  return FW_OK;
}

// Time-step kernels are launched with programmatic dependent launch (FWGB_PDL=0 turns it off):
// each may be scheduled while the previous kernel of the stream drains, and waits for it on the
// device (pdl_entry). Captured into graphs as programmatic dependency edges.
bool pdl_enabled() {
  static const bool on = [] {
    const char* v = std::getenv("FWGB_PDL");
    return !(v && std::strcmp(v, "0") == 0);
  }();
  return on;
}

template <typename... KArgs, typename... Args>
void launch_k(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
              Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = pdl_enabled() ? 1 : 0;
  cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

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
    static_assert(kNumShapes2D == 7, "one case per 2D kernel shape");
    switch (h->shape2d) {
      case 0:
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
  if (h->exp) {
    launch_typed<ND, CellVelExpT<ND>, CellPrsExpT<ND, kBeta>, 3>(h, s);
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
  const int max_blocks = std::min(per_sm * sms, kBarGroup * kBarMaxGroups);
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

int encode_map(fw_handle* h, CUtensorMap* map, void* base, cuuint32_t rank,
               const cuuint64_t* dims, const cuuint64_t* strides, const cuuint32_t* box,
               CUtensorMapDataType type = CU_TENSOR_MAP_DATA_TYPE_FLOAT32) {
  static EncodeTiledFn encode = nullptr;
  if (!encode) {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q{};
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000,
                                                     cudaEnableDefault, &q);
    if (e != cudaSuccess || !fn || q != cudaDriverEntryPointSuccess)
      return fail(h, FW_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
    encode = reinterpret_cast<EncodeTiledFn>(fn);
  }
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
  const cuuint64_t strides[2] = {(cuuint64_t)h->pitch * 4, (cuuint64_t)(h->pitch * h->ny) * 4};
  const cuuint32_t box[3] = {(cuuint32_t)kMTZ, (cuuint32_t)kMTY, 1};
  int st;
  if ((st = encode_stack_map(h, &m.vstate, h->state, ns, kVelStateF)) ||
      (st = encode_stack_map(h, &m.vmaps, h->maps, nm, kVelMapF)) ||
      (st = encode_stack_map(h, &m.pstate, h->state, ns, 1)) ||
      (st = encode_stack_map(h, &m.phi, h->state, ns, kPrsPhiF)) ||
      (st = encode_stack_map(h, &m.pmaps6, h->maps, nm, kVelMapF)) ||
      (st = encode_stack_map(h, &m.pmaps7, h->maps, nm, kVelMapF + 1)) ||
      (st = encode_map(h, &m.dcmap, h->dcmap, 3, dims, strides, box, CU_TENSOR_MAP_DATA_TYPE_INT32)))
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
  const cuuint64_t strides[1] = {(cuuint64_t)h->pitch * 4};
  const cuuint32_t box[2] = {ty, 1};
  if ((st = encode_row_stack_map(h, &m->vst, h->state, ns, ty, kV2StateF)) ||
      (st = encode_row_stack_map(h, &m->vmp, h->maps, nm, ty, kV2MapF)) ||
      (st = encode_row_stack_map(h, &m->pp, h->state, ns, ty, 1)) ||
      (st = encode_row_stack_map(h, &m->phi, h->state, ns, ty, kP2PhiF)) ||
      (st = encode_row_stack_map(h, &m->pmp6, h->maps, nm, ty, kV2MapF)) ||
      (st = encode_row_stack_map(h, &m->pmp7, h->maps, nm, ty, kV2MapF + 1)) ||
      (st = encode_map(h, &m->dc, h->dcmap, 2, dims, strides, box, CU_TENSOR_MAP_DATA_TYPE_INT32)))
    return st;
  return FW_OK;
}

// Select 2D kernel shape k: encode the row tensor maps for its width, drop the step graph.
int set_shape2d(fw_handle* h, int k) {
  if (kShapes2D[k].ty > 0) {
    int st = encode_march2_maps(h, (uint32_t)kShapes2D[k].ty, &h->tmaps2);
    if (st) return st;
  }
  h->shape2d = k;
  h->variant = kShapes2D[k].persistent ? kPersistent : kShapes2D[k].ty > 0 ? kMarch : kDirect;
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

// Device status word (step buffer slot 1): non-zero if a kernel gave up on a bounded wait.
int check_device_status(fw_handle* h, cudaStream_t s) {
  int st = 0;
  FW_CUDA(h, cudaMemcpyAsync(&st, h->step + 1, sizeof(int), cudaMemcpyDeviceToHost, s));
  FW_CUDA(h, cudaStreamSynchronize(s));
  if (st) return fail(h, FW_ERR_DEVICE, "a kernel reported device status 0x%x (bounded wait timed out)", st);
  return FW_OK;
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
      (st = alloc((void**)&h->dcmap, cells * sizeof(int32_t))) ||
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
      cudaMemset(h->dcmap, 0, cells * sizeof(int32_t)) != cudaSuccess ||
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
  int s = 0;
  A.f.p = state_field(h, s++);
  for (int a = 0; a < 3; ++a) A.f.v[a] = a < h->ndim ? state_field(h, s++) : nullptr;
  for (int a = 0; a < 3; ++a)
    for (int nu = 0; nu < 2; ++nu) A.f.psi[a][nu] = a < h->ndim ? state_field(h, s++) : nullptr;
  for (int a = 0; a < 3; ++a)
    for (int nu = 0; nu < 2; ++nu) A.f.phi[a][nu] = a < h->ndim ? state_field(h, s++) : nullptr;
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
  if ((st = upload_grid(h, h->dcmap, dcm.data(), sizeof(int32_t), false, s))) return st;
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

int fw_adjoint_forward(fw_handle* h, void* stream, int32_t checkpoint_every) {
  if (!h) return fail(nullptr, FW_ERR_ARGUMENT, "handle is NULL");
  if (h->ndim != 2) return fail(h, FW_ERR_UNSUPPORTED, "the adjoint is implemented for 2D grids");
  if (h->has_beta) return fail(h, FW_ERR_UNSUPPORTED, "the adjoint needs beta = 0 everywhere");
  if (h->aniso || h->exp)
    return fail(h, FW_ERR_UNSUPPORTED, "the adjoint covers the isotropic relaxation engine");
  if (!h->fields_set) return fail(h, FW_ERR_STATE, "fw_set_fields must be called first");
  if (checkpoint_every < 1) return fail(h, FW_ERR_ARGUMENT, "checkpoint_every must be >= 1");
  const size_t state_elems = (size_t)h->ncells_padded * n_state(h->ndim);
  const int nckpt = (h->d.nt + checkpoint_every - 1) / checkpoint_every;
  if (checkpoint_every != h->adj_every || nckpt != h->adj_nckpt) {
    void* bufs[] = {h->adj_ckpt, h->adj_store, h->adj_lam, h->adj_grad};
    for (void* b : bufs)
      if (b) cudaFree(b);
    h->bytes -= h->adj_bytes;
    h->adj_ckpt = h->adj_store = h->adj_lam = nullptr;
    h->adj_grad = nullptr;
    const size_t b_ckpt = state_elems * std::max(nckpt, 1) * sizeof(float);
    const size_t b_store = state_elems * (checkpoint_every + 1) * sizeof(float);
    // 15 adjoint fields and temporaries, then the FP32 per-segment gradient partials
    const size_t b_lam = (size_t)h->ncells_padded * (15 + kNumGrad) * sizeof(float);
    const size_t b_grad = (size_t)h->ncells_padded * kNumGrad * sizeof(double);
    FW_CUDA(h, cudaMalloc(&h->adj_ckpt, b_ckpt));
    FW_CUDA(h, cudaMalloc(&h->adj_store, b_store));
    FW_CUDA(h, cudaMalloc(&h->adj_lam, b_lam));
    FW_CUDA(h, cudaMalloc(&h->adj_grad, b_grad));
    h->adj_bytes = b_ckpt + b_store + b_lam + b_grad;
    h->bytes += h->adj_bytes;
    h->adj_every = checkpoint_every;
    h->adj_nckpt = nckpt;
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
  if (!residual && h->d.ncoordsout) return fail(h, FW_ERR_ARGUMENT, "residual is NULL");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int64_t fs = h->ncells_padded;
  const size_t state_elems = (size_t)fs * n_state(h->ndim);
  FW_CUDA(h, cudaMemsetAsync(h->adj_lam, 0, (size_t)fs * (15 + kNumGrad) * sizeof(float), s));
  FW_CUDA(h, cudaMemsetAsync(h->adj_grad, 0, (size_t)fs * kNumGrad * sizeof(double), s));
  AdjArgs A{};
  A.g = h->args.g;
  A.m = h->args.m;
  A.fs = fs;
  A.lam_p = h->adj_lam;
  for (int a = 0; a < 2; ++a) {
    A.lam_v[a] = h->adj_lam + (1 + a) * fs;
    for (int nu = 0; nu < 2; ++nu) {
      A.lam_psi[a][nu] = h->adj_lam + (3 + 2 * a + nu) * fs;
      A.lam_phi[a][nu] = h->adj_lam + (7 + 2 * a + nu) * fs;
    }
    A.lam_d[a] = h->adj_lam + (11 + a) * fs;
    A.lam_g[a] = h->adj_lam + (13 + a) * fs;
  }
  for (int q = 0; q < kNumGrad; ++q) {
    A.grad[q] = h->adj_grad + (size_t)q * fs;
    A.g32[q] = h->adj_lam + (size_t)(15 + q) * fs;
  }
  A.ndmap = h->d.ndmap;
  // the tap table goes to shared memory when it fits next to the tiled kernels' static tiles
  // (11 KB) within the default 48 KB per block (up to 682 tap sets)
  const size_t tap_bytes = (size_t)h->d.ndmap * kTapStride * sizeof(float);
  const bool smem_taps = tap_bytes <= 32 * 1024;
  // FWGB_ADJ_FUSED=0: the five-launch reverse step (assemble, record, projections, pressure,
  // velocity) instead of the two tiled launches
  const char* fenv = std::getenv("FWGB_ADJ_FUSED");
  const bool fused = !(fenv && std::strcmp(fenv, "0") == 0);
  const size_t sm = smem_taps ? tap_bytes : 0;
  // FWGB_ADJ_F64_STEPS=1: form and add every step's contributions in FP64 (slow on GB300's FP64
  // pipe; kept to validate the default segmented FP32-partial / FP64-total accumulation)
  const char* f64env = std::getenv("FWGB_ADJ_F64_STEPS");
  const bool f64_steps = f64env && std::strcmp(f64env, "1") == 0;
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
  const int K = h->adj_every;
  bool first = true;
  for (int seg = h->adj_nckpt - 1; seg >= 0; --seg) {
    const int n0 = seg * K, n1 = std::min(n0 + K, (int)h->d.nt);
    // recompute the segment from its checkpoint, keeping every state
    FW_CUDA(h, cudaMemcpyAsync(h->state, h->adj_ckpt + state_elems * seg, state_elems * sizeof(float),
                               cudaMemcpyDeviceToDevice, s));
    set_step_counter<<<1, 1, 0, s>>>(h->step, n0);
    for (int n = n0; n < n1; ++n) {
      FW_CUDA(h, cudaMemcpyAsync(h->adj_store + state_elems * (n - n0), h->state,
                                 state_elems * sizeof(float), cudaMemcpyDeviceToDevice, s));
      launch_step(h, s);
    }
    FW_CUDA(h, cudaMemcpyAsync(h->adj_store + state_elems * (n1 - n0), h->state,
                               state_elems * sizeof(float), cudaMemcpyDeviceToDevice, s));
    for (int n = n1 - 1; n >= n0; --n) {
      A.Sn = h->adj_store + state_elems * (n - n0);
      A.Sn1 = h->adj_store + state_elems * (n - n0 + 1);
      if (fused) {
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
        continue;
      }
      if (!first) {
        if (smem_taps) adj2d_assemble<true><<<grid, block, sm, s>>>(A);
        else adj2d_assemble<false><<<grid, block, 0, s>>>(A);
      }
      first = false;
      if (counts[2]) adj2d_io<<<(counts[2] + 255) / 256, 256, 0, s>>>(A, L, residual, n, 0, 0, counts[2]);
      if (counts[0] || counts[1])
        adj2d_zero<<<(std::max(counts[0], counts[1]) + 255) / 256, 256, 0, s>>>(A, L, n, counts[0], counts[1]);
      if (f64_steps && smem_taps) {
        adj2d_prs<true, true><<<grid, block, sm, s>>>(A);
        adj2d_vel<true, true><<<grid, block, sm, s>>>(A);
      } else if (f64_steps) {
        adj2d_prs<true, false><<<grid, block, 0, s>>>(A);
        adj2d_vel<true, false><<<grid, block, 0, s>>>(A);
      } else if (smem_taps) {
        adj2d_prs<false, true><<<grid, block, sm, s>>>(A);
        adj2d_vel<false, true><<<grid, block, sm, s>>>(A);
      } else {
        adj2d_prs<false, false><<<grid, block, 0, s>>>(A);
        adj2d_vel<false, false><<<grid, block, 0, s>>>(A);
      }
    }
    if (!f64_steps) adj2d_merge<<<grid, block, 0, s>>>(A);
    FW_CUDA(h, cudaGetLastError());
  }
  if (grad_out) {
    for (int q = 0; q < kNumGrad; ++q)
      FW_CUDA(h, cudaMemcpy2DAsync(grad_out + (size_t)q * h->nx * h->ny, h->ny * sizeof(double),
                                   A.grad[q], h->pitch * sizeof(double), h->ny * sizeof(double),
                                   h->nx, cudaMemcpyDeviceToDevice, s));
  }
  return FW_OK;
}

int fw_destroy(fw_handle* h) {
  if (!h) return FW_OK;
  {
    void* bufs[] = {h->adj_ckpt, h->adj_store, h->adj_lam, h->adj_grad, h->groups};
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

// ------------------------------------------------------------------------------------- groups
struct fw_group {
  std::vector<fw_handle*> members;  // sorted by steps left, descending (tiles in the same order)
  StepArgs* d_args = nullptr;       // one argument block per member (its own step counter)
  // work list: direct kernels {member, tile_y, tile_x, tile index within the member};
  //            march kernels  {member, y block, x chunk, 1 for the block that counts the step}
  int4* d_tiles = nullptr;
  March2Maps* d_maps = nullptr;     // march kernels: one March2Maps per member
  bool stream = true;               // march kernels with TMA-staged point-wise operands
  size_t args_cap = 0, tiles_cap = 0;
  int shape = 0;                    // index into kShapes2D (0 = direct group kernels)
  bool shape_fixed = false;         // forced by the environment or already tuned
  std::vector<int> tiles_upto;      // tiles of the first k members (k = 0..n)
  bool beta = false;
  cudaStream_t capture_stream = nullptr;
  std::map<int, cudaGraphExec_t> graphs;  // active tile count -> graph of kGroupGraphSteps steps
};

namespace {

constexpr int kGroupGraphSteps = 64;

template <int TY, int XC, bool kStream>
void group_launch_march_t(fw_group* g, int n_blocks, cudaStream_t s) {
  const StepArgs* a = g->d_args;
  const March2Maps* m = g->d_maps;
  const int4* w = g->d_tiles;
  const dim3 grid(n_blocks), block(TY);
  launch_k(vel2d_march_group<TY, XC, kStream, kMRdtRho>, grid, block, 0, s, a, m, w);
  if (g->beta) launch_k(prs2d_march_group<TY, XC, true, kStream, kMDtK>, grid, block, 0, s, a, m, w);
  else launch_k(prs2d_march_group<TY, XC, false, kStream, kMDtK>, grid, block, 0, s, a, m, w);
}

template <int TY, int XC>
void group_launch_march(fw_group* g, int n_blocks, cudaStream_t s) {
  if (g->stream) group_launch_march_t<TY, XC, true>(g, n_blocks, s);
  else group_launch_march_t<TY, XC, false>(g, n_blocks, s);
}

void group_launch_step(fw_group* g, int n_tiles, cudaStream_t s) {
  static_assert(kNumShapes2D == 7, "one case per 2D kernel shape");
  switch (g->shape) {
    case 0: {
      const dim3 block(kD2TY, kD2TX);
      const StepArgs* a = g->d_args;
      const int4* w = g->d_tiles;
      launch_k(vel2d_group, dim3(n_tiles), block, 0, s, a, w);
      if (g->beta) launch_k(prs2d_group<true>, dim3(n_tiles), block, 0, s, a, w);
      else launch_k(prs2d_group<false>, dim3(n_tiles), block, 0, s, a, w);
      break;
    }
    case 1: group_launch_march<64, 16>(g, n_tiles, s); break;
    case 2: group_launch_march<64, 32>(g, n_tiles, s); break;
    case 3: group_launch_march<128, 16>(g, n_tiles, s); break;
    case 4: group_launch_march<128, 32>(g, n_tiles, s); break;
    case 5: group_launch_march<128, 64>(g, n_tiles, s); break;
    default: break;  // no persistent group kernel: group shapes are 0-5
  }
}

int group_graph(fw_group* g, int n_tiles, cudaGraphExec_t* out) {
  auto it = g->graphs.find(n_tiles);
  if (it != g->graphs.end()) {
    *out = it->second;
    return FW_OK;
  }
  cudaGraph_t graph = nullptr;
  FW_CUDA(nullptr, cudaStreamBeginCapture(g->capture_stream, cudaStreamCaptureModeThreadLocal));
  for (int n = 0; n < kGroupGraphSteps; ++n) group_launch_step(g, n_tiles, g->capture_stream);
  FW_CUDA(nullptr, cudaStreamEndCapture(g->capture_stream, &graph));
  cudaGraphExec_t exec = nullptr;
  cudaError_t e = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return fail(nullptr, FW_ERR_CUDA, "group graph: %s", cudaGetErrorString(e));
  g->graphs[n_tiles] = exec;
  *out = exec;
  return FW_OK;
}

// (Re)build the member order, argument blocks and tile work list of a group. Members are
// ordered by steps left (descending) so that, as members finish, the active tiles stay a prefix.
int group_set(fw_group* g, fw_handle* const* handles, int32_t n) {
  for (int i = 0; i < n; ++i) {
    const fw_handle* h = handles[i];
    if (!h) return fail(nullptr, FW_ERR_ARGUMENT, "handle %d is NULL", i);
    if (h->ndim != 2 || h->aniso || h->exp)
      return fail(nullptr, FW_ERR_UNSUPPORTED,
                  "group members must be isotropic 2D simulations (member %d)", i);
    if (!h->fields_set) return fail(nullptr, FW_ERR_STATE, "member %d has no fields set", i);
  }
  std::vector<fw_handle*> m(handles, handles + n);
  std::stable_sort(m.begin(), m.end(), [](const fw_handle* a, const fw_handle* b) {
    return a->d.nt - a->host_step > b->d.nt - b->host_step;
  });
  std::vector<StepArgs> args(n);
  std::vector<int4> tiles;
  std::vector<March2Maps> maps;
  g->members = m;
  g->tiles_upto.assign(1, 0);
  g->beta = false;
  for (int r = 0; r < n; ++r) g->beta = g->beta || m[r]->has_beta;
  for (int r = 0; r < n; ++r) {
    fw_handle* h = m[r];
    args[r] = h->args;
    // members without beta read their (all-zero) beta buffer when the group uses the beta kernel
    args[r].m.beta2dt = map_field(h, kMBeta2dt);
    if (g->shape == 0) {
      const Tiling& t = h->tiling;
      for (int tx = 0; tx < t.n[0]; ++tx)
        for (int ty = 0; ty < t.n[1]; ++ty) tiles.push_back(make_int4(r, ty, tx, tx * t.n[1] + ty));
    } else {
      const int ty_ = kShapes2D[g->shape].ty, xc = kShapes2D[g->shape].xc;
      const int nby = (int)(h->ny - 2 * kGhost + ty_ - 1) / ty_;
      const int nbx = (int)(h->nx - 2 * kGhost + xc - 1) / xc;
      for (int bx = 0; bx < nbx; ++bx)
        for (int by = 0; by < nby; ++by) tiles.push_back(make_int4(r, by, bx, bx == 0 && by == 0));
      March2Maps tm{};
      if (encode_march2_maps(h, (uint32_t)ty_, &tm))
        return fail(nullptr, FW_ERR_CUDA, "row tensor maps of member %d: %s", r, h->err.c_str());
      maps.push_back(tm);
    }
    g->tiles_upto.push_back((int)tiles.size());
  }
  if ((size_t)n > g->args_cap || tiles.size() > g->tiles_cap) {
    for (auto& kv : g->graphs) cudaGraphExecDestroy(kv.second);
    g->graphs.clear();
    if (g->d_args) cudaFree(g->d_args);
    if (g->d_tiles) cudaFree(g->d_tiles);
    if (g->d_maps) cudaFree(g->d_maps);
    g->d_args = nullptr;
    g->d_tiles = nullptr;
    g->d_maps = nullptr;
    g->args_cap = std::max<size_t>(n, 2 * g->args_cap);
    g->tiles_cap = std::max<size_t>(tiles.size(), 2 * g->tiles_cap);
    if (cudaMalloc(&g->d_args, sizeof(StepArgs) * g->args_cap) != cudaSuccess ||
        cudaMalloc(&g->d_tiles, sizeof(int4) * g->tiles_cap) != cudaSuccess ||
        cudaMalloc(&g->d_maps, sizeof(March2Maps) * g->args_cap) != cudaSuccess) {
      g->args_cap = g->tiles_cap = 0;
      return fail(nullptr, FW_ERR_OOM, "group device allocation failed");
    }
  }
  // graphs read the work list through stable pointers, so they stay valid across rebuilds
  FW_CUDA(nullptr, cudaMemcpyAsync(g->d_args, args.data(), sizeof(StepArgs) * n,
                                   cudaMemcpyHostToDevice, g->capture_stream));
  FW_CUDA(nullptr, cudaMemcpyAsync(g->d_tiles, tiles.data(), sizeof(int4) * tiles.size(),
                                   cudaMemcpyHostToDevice, g->capture_stream));
  if (!maps.empty())
    FW_CUDA(nullptr, cudaMemcpyAsync(g->d_maps, maps.data(), sizeof(March2Maps) * maps.size(),
                                     cudaMemcpyHostToDevice, g->capture_stream));
  FW_CUDA(nullptr, cudaStreamSynchronize(g->capture_stream));
  return FW_OK;
}

// Switch the group's kernel shape: drop the captured graphs and rebuild the work list.
int group_set_shape(fw_group* g, int k) {
  for (auto& kv : g->graphs) cudaGraphExecDestroy(kv.second);
  g->graphs.clear();
  g->shape = k;
  std::vector<fw_handle*> m = g->members;
  return m.empty() ? FW_OK : group_set(g, m.data(), (int)m.size());
}

int group_advance(fw_group* g, cudaStream_t s, int n_steps);

// Group kernel-shape autotuner, run by the first fw_group_run (every member reset to step 0):
// each shape advances the group kTuneSteps steps untimed, then kTuneSteps steps timed with events
// on the caller's stream; the members are reset after each trial and the fastest shape is kept.
// All shapes give bit-identical results.
int group_autotune(fw_group* g, cudaStream_t s) {
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  FW_CUDA(nullptr, cudaEventCreate(&e0));
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return fail(nullptr, FW_ERR_CUDA, "cudaEventCreate failed");
  }
  int st = FW_OK, best = 0;
  float best_ms = 0.f;
  for (int k = 0; k < kNumShapes2D && st == FW_OK; ++k) {
    if (kShapes2D[k].persistent) continue;  // single-simulation kernel only
    float ms = 0.f;
    if ((st = group_set_shape(g, k)) || (st = group_advance(g, s, kTuneSteps))) break;
    if (cudaEventRecord(e0, s) != cudaSuccess) { st = fail(nullptr, FW_ERR_CUDA, "event record failed"); break; }
    if ((st = group_advance(g, s, kTuneSteps))) break;
    if (cudaEventRecord(e1, s) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
        cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) {
      st = fail(nullptr, FW_ERR_CUDA, "group autotuning trial of shape %d failed", k);
      break;
    }
    for (fw_handle* h : g->members) {
      if ((st = check_device_status(h, s)) || (st = fw_reset(h, s))) {
        st = fail(nullptr, st, "group autotuning: %s", h->err.c_str());
        break;
      }
    }
    if (k == 0 || ms < best_ms) { best_ms = ms; best = k; }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st) return st;
  g->shape_fixed = true;
  return best == g->shape ? FW_OK : group_set_shape(g, best);
}

// Advance every member by up to n_steps, each stopping at its own nt.
int group_advance(fw_group* g, cudaStream_t s, int n_steps) {
  const int n = (int)g->members.size();
  int done = 0;
  while (done < n_steps) {
    // members still running: a prefix of the order (sorted by steps left)
    int k = 0;
    int seg = n_steps - done;
    for (int r = 0; r < n; ++r) {
      const int left = g->members[r]->d.nt - g->members[r]->host_step;
      if (left <= 0) break;
      k = r + 1;
      seg = std::min(seg, left);
    }
    if (k == 0) break;
    const int n_tiles = g->tiles_upto[k];
    int left = seg;
    if (left >= kGroupGraphSteps) {
      cudaGraphExec_t exec = nullptr;
      int st = group_graph(g, n_tiles, &exec);
      if (st) return st;
      for (; left >= kGroupGraphSteps; left -= kGroupGraphSteps) FW_CUDA(nullptr, cudaGraphLaunch(exec, s));
    }
    for (; left > 0; --left) group_launch_step(g, n_tiles, s);
    FW_CUDA(nullptr, cudaGetLastError());
    for (int r = 0; r < k; ++r) g->members[r]->host_step += seg;
    done += seg;
  }
  return FW_OK;
}

}  // namespace

extern "C" {

int fw_group_create(fw_handle* const* handles, int32_t n, fw_group** out) {
  if (!out || !handles || n <= 0) return fail(nullptr, FW_ERR_ARGUMENT, "need n > 0 handles and out");
  *out = nullptr;
  fw_group* g = new (std::nothrow) fw_group();
  if (!g) return fail(nullptr, FW_ERR_OOM, "host allocation failed");
  {
    // kernel shape: FWGB_VARIANT=direct or FWGB_SHAPE2D=<k> fix it; otherwise the 128 x 32 row
    // march until the first fw_group_run has timed every shape on the group itself
    const char* v = std::getenv("FWGB_VARIANT");
    const char* sh = std::getenv("FWGB_SHAPE2D");
    const char* a = std::getenv("FWGB_AUTOTUNE");
    const char* s2 = std::getenv("FWGB_STREAM2D");
    g->stream = !(s2 && std::strcmp(s2, "0") == 0);
    g->shape = 4;
    if (v && std::strcmp(v, "direct") == 0) {
      g->shape = 0;
      g->shape_fixed = true;
    } else if (sh && *sh) {
      const int k = std::atoi(sh);
      if (k < 0 || k >= kNumShapes2D) {
        delete g;
        return fail(nullptr, FW_ERR_ARGUMENT, "FWGB_SHAPE2D=%s outside [0, %d)", sh, kNumShapes2D);
      }
      g->shape = kShapes2D[k].persistent ? 0 : k;
      g->shape_fixed = true;
    } else if (a && std::strcmp(a, "0") == 0) {
      g->shape_fixed = true;
    }
  }
  if (cudaStreamCreateWithFlags(&g->capture_stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete g;
    return fail(nullptr, FW_ERR_CUDA, "stream creation failed");
  }
  int st = group_set(g, handles, n);
  if (st) {
    fw_group_destroy(g);
    return st;
  }
  *out = g;
  return FW_OK;
}

int fw_group_set_members(fw_group* g, fw_handle* const* handles, int32_t n) {
  if (!g || (n > 0 && !handles) || n < 0) return fail(nullptr, FW_ERR_ARGUMENT, "bad group arguments");
  if (n == 0) {
    g->members.clear();
    g->tiles_upto.assign(1, 0);
    return FW_OK;
  }
  return group_set(g, handles, n);
}

int fw_group_advance(fw_group* g, void* stream, int32_t n_steps) {
  if (!g || n_steps < 0) return fail(nullptr, FW_ERR_ARGUMENT, "bad group arguments");
  // the work list order depends on steps left: refresh it before stepping
  std::vector<fw_handle*> m = g->members;
  if (!m.empty()) {
    int st = group_set(g, m.data(), (int)m.size());
    if (st) return st;
  }
  return group_advance(g, static_cast<cudaStream_t>(stream), n_steps);
}

int fw_group_run(fw_group* g, void* stream) {
  if (!g) return fail(nullptr, FW_ERR_ARGUMENT, "group is NULL");
  int max_nt = 0;
  for (fw_handle* h : g->members) {
    int st = fw_reset(h, stream);
    if (st) return fail(nullptr, st, "member reset failed: %s", h->err.c_str());
    max_nt = std::max(max_nt, (int)h->d.nt);
  }
  if (!g->shape_fixed && !g->members.empty()) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(static_cast<cudaStream_t>(stream), &cs) == cudaSuccess &&
        cs == cudaStreamCaptureStatusNone) {
      int st = group_autotune(g, static_cast<cudaStream_t>(stream));
      if (st) return st;
    }
  }
  return fw_group_advance(g, stream, max_nt);
}

int fw_group_block_tile(const fw_group* g, int32_t tile[3]) {
  if (!g || !tile) return FW_ERR_ARGUMENT;
  tile[0] = g->shape ? kShapes2D[g->shape].xc : kD2TX;
  tile[1] = g->shape ? kShapes2D[g->shape].ty : kD2TY;
  tile[2] = 1;
  return FW_OK;
}

int fw_group_destroy(fw_group* g) {
  if (!g) return FW_OK;
  for (auto& kv : g->graphs) cudaGraphExecDestroy(kv.second);
  if (g->capture_stream) cudaStreamDestroy(g->capture_stream);
  if (g->d_args) cudaFree(g->d_args);
  if (g->d_tiles) cudaFree(g->d_tiles);
  if (g->d_maps) cudaFree(g->d_maps);
  delete g;
  return FW_OK;
}

}  // extern "C"
