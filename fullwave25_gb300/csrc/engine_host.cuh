// Host-side internals of the engine library shared by its translation units (engine.cu: the
// handle API; launch.cu: step launches, graphs and tensor maps; group.cu: the batched group
// engine; adjoint.cu: the discrete adjoint). Not part of the C ABI (include/fwgb.h).
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <string>
#include <utility>
#include <vector>

#include "../../include/fwgb.h"
#include "engine_common.cuh"
#include "kernels_adjoint2d.cuh"
#include "kernels_direct.cuh"
#include "kernels_march2d.cuh"
#include "kernels_march3d.cuh"
#include "kernels_persistent2d.cuh"
#include "kernels_stream3d.cuh"
#include "kernels_tile2d.cuh"

using namespace fwgb;

namespace fwgbh {

constexpr int kMarchXC = 64;   // x planes per block of the 3D register-load plane march
constexpr int kStreamXC = 32;  // x planes per block of the streaming 3D march (default)

// 2D kernel shapes the autotuner chooses from: 0 = direct kernels (one block per 32 y x 8 x tile),
// 1-5 = row-march kernels with TY threads (y columns) walking XC rows (TY + 16 <= 256, the TMA box
// limit; TY a multiple of 32 and XC of 8, whole list tiles per block), 6 = the persistent kernel
// (direct bodies, one cooperative launch per block of steps, grid barriers between phases),
// 7 = the TMA tile kernels (one 32 x 8 tile per block, every operand staged by TMA; every cell
// physics).
struct Shape2D { int ty, xc; bool persistent, tile; };
constexpr Shape2D kShapes2D[] = {{0, 0, false, false},   {64, 16, false, false},
                                 {64, 32, false, false},  {128, 16, false, false},
                                 {128, 32, false, false}, {128, 64, false, false},
                                 {0, 0, true, false},     {0, 0, false, true}};
constexpr int kPersistentShape = 6;
constexpr int kTileShape = 7;
constexpr int kNumShapes2D = sizeof(kShapes2D) / sizeof(kShapes2D[0]);
constexpr int kTuneSteps = 64;   // time steps per autotuning trial (one graph)

enum Variant { kDirect = 0, kMarch = 1, kPersistent = 2, kStream = 3, kTile = 4 };

struct Tiling {
  int t[3];   // tile extent along x, y, z (z unused in 2D)
  int n[3];   // tiles along x, y, z
  int count() const { return n[0] * n[1] * n[2]; }
};


}  // namespace fwgbh

struct fw_handle {
  fw_desc d{};
  int ndim = 0;
  int64_t nx = 0, ny = 0, nz = 1, pitch = 0;  // pitch = padded length of the last axis
  int64_t ncells_padded = 0;
  std::string err = "no error";
  // device memory
  float* state = nullptr;      // n_state padded arrays
  float* maps = nullptr;       // n_maps padded arrays
  uint16_t* dcmap = nullptr;   // tap-set index per cell, 16-bit (ndmap <= 65535)
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
  bool ghost_writes = false;   // a source or air cell lies in the ghost layer (p written there)
  bool aniso = false;          // per-axis relaxation maps (the anisotropic engine)
  bool exp = false;            // exponential-attenuation engine (n_relax = 0, map a_exp)
  int n_out = 0;
  int32_t host_step = 0;
  fwgbh::Tiling tiling{};
  fwgb::StepArgs args{};
  cudaStream_t capture_stream = nullptr;
  cudaGraphExec_t graph = nullptr;
  int graph_steps = 0;
  int variant = fwgbh::kDirect;
  int shape2d = 0;             // index into kShapes2D (2D handles)
  bool shape_fixed = false;    // 2D shape forced (FWGB_SHAPE2D / FWGB_VARIANT) or already tuned
  fwgb::MarchMaps tmaps{};
  fwgb::March2Maps tmaps2{};
  fwgb::Tile2Maps tmaps_t{};   // TMA tile kernels (2D)
  bool stream2d = false;       // 2D isotropic row march: point-wise operands staged by TMA too
  fwgb::StreamMaps smaps{};
  bool stream3d = false;       // 3D isotropic: point-wise operands staged by TMA too
  int ps3d = 2;                // stages of the point-wise ring of the streaming kernels
  int march_xc = fwgbh::kMarchXC;     // x planes per block of the 3D march (streaming: kStreamXC)
  // adjoint: checkpoints every adj_every steps, per-segment state store, adjoint fields and
  // gradient maps (adj_ngrad of them: the allocation depends on the engine and on beta)
  int adj_every = 0, adj_nckpt = 0, adj_ngrad = 0;
  float* adj_ckpt = nullptr;     // adj_nckpt states
  float* adj_store = nullptr;    // adj_every + 1 states
  float* adj_store2 = nullptr;   // second store: the next segment is recomputed into it while
                                 // the current one is reversed (nullptr: no overlap)
  float* adj_lam = nullptr;      // adjoint fields and temporaries, then FP32 gradient partials
  double* adj_grad = nullptr;    // adj_ngrad padded FP64 arrays
  size_t adj_bytes = 0;
};

namespace fwgbh {

// Record the failure text on the handle (or as the last handle-less error) and return code.
int fail(fw_handle* h, int code, const char* fmt, ...);
const char* last_global_error();
void set_global_error(const std::string& msg);

// Return from the calling function with FW_ERR_OOM / FW_ERR_CUDA if a CUDA call fails.
#define FW_CUDA(h, call)                                                                   \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess)                                                                 \
      return ::fwgbh::fail(h, e_ == cudaErrorMemoryAllocation ? FW_ERR_OOM : FW_ERR_CUDA,  \
                           "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, \
                           __LINE__);                                                      \
  } while (0)

inline int64_t round_up(int64_t v, int64_t m) { return (v + m - 1) / m * m; }

inline int n_state(int ndim) { return 1 + ndim + 4 * ndim; }
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
inline int n_maps(const fw_handle* h) { return kMaps + (h->aniso ? 10 * (h->ndim - 1) : 0); }
inline int axis_map(int a, int k) { return kMaps + 10 * (a - 1) + k; }
inline float* state_field(fw_handle* h, int idx) { return h->state + (size_t)idx * h->ncells_padded; }
// Point the state-field pointers of A at a state laid out like h->state (state order) at base.
inline void set_state_pointers(const fw_handle* h, fwgb::StepArgs* A, float* base) {
  int s = 0;
  auto field = [&]() { return base + (size_t)(s++) * h->ncells_padded; };
  A->f.p = field();
  for (int a = 0; a < 3; ++a) A->f.v[a] = a < h->ndim ? field() : nullptr;
  for (int a = 0; a < 3; ++a)
    for (int nu = 0; nu < 2; ++nu) A->f.psi[a][nu] = a < h->ndim ? field() : nullptr;
  for (int a = 0; a < 3; ++a)
    for (int nu = 0; nu < 2; ++nu) A->f.phi[a][nu] = a < h->ndim ? field() : nullptr;
}
inline float* map_field(fw_handle* h, int idx) { return h->maps + (size_t)idx * h->ncells_padded; }

// Time-step kernels are launched with programmatic dependent launch (FWGB_PDL=0 turns it off):
// each may be scheduled while the previous kernel of the stream drains, and waits for it on the
// device (pdl_entry). Captured into graphs as programmatic dependency edges.
inline bool pdl_enabled() {
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

// launch.cu
// Tiled tensor map of `rank` dimensions (innermost first; strides in bytes of dims 1..rank-1).
int encode_map(fw_handle* h, CUtensorMap* map, void* base, cuuint32_t rank,
               const cuuint64_t* dims, const cuuint64_t* strides, const cuuint32_t* box,
               CUtensorMapDataType type = CU_TENSOR_MAP_DATA_TYPE_FLOAT32);
void launch_step(fw_handle* h, cudaStream_t s);
int launch_persistent(fw_handle* h, cudaStream_t s, int n0, int n_steps);
int build_graph(fw_handle* h, int steps);
int encode_field_map(fw_handle* h, CUtensorMap* map, float* base, uint32_t bz, uint32_t by);
int encode_stream_maps(fw_handle* h);
int encode_march2_maps(fw_handle* h, uint32_t ty, March2Maps* m);
int set_shape2d(fw_handle* h, int k);
int encode_tile2_maps(fw_handle* h, fwgb::Tile2Maps* m, float* store, int slots);
int prepare_stream3d(fw_handle* h);

// engine.cu
int check_device_status(fw_handle* h, cudaStream_t s);

}  // namespace fwgbh
