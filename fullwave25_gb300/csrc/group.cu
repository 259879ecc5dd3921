// The batched group engine (fw_group_*): many 2D simulations stepped together, one launch per
// phase per step over a device work list, with its own kernel-shape autotuner.
#include "engine_host.cuh"

using namespace fwgbh;

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
  // fw_group_run: the whole run (every member from step 0 to its own nt) as one graph, rebuilt
  // when the members, their order or the kernel shape change
  cudaGraphExec_t run_graph = nullptr;
  std::vector<fw_handle*> run_graph_members;
  int run_graph_shape = -1;
  // persistent run (FWGB_GROUP_PERSISTENT=1): member nt (run order), tiles_upto, barrier words,
  // the launch's status word and its 64-bit work-ticket counter
  int* d_persist = nullptr;
  size_t persist_cap = 0;   // ints
};

namespace {

constexpr int kGroupGraphSteps = 64;

void drop_run_graph(fw_group* g) {
  if (g->run_graph) cudaGraphExecDestroy(g->run_graph);
  g->run_graph = nullptr;
  g->run_graph_members.clear();
  g->run_graph_shape = -1;
}

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
  static_assert(kNumShapes2D == 8, "one case per 2D kernel shape");
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
    default: break;  // no persistent or tile group kernels: group shapes are 0-5
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
    drop_run_graph(g);
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
  drop_run_graph(g);
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
    if (kShapes2D[k].persistent || kShapes2D[k].tile) continue;  // single-simulation kernels
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

// The whole run of a freshly reset group as one CUDA graph: the same segments as group_advance
// (members ordered by nt, the active tiles a prefix that shrinks as members finish), every step
// captured as its two launches. Replayed by later runs while the members and shape stay the same.
int group_run_graph(fw_group* g, cudaGraphExec_t* out) {
  if (g->run_graph && g->run_graph_members == g->members && g->run_graph_shape == g->shape) {
    *out = g->run_graph;
    return FW_OK;
  }
  drop_run_graph(g);
  const int n = (int)g->members.size();
  std::vector<int> left(n);
  for (int r = 0; r < n; ++r) left[r] = g->members[r]->d.nt;
  cudaGraph_t graph = nullptr;
  FW_CUDA(nullptr, cudaStreamBeginCapture(g->capture_stream, cudaStreamCaptureModeThreadLocal));
  for (;;) {
    int k = 0, seg = 0;
    for (int r = 0; r < n && left[r] > 0; ++r) {
      seg = k == 0 ? left[r] : std::min(seg, left[r]);
      k = r + 1;
    }
    if (k == 0) break;
    for (int i = 0; i < seg; ++i) group_launch_step(g, g->tiles_upto[k], g->capture_stream);
    for (int r = 0; r < k; ++r) left[r] -= seg;
  }
  const cudaError_t ce = cudaStreamEndCapture(g->capture_stream, &graph);
  if (ce != cudaSuccess) return fail(nullptr, FW_ERR_CUDA, "group run capture: %s", cudaGetErrorString(ce));
  cudaGraphExec_t exec = nullptr;
  const cudaError_t e = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return fail(nullptr, FW_ERR_CUDA, "group run graph: %s", cudaGetErrorString(e));
  g->run_graph = exec;
  g->run_graph_members = g->members;
  g->run_graph_shape = g->shape;
  *out = exec;
  return FW_OK;
}

// The whole run of a freshly reset group as one persistent cooperative launch of the streaming
// row-march bodies (step2d_group_persistent): grid = every block that fits on the device at once
// (at most kBarMaxBlocks), each walking the work list with a grid stride.
template <int TY, int XC, bool kBeta>
int group_run_persistent_t(fw_group* g, cudaStream_t s, int* d_nt, int* d_upto, unsigned* d_bar,
                           int max_nt) {
  auto kern = step2d_group_persistent<TY, XC, kBeta, kMRdtRho, kMDtK>;
  int per_sm = 0, dev = 0, sms = 0;
  FW_CUDA(nullptr, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, TY, 0));
  FW_CUDA(nullptr, cudaGetDevice(&dev));
  FW_CUDA(nullptr, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  int n = (int)g->members.size();
  const int grid = std::min({per_sm * sms, kBarMaxBlocks, g->tiles_upto[n]});
  if (grid < 1) return fail(nullptr, FW_ERR_CUDA, "persistent group kernel: no block fits an SM");
  const StepArgs* a = g->d_args;
  const March2Maps* m = g->d_maps;
  const int4* w = g->d_tiles;
  void* args[] = {&a, &m, &w, &d_nt, &d_upto, &n, &max_nt, &d_bar};
  FW_CUDA(nullptr, cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(kern), dim3(grid),
                                               dim3(TY), args, 0, s));
  return FW_OK;
}

int group_run_persistent(fw_group* g, cudaStream_t s) {
  const int n = (int)g->members.size();
  // ints: member nt, tiles_upto, barrier words, status word, pad, 64-bit ticket counter
  const size_t need = (size_t)n + (n + 1) + kBarWords + 4 + 1;
  if (need > g->persist_cap) {
    if (g->d_persist) cudaFree(g->d_persist);
    g->d_persist = nullptr;
    g->persist_cap = 0;
    FW_CUDA(nullptr, cudaMalloc(&g->d_persist, need * sizeof(int)));
    g->persist_cap = need;
  }
  std::vector<int> host(n + n + 1, 0);
  int max_nt = 0;
  for (int r = 0; r < n; ++r) {
    host[r] = (int)g->members[r]->d.nt;
    max_nt = std::max(max_nt, host[r]);
  }
  for (int r = 0; r <= n; ++r) host[n + r] = g->tiles_upto[r];
  int* d_nt = g->d_persist;
  int* d_upto = d_nt + n;
  // barrier words on an 8-byte boundary: the ticket counter after them is 64-bit
  unsigned* d_bar = reinterpret_cast<unsigned*>(d_upto + n + 1 + ((2 * n + 1) & 1));
  FW_CUDA(nullptr, cudaMemcpyAsync(d_nt, host.data(), host.size() * sizeof(int),
                                   cudaMemcpyHostToDevice, s));
  FW_CUDA(nullptr, cudaMemsetAsync(d_bar, 0, (kBarWords + 4) * sizeof(unsigned), s));
  FW_CUDA(nullptr, cudaStreamSynchronize(s));   // the host vector goes out of scope
  switch (g->shape * 2 + (g->beta ? 1 : 0)) {
    case 2: return group_run_persistent_t<64, 16, false>(g, s, d_nt, d_upto, d_bar, max_nt);
    case 3: return group_run_persistent_t<64, 16, true>(g, s, d_nt, d_upto, d_bar, max_nt);
    case 4: return group_run_persistent_t<64, 32, false>(g, s, d_nt, d_upto, d_bar, max_nt);
    case 5: return group_run_persistent_t<64, 32, true>(g, s, d_nt, d_upto, d_bar, max_nt);
    case 6: return group_run_persistent_t<128, 16, false>(g, s, d_nt, d_upto, d_bar, max_nt);
    case 7: return group_run_persistent_t<128, 16, true>(g, s, d_nt, d_upto, d_bar, max_nt);
    case 8: return group_run_persistent_t<128, 32, false>(g, s, d_nt, d_upto, d_bar, max_nt);
    case 9: return group_run_persistent_t<128, 32, true>(g, s, d_nt, d_upto, d_bar, max_nt);
    case 10: return group_run_persistent_t<128, 64, false>(g, s, d_nt, d_upto, d_bar, max_nt);
    case 11: return group_run_persistent_t<128, 64, true>(g, s, d_nt, d_upto, d_bar, max_nt);
    default: return fail(nullptr, FW_ERR_UNSUPPORTED, "persistent group run: row-march shapes only");
  }
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
      g->shape = kShapes2D[k].persistent || kShapes2D[k].tile ? 0 : k;
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
  // FWGB_GROUP_RUN_GRAPH=0: blocks of kGroupGraphSteps steps as fw_group_advance issues them
  const char* rg = std::getenv("FWGB_GROUP_RUN_GRAPH");
  if ((rg && std::strcmp(rg, "0") == 0) || g->members.empty()) return fw_group_advance(g, stream, max_nt);
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(static_cast<cudaStream_t>(stream), &cs) != cudaSuccess ||
      cs != cudaStreamCaptureStatusNone)
    return fw_group_advance(g, stream, max_nt);
  std::vector<fw_handle*> m = g->members;
  int st = group_set(g, m.data(), (int)m.size());   // order by steps left (all at step 0)
  if (st) return st;
  // FWGB_GROUP_PERSISTENT=1: the whole run as one persistent cooperative launch (row-march
  // shapes with streamed operands) instead of one graph of per-step launches
  const char* pe = std::getenv("FWGB_GROUP_PERSISTENT");
  if (pe && std::strcmp(pe, "1") == 0 && g->shape >= 1 && g->shape <= 5 && g->stream) {
    if ((st = group_run_persistent(g, static_cast<cudaStream_t>(stream)))) return st;
    for (fw_handle* h : g->members) h->host_step = h->d.nt;
    return FW_OK;
  }
  cudaGraphExec_t exec = nullptr;
  if ((st = group_run_graph(g, &exec))) return st;
  FW_CUDA(nullptr, cudaGraphLaunch(exec, static_cast<cudaStream_t>(stream)));
  for (fw_handle* h : g->members) h->host_step = h->d.nt;
  return FW_OK;
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
  drop_run_graph(g);
  if (g->capture_stream) cudaStreamDestroy(g->capture_stream);
  if (g->d_args) cudaFree(g->d_args);
  if (g->d_tiles) cudaFree(g->d_tiles);
  if (g->d_maps) cudaFree(g->d_maps);
  if (g->d_persist) cudaFree(g->d_persist);
  delete g;
  return FW_OK;
}

}  // extern "C"
