// Host engine implementation (see engine.h).
#include "engine.h"
#include "rfmm_math.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "rfmm_internal.h"

namespace rfmm {

namespace {

constexpr uint32_t kMaxScenes = kMaxSceneCount;

uint32_t pad_tiles(uint32_t n) { return (n + kTile - 1u) / kTile; }

uint32_t log2_ceil(uint32_t v) {
  uint32_t b = 0;
  while ((1u << b) < v) ++b;
  return b;
}

using EncodeTiledFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                   const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                   const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                   CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn get_encode_tiled() {
  static EncodeTiledFn fn = nullptr;
  if (fn == nullptr) {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  }
  return fn;
}

const StepLaunchers kExactLaunchers = {launch_upward,    launch_m2l,      launch_l2l_near,
                                       launch_integrate, launch_near_p2p, launch_accel,
                                       launch_accel_targets};
const StepLaunchers kFastLaunchers = {fast::launch_upward,   fast::launch_m2l,
                                      fast::launch_l2l_near, fast::launch_integrate,
                                      fast::launch_near_p2p, fast::launch_accel,
                                      fast::launch_accel_targets};

}  // namespace

const StepLaunchers &Engine::K() const {
  return float_mode_ == RFMM_FLOAT_FAST ? kFastLaunchers : kExactLaunchers;
}

int Engine::set_float_mode(uint32_t mode) {
  if (mode != RFMM_FLOAT_EXACT && mode != RFMM_FLOAT_FAST) return RFMM_ERR_INVALID;
  if (mode == float_mode_) return RFMM_OK;
  clear_graphs();  // captured with the other variant's kernels
  float_mode_ = mode;
  return RFMM_OK;
}

int cuda_status(cudaError_t e) {
  if (e == cudaSuccess) return RFMM_OK;
  if (e == cudaErrorMemoryAllocation) return RFMM_ERR_OOM;
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver || e == cudaErrorNoKernelImageForDevice)
    return RFMM_ERR_NO_DEVICE;
  return RFMM_ERR_CUDA;
}

#define RF_CK(call)                                 \
  do {                                              \
    cudaError_t e_ = (call);                        \
    if (e_ != cudaSuccess) return cuda_status(e_);  \
  } while (0)

const char *status_string(int status) {
  switch (status) {
    case RFMM_OK: return "ok";
    case RFMM_ERR_INVALID: return "invalid argument";
    case RFMM_ERR_CUDA: return "CUDA runtime error";
    case RFMM_ERR_OOM: return "device memory exhausted";
    case RFMM_ERR_STATE: return "call out of order";
    case RFMM_ERR_TIMEOUT: return "kernel wait timed out";
    case RFMM_ERR_NO_DEVICE: return "no sm_103 CUDA device";
    case RFMM_ERR_DEVICE: return "kernel reported an error";
    case RFMM_ERR_BUDGET: return "request exceeds the memory budget";
    default: return "unknown status";
  }
}

int Engine::alloc(void **p, size_t bytes) {
  bytes = std::max<size_t>(bytes, 256);
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    *p = nullptr;
    return cuda_status(e);
  }
  allocations_.push_back(*p);
  device_bytes_ += bytes;
  return RFMM_OK;
}

int Engine::create(const std::vector<SceneSpec> &specs, Engine **out) {
  if (out == nullptr || specs.empty() || specs.size() > kMaxScenes) return RFMM_ERR_INVALID;
  *out = nullptr;
  for (const SceneSpec &s : specs) {
    if (s.n == 0u || s.n > (1u << 23)) return RFMM_ERR_INVALID;
    if (s.params.depth != 0u && (s.params.depth < 4u || s.params.depth > 6u)) return RFMM_ERR_INVALID;
    if (!(s.params.fixed_point_scale >= 0.0f)) return RFMM_ERR_INVALID;
  }
  {
    // Kernels index bodies (2 float4 each) and cells with 32-bit arithmetic.
    uint64_t slots = 0, cells = 0;
    for (const SceneSpec &s : specs) {
      slots += (uint64_t)pad_tiles(s.n) * kTile;
      cells += total_cells(s.params.depth ? s.params.depth : depth_for_particles(s.n));
    }
    if (slots > (1ull << 30) || cells > (1ull << 28)) return RFMM_ERR_BUDGET;
  }
  int dev = 0;
  RF_CK(cudaGetDevice(&dev));
  cudaDeviceProp prop;
  RF_CK(cudaGetDeviceProperties(&prop, dev));
  if (prop.major != 10 || prop.minor != 3) return RFMM_ERR_NO_DEVICE;
  if (get_encode_tiled() == nullptr) return RFMM_ERR_NO_DEVICE;

  Engine *E = new Engine();
  E->device_ = dev;
  E->sms_ = prop.multiProcessorCount;
  uint32_t body_off = 0, cell_off = 0, task_off = 0;
  for (uint32_t i = 0; i < specs.size(); ++i) {
    const SceneSpec &sp = specs[i];
    SceneDesc d{};
    d.n = sp.n;
    d.depth = sp.params.depth ? sp.params.depth : depth_for_particles(sp.n);
    d.body_off = body_off;
    d.tile_off = body_off / kTile;
    d.cell_off = cell_off;
    d.cells = total_cells(d.depth);
    d.sub_level = d.depth - 3u;
    d.task_off = task_off;
    d.scale = sp.params.fixed_point_scale > 0.0f ? sp.params.fixed_point_scale : fixed_point_scale(sp.n);
    d.gravity = sp.params.gravity;
    d.softening = sp.params.softening;
    d.dt_eff = sp.params.dt * sp.params.speed;
    d.n_f = (float)sp.n;
    d.control_strength = sp.params.control_strength;
    d.control_radius = sp.params.control_radius;
    d.key_base = 0u;  // set below, once the number of scenes fixes the key width
    d.max_depth = d.depth;
    d.tile_cap = pad_tiles(sp.n);
    if (sp.slot) E->use_lists_ = true;
    for (int k = 0; k < 4; k++) {
      d.control_point[k] = sp.params.control_point[k];
      d.control_axis_mode[k] = sp.params.control_axis_mode[k];
    }
    const uint32_t tiles = pad_tiles(sp.n);
    for (uint32_t t = 0; t < tiles; t++) E->tile_scene_h_.push_back(i);
    const uint32_t ntasks = 1u << (3u * d.sub_level);
    for (uint32_t t = 0; t < ntasks; t++) E->task_scene_h_.push_back(i);
    if (sp.slot) d.n = 0u;  // an empty slot: no bodies until activate()
    E->plist_cap_ += total_cells(d.depth - 1u);
    body_off += tiles * kTile;
    cell_off += d.cells;
    task_off += ntasks;
    E->scenes_.push_back(d);
  }
  E->slots_ = body_off;
  E->tiles_ = body_off / kTile;
  E->cells_ = cell_off;
  E->tasks_ = task_off;
  // Sort key = scene rank above a Morton code of fine cells (level F >= depth,
  // at most 8: one scene sorts in three 8-bit radix passes): bodies of one
  // leaf stay contiguous and a warp's bodies stay spatially compact, so a few
  // steps of drift still leave few leaf runs per warp.
  {
    const uint32_t scene_bits = log2_ceil((uint32_t)specs.size());
    const uint32_t fine = std::min(8u, (32u - scene_bits) / 3u);
    for (uint32_t i = 0; i < E->scenes_.size(); i++) {
      E->scenes_[i].key_level = fine;
      E->scenes_[i].key_base = scene_bits ? (i << (3u * fine)) : 0u;
    }
    E->key_bits_ = scene_bits + 3u * fine;
  }
  E->uploaded_.assign(specs.size(), false);

  int st = RFMM_OK;
  auto A = [&](void **p, size_t bytes) {
    if (st == RFMM_OK) st = E->alloc(p, bytes);
  };
  const size_t S = E->slots_, C = E->cells_;
  A((void **)&E->d_scenes_, sizeof(SceneDesc) * specs.size());
  A((void **)&E->d_tile_scene_, 4 * E->tiles_);
  A((void **)&E->d_task_scene_, 4 * E->tasks_);
  A((void **)&E->d_tile_list_, 4 * E->tiles_);
  A((void **)&E->d_task_list_, 4 * E->tasks_);
  A((void **)&E->d_scene_list_, 4 * specs.size());
  for (int b = 0; b < 2; b++) {
    A((void **)&E->d_part_[b], 32 * S);
    A((void **)&E->d_ids_[b], 4 * S);
    A((void **)&E->d_mom_[b], 16 * C);
    A((void **)&E->d_plist_[b], sizeof(WorkItem) * E->plist_cap_);
    A((void **)&E->sort_.keys[b], 4 * S);
    A((void **)&E->sort_.vals[b], 4 * S);
  }
  A((void **)&E->d_src_, 16 * C);
  A((void **)&E->d_aux_, 16 * C);
  A((void **)&E->d_choice_, 4 * C);
  A((void **)&E->d_lfield_, 48 * C);
  A((void **)&E->d_fields_, 48 * C);
  A((void **)&E->d_ctr_, sizeof(Counters));
  A((void **)&E->d_tickets_, 4 * kTicketStride * specs.size());
  A((void **)&E->d_tmaps_, sizeof(CUtensorMap) * 8 * specs.size());
  A((void **)&E->sort_.hist, 4 * 256 * (size_t)sort_tiles(E->slots_));
  A((void **)&E->sort_.totals, 4 * 256);
  for (const SceneDesc &d : E->scenes_) E->max_depth_ = std::max(E->max_depth_, d.max_depth);
  A((void **)&E->d_starts_, 4 * C);
  A((void **)&E->d_leaf_blocks_, 4 * (size_t)leaf_sort_blocks(E->max_depth_) * specs.size());
  E->sort_.capacity = E->slots_;
  if (st != RFMM_OK) {
    delete E;
    return st;
  }
  cudaError_t e = cudaHostAlloc((void **)&E->h_ctr_, sizeof(Counters), cudaHostAllocDefault);
  if (e != cudaSuccess) {
    E->h_ctr_ = nullptr;
    delete E;
    return cuda_status(e);
  }
  e = cudaStreamCreateWithFlags(&E->own_stream_, cudaStreamNonBlocking);
  if (e == cudaSuccess) {
    E->stream_ = E->own_stream_;
    for (auto &ev : E->ev_)
      if (e == cudaSuccess) e = cudaEventCreate(&ev);
  }
  if (e == cudaSuccess && E->use_lists_) e = cudaStreamCreateWithFlags(&E->admit_stream_, cudaStreamNonBlocking);
  if (e == cudaSuccess && E->use_lists_) e = cudaEventCreateWithFlags(&E->admit_ev_, cudaEventDisableTiming);
  if (e == cudaSuccess && E->use_lists_) e = cudaEventCreateWithFlags(&E->refresh_ev_, cudaEventDisableTiming);
  if (e == cudaSuccess) e = configure_tree_kernels();
  if (e == cudaSuccess) e = fast::configure_tree_kernels();
  // Both variants' integrate grids must fit: the smaller resident count.
  if (e == cudaSuccess) E->body_limit_ = std::min(body_ctas_per_sm(), fast::body_ctas_per_sm());
  {
    rfmm_tuning t{};
    // Many scenes: the warp-per-subtree upward gains from more CTAs than stay
    // resident (queued CTAs pick up the tasks as others finish; measured 16
    // against 6: -14% at 256 scenes); one scene's grid is bounded by its
    // 512 subtrees either way.
    t.upward_ctas_per_sm = specs.size() > 1 ? 16 : 6;
    t.m2l_ctas_per_sm = 6;
    t.l2l_ctas_per_sm = 5;
    t.integrate_ctas_per_sm = E->body_limit_;
    t.integrate_dynamic = 0;
    t.resort_interval = 16u;
    t.graph_steps = 16;
    t.pdl = 1;
    // The compacting M2L variant evaluates only the contributing stencil
    // slots; measured faster for one scene and for many.
    t.m2l_compact = 1u;
    // Warp-per-subtree and lane-per-target paths when the work lists are
    // long (many scenes), the CTA- and warp-per-item paths otherwise.
    t.m2l_lanes = 2u;
    t.l2l_lanes = 2u;
    t.upward_warps = 2u;
    if (e == cudaSuccess) e = E->set_tuning(t) == RFMM_OK ? cudaSuccess : cudaErrorInvalidValue;
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(E->d_scenes_, E->scenes_.data(), sizeof(SceneDesc) * specs.size(),
                        cudaMemcpyHostToDevice, E->stream_);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(E->d_tile_scene_, E->tile_scene_h_.data(), 4 * E->tiles_,
                        cudaMemcpyHostToDevice, E->stream_);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(E->d_task_scene_, E->task_scene_h_.data(), 4 * E->tasks_,
                        cudaMemcpyHostToDevice, E->stream_);
  for (int b = 0; b < 2 && e == cudaSuccess; b++) {
    e = cudaMemsetAsync(E->d_part_[b], 0, 32 * S, E->stream_);
    if (e == cudaSuccess) e = cudaMemsetAsync(E->d_mom_[b], 0, 16 * C, E->stream_);
    if (e == cudaSuccess) e = cudaMemsetAsync(E->d_ids_[b], 0, 4 * S, E->stream_);
  }
  if (e == cudaSuccess) e = cudaMemsetAsync(E->d_src_, 0, 16 * C, E->stream_);
  if (e == cudaSuccess) e = cudaMemsetAsync(E->d_aux_, 0, 16 * C, E->stream_);
  if (e == cudaSuccess) e = cudaMemsetAsync(E->d_choice_, 0xFF, 4 * C, E->stream_);
  if (e == cudaSuccess) e = cudaMemsetAsync(E->d_lfield_, 0, 48 * C, E->stream_);
  if (e == cudaSuccess) e = cudaMemsetAsync(E->d_fields_, 0, 48 * C, E->stream_);
  if (e == cudaSuccess) e = cudaMemsetAsync(E->d_ctr_, 0, sizeof(Counters), E->stream_);
  if (e == cudaSuccess)
    e = cudaMemsetAsync(E->d_tickets_, 0, 4 * kTicketStride * specs.size(), E->stream_);
  if (e != cudaSuccess) {
    delete E;
    return cuda_status(e);
  }
  st = E->build_tensor_maps();
  if (st == RFMM_OK) st = E->rebuild_lists();
  if (st == RFMM_OK) st = cuda_status(cudaStreamSynchronize(E->stream_));
  if (st != RFMM_OK) {
    delete E;
    return st;
  }
  *out = E;
  return RFMM_OK;
}

int Engine::build_tensor_maps() {
  EncodeTiledFn encode = get_encode_tiled();
  std::vector<CUtensorMap> maps(8 * scenes_.size());
  std::memset(maps.data(), 0, sizeof(CUtensorMap) * maps.size());
  for (uint32_t s = 0; s < scenes_.size(); s++) {
    const SceneDesc &d = scenes_[s];
    for (uint32_t l = 3; l <= d.depth; l++) {
      const uint64_t dim = 1ull << l;
      void *base = reinterpret_cast<char *>(d_src_) + 16ull * (d.cell_off + level_offset(l));
      const cuuint64_t gdim[3] = {4 * dim, dim, dim};
      const cuuint64_t gstride[2] = {16 * dim, 16 * dim * dim};
      const cuuint32_t box[3] = {24, 6, 6};
      const cuuint32_t estride[3] = {1, 1, 1};
      CUresult r = encode(&maps[8 * s + l], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, base, gdim, gstride,
                          box, estride, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
      if (r != CUDA_SUCCESS) return RFMM_ERR_CUDA;
    }
  }
  RF_CK(cudaMemcpyAsync(d_tmaps_, maps.data(), sizeof(CUtensorMap) * maps.size(),
                        cudaMemcpyHostToDevice, stream_));
  return RFMM_OK;
}

Engine::~Engine() {
  if (stream_ != nullptr) cudaStreamSynchronize(stream_);
  for (auto &kv : graphs_) cudaGraphExecDestroy(kv.second.exec);
  graphs_.clear();
  for (auto &ev : ev_)
    if (ev != nullptr) cudaEventDestroy(ev);
  for (void *p : allocations_) cudaFree(p);
  if (h_ctr_ != nullptr) cudaFreeHost(h_ctr_);
  for (int b = 0; b < 2; b++) {
    if (list_pin_[b] != nullptr) cudaFreeHost(list_pin_[b]);
    if (list_ev_[b] != nullptr) cudaEventDestroy(list_ev_[b]);
  }
  for (int b = 0; b < 2; b++) {
    if (scene_pin_[b] != nullptr) cudaFreeHost(scene_pin_[b]);
    if (scene_ev_[b] != nullptr) cudaEventDestroy(scene_ev_[b]);
    for (MapBlock *m : {&admit_map_, &retire_map_}) {
      if (m->pin[b] != nullptr) cudaFreeHost(m->pin[b]);
      if (m->ev[b] != nullptr) cudaEventDestroy(m->ev[b]);
    }
  }
  if (admit_stream_ != nullptr) {
    cudaStreamSynchronize(admit_stream_);
    cudaStreamDestroy(admit_stream_);
  }
  if (admit_ev_ != nullptr) cudaEventDestroy(admit_ev_);
  if (refresh_ev_ != nullptr) cudaEventDestroy(refresh_ev_);
  if (own_stream_ != nullptr) cudaStreamDestroy(own_stream_);
}

int Engine::set_stream(cudaStream_t s) {
  RF_CK(cudaStreamSynchronize(stream_));
  stream_ = s != nullptr ? s : own_stream_;
  return RFMM_OK;
}

int Engine::set_params(uint32_t scene, const rfmm_params &p) {
  if (scene >= scenes_.size()) return RFMM_ERR_INVALID;
  SceneDesc &d = scenes_[scene];
  if (p.depth != 0u && p.depth != d.depth) return RFMM_ERR_INVALID;
  if (p.fixed_point_scale != 0.0f && p.fixed_point_scale != d.scale) return RFMM_ERR_INVALID;
  d.gravity = p.gravity;
  d.softening = p.softening;
  d.dt_eff = p.dt * p.speed;
  d.control_strength = p.control_strength;
  d.control_radius = p.control_radius;
  for (int k = 0; k < 4; k++) {
    d.control_point[k] = p.control_point[k];
    d.control_axis_mode[k] = p.control_axis_mode[k];
  }
  // Kernels read the scene table from device memory, so captured graphs stay valid.
  RF_CK(cudaMemcpyAsync(d_scenes_ + scene, &d, sizeof(SceneDesc), cudaMemcpyHostToDevice, stream_));
  RF_CK(cudaStreamSynchronize(stream_));
  return RFMM_OK;
}

int Engine::set_resort_interval(uint32_t steps) {
  resort_interval_ = steps;
  tuning_.resort_interval = steps;
  since_sort_ = 0;
  return RFMM_OK;
}

void Engine::clear_graphs() {
  if (stream_ != nullptr) cudaStreamSynchronize(stream_);
  for (auto &kv : graphs_) cudaGraphExecDestroy(kv.second.exec);
  graphs_.clear();
  stamp_regions_used_ = 0;
}

int Engine::set_timeline(bool on) {
  if (on && d_stamps_ == nullptr) {
    const int st = alloc((void **)&d_stamps_, 8ull * kStampRegions * kStampSteps * kStampWordsPerStep);
    if (st != RFMM_OK) return st;
  }
  clear_graphs();  // recaptured with (or without) the stamps
  timeline_ = on;
  return RFMM_OK;
}

// Each region holds the last run of its graph.  Per step and kernel kind:
// busy = last CTA end - first CTA begin (after the dependency wait); gap =
// that begin - the previous recorded kernel's end in the same graph run (the
// launch and dependency latency in front of the kernel).
int Engine::get_timeline(rfmm_timeline *out) {
  if (out == nullptr) return RFMM_ERR_INVALID;
  *out = rfmm_timeline{};
  if (d_stamps_ == nullptr || stamp_regions_used_ == 0u) return RFMM_OK;
  const size_t words = (size_t)stamp_regions_used_ * kStampSteps * kStampWordsPerStep;
  std::vector<unsigned long long> h(words);
  RF_CK(cudaMemcpyAsync(h.data(), d_stamps_, 8ull * words, cudaMemcpyDeviceToHost, stream_));
  const int st = sync();
  if (st != RFMM_OK) return st;
  for (const auto &kv : graphs_) {
    const Graph &g = kv.second;
    if (g.region < 0) continue;
    const unsigned long long *r = h.data() + (size_t)g.region * kStampSteps * kStampWordsPerStep;
    unsigned long long first = 0, prev_end = 0, last = 0;
    bool any = false;
    for (uint32_t j = 0; j < g.len; j++) {
      for (uint32_t k = 0; k < (uint32_t)kKernelKinds; k++) {
        const unsigned long long *w = r + (size_t)j * kStampWordsPerStep + 2u * k;
        if (w[1] == 0ull) continue;  // not launched in this step (or not stamped)
        const unsigned long long begin = ~w[0], end = w[1];
        if (end < begin) continue;
        out->launches[k] += 1u;
        out->busy_ms[k] += (double)(end - begin) * 1e-6;
        if (any && begin > prev_end) out->gap_ms[k] += (double)(begin - prev_end) * 1e-6;
        if (!any) first = begin;
        any = true;
        prev_end = end;
        last = end;
      }
    }
    if (any) {
      out->steps += g.len;
      out->span_ms += (double)(last - first) * 1e-6;
    }
  }
  return RFMM_OK;
}

int Engine::get_tuning(rfmm_tuning *out) const {
  if (out == nullptr) return RFMM_ERR_INVALID;
  *out = tuning_;
  return RFMM_OK;
}

int Engine::set_tuning(const rfmm_tuning &t) {
  if (t.upward_ctas_per_sm < 1u || t.upward_ctas_per_sm > 16u || t.m2l_ctas_per_sm < 1u ||
      t.m2l_ctas_per_sm > 6u || t.l2l_ctas_per_sm < 1u || t.l2l_ctas_per_sm > 8u ||
      t.integrate_ctas_per_sm < 1u || t.integrate_ctas_per_sm > body_limit_ || t.graph_steps < 1u ||
      t.graph_steps > 64u || t.integrate_dynamic > 1u || t.pdl > 1u || t.m2l_compact > 1u ||
      t.m2l_lanes > 2u || t.l2l_lanes > 2u || t.upward_warps > 2u)
    return RFMM_ERR_INVALID;
  clear_graphs();  // captured launch shapes change
  tuning_ = t;
  body_ctas_ = (uint32_t)sms_ * t.integrate_ctas_per_sm;
  tree_ctas_ = (uint32_t)sms_ * t.upward_ctas_per_sm;
  pdl_ = t.pdl != 0u;
  if (resort_interval_ != t.resort_interval) {
    resort_interval_ = t.resort_interval;
    since_sort_ = 0;
  }
  return RFMM_OK;
}

int Engine::autotune(uint32_t steps_per_trial, rfmm_tuning *best) {
  if (!committed_ || steps_per_trial == 0u) return RFMM_ERR_STATE;
  cudaEvent_t a = nullptr, b = nullptr;
  RF_CK(cudaEventCreate(&a));
  RF_CK(cudaEventCreate(&b));
  // Long enough for every candidate resort interval to refresh the order at
  // least twice, so the trials see its amortised cost.
  const uint32_t trial_steps = std::max(steps_per_trial, 64u);
  auto trial = [&](const rfmm_tuning &t, float *ms) -> int {
    int st = set_tuning(t);
    if (st == RFMM_OK) st = step(t.graph_steps);  // capture + warm
    if (st != RFMM_OK) return st;
    RF_CK(cudaEventRecord(a, stream_));
    st = step(trial_steps);
    if (st != RFMM_OK) return st;
    RF_CK(cudaEventRecord(b, stream_));
    RF_CK(cudaEventSynchronize(b));
    RF_CK(cudaEventElapsedTime(ms, a, b));
    return check_device_error();
  };
  rfmm_tuning cur = tuning_;
  float cur_ms = 0.0f;
  int st = trial(cur, &cur_ms);
  // Coordinate descent, two sweeps over the knobs.
  for (int sweep = 0; sweep < 2 && st == RFMM_OK; sweep++) {
    for (int knob = 0; knob < 12 && st == RFMM_OK; knob++) {
      std::vector<uint32_t> values;
      switch (knob) {
        case 0: values = {2, 4, 6, 8, 16}; break;
        case 1: values = {2, 4, 6}; break;
        case 2: values = {2, 4, 5, 8}; break;
        case 3: for (uint32_t v = 1; v <= body_limit_; v++) values.push_back(v); break;
        case 4: values = {0, 1}; break;
        case 5: values = {0, 1}; break;
        case 6: values = {4, 8, 16, 32}; break;
        case 7:
          values = {8, 16, 32, 64};
          break;
        case 8: values = {0, 1}; break;
        case 9: values = {0, 1, 2}; break;
        case 10: values = {0, 1, 2}; break;
        case 11: values = {0, 1, 2}; break;
      }
      for (uint32_t v : values) {
        rfmm_tuning t = cur;
        uint32_t *field[12] = {&t.upward_ctas_per_sm, &t.m2l_ctas_per_sm, &t.l2l_ctas_per_sm,
                               &t.integrate_ctas_per_sm, &t.integrate_dynamic, &t.pdl,
                               &t.graph_steps, &t.resort_interval, &t.m2l_compact,
                               &t.m2l_lanes, &t.l2l_lanes, &t.upward_warps};
        if (*field[knob] == v) continue;
        *field[knob] = v;
        float ms = 0.0f;
        st = trial(t, &ms);
        if (st != RFMM_OK) break;
        if (ms < cur_ms * 0.995f) {
          cur = t;
          cur_ms = ms;
        }
      }
    }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (st != RFMM_OK) return st;
  st = set_tuning(cur);
  if (best != nullptr) *best = cur;
  return st;
}

LaunchCtx Engine::ctx(uint32_t mpar, uint32_t lpar, uint32_t ppar) const {
  LaunchCtx L;
  L.stream = stream_;
  L.scenes = d_scenes_;
  L.tile_scene = d_tile_scene_;
  L.task_scene = d_task_scene_;
  L.part = d_part_[ppar];
  L.mom = d_mom_[mpar];
  L.mom_next = d_mom_[mpar ^ 1u];
  L.src = d_src_;
  L.aux = d_aux_;
  L.choice = d_choice_;
  L.lfield = d_lfield_;
  L.fields = d_fields_;
  L.plist = d_plist_[lpar];
  L.plist_prev = d_plist_[lpar ^ 1u];
  L.plist_cap = plist_cap_;
  L.ctr = d_ctr_;
  L.tickets = d_tickets_;
  L.tmaps = d_tmaps_;
  L.sms = (uint32_t)sms_;
  L.body_ctas = body_ctas_;
  L.tree_ctas = tree_ctas_;
  L.m2l_ctas = (uint32_t)sms_ * tuning_.m2l_ctas_per_sm;
  L.l2l_ctas = (uint32_t)sms_ * tuning_.l2l_ctas_per_sm;
  L.integrate_dynamic = tuning_.integrate_dynamic != 0u;
  L.m2l_compact = tuning_.m2l_compact != 0u;
  L.m2l_lanes = tuning_.m2l_lanes;
  L.l2l_lanes = tuning_.l2l_lanes;
  L.upward_warps = tuning_.upward_warps;
  L.many_scenes = scenes_.size() > 1u;
  L.tile_list = use_lists_ ? d_tile_list_ : nullptr;
  L.task_list = use_lists_ ? d_task_list_ : nullptr;
  L.scene_list = use_lists_ ? d_scene_list_ : nullptr;
  L.pdl = pdl_;
  L.p2p = near_mode_ == kNearP2P;
  L.pos4 = d_pos4_;
  L.near4 = d_near4_;
  L.starts_out = d_starts_;
  L.stamps = nullptr;
  return L;
}

int Engine::upload(uint32_t scene, const void *src, size_t bytes, cudaMemcpyKind kind) {
  if (scene >= scenes_.size() || src == nullptr) return RFMM_ERR_INVALID;
  const SceneDesc &d = scenes_[scene];
  if (bytes != 32ull * d.n) return RFMM_ERR_INVALID;
  RF_CK(cudaMemcpyAsync(d_part_[pcur_] + 2ull * d.body_off, src, bytes, kind, stream_));
  mark_fresh(scene);  // ids are numbered by the commit's key pass
  uploaded_[scene] = true;
  committed_ = false;
  return RFMM_OK;
}

int Engine::upload_all_device(const void *const *src) {
  if (src == nullptr) return RFMM_ERR_INVALID;
  for (uint32_t i = 0; i < scenes_.size(); i++)
    if (scenes_[i].n != 0u && src[i] == nullptr) return RFMM_ERR_INVALID;
  LaunchCtx L = ctx(mcur_, lpar_, pcur_);
  static_assert(sizeof(UploadSources) <= 16384, "kernel parameter size");
  UploadSources us;
  for (uint32_t base = 0; base < scenes_.size(); base += kUploadChunk) {
    const uint32_t count = std::min<uint32_t>(kUploadChunk, (uint32_t)scenes_.size() - base);
    for (uint32_t j = 0; j < count; j++) {
      const SceneDesc &d = scenes_[base + j];
      us.p[j] = nullptr;
      if (d.n == 0u) continue;
      // The copy kernel takes 16-byte aligned device (or managed) memory;
      // anything else is copied by the runtime.
      cudaPointerAttributes a{};
      const bool direct = cudaPointerGetAttributes(&a, src[base + j]) == cudaSuccess &&
                          (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) &&
                          (reinterpret_cast<uintptr_t>(src[base + j]) & 15u) == 0u;
      if (direct) {
        us.p[j] = static_cast<const float4 *>(src[base + j]);
      } else {
        (void)cudaGetLastError();  // a failed attribute query leaves no error behind
        RF_CK(cudaMemcpyAsync(d_part_[pcur_] + 2ull * d.body_off, src[base + j], 32ull * d.n,
                              cudaMemcpyDefault, stream_));
      }
    }
    const SceneDesc &first = scenes_[base], &last = scenes_[base + count - 1u];
    const uint32_t tile_end = last.tile_off + pad_tiles(last.n);
    if (tile_end > first.tile_off) {
      launch_upload_scenes(L, d_part_[pcur_], first.tile_off, tile_end - first.tile_off, base, us);
      RF_CK(cudaGetLastError());
      launches_ += 1;
    }
  }
  for (uint32_t i = 0; i < scenes_.size(); i++) {
    if (scenes_[i].n == 0u) continue;
    mark_fresh(i);  // ids are numbered by the commit's key pass
    uploaded_[i] = true;
  }
  committed_ = false;
  return RFMM_OK;
}

int Engine::seed_galaxy(uint32_t scene) {
  if (scene >= scenes_.size()) return RFMM_ERR_INVALID;
  const SceneDesc &d = scenes_[scene];
  LaunchCtx L = ctx(mcur_, lpar_, pcur_);
  launch_initialize(L, d_part_[pcur_], d.tile_off, pad_tiles(d.n));
  RF_CK(cudaGetLastError());
  launches_ += 1;
  mark_fresh(scene);
  uploaded_[scene] = true;
  committed_ = false;
  return RFMM_OK;
}

uint32_t Engine::radix_sort_kernels() const { return 2u + 3u * ((key_bits_ + 7u) / 8u); }

void Engine::enqueue_resort(uint32_t ppar, uint32_t count_par, unsigned long long *stamps) {
  // Leaf counting sort from the deposit of the current positions; `stamps`
  // is the timeline record block of the step it follows.
  LaunchCtx L = ctx(mcur_, lpar_, ppar);
  L.stamps = stamps;
  leaf_counting_sort(L, (uint32_t)scenes_.size(), max_depth_, d_mom_[count_par], d_leaf_blocks_,
                     d_starts_, d_part_[ppar], d_ids_[ppar], d_part_[ppar ^ 1u], d_ids_[ppar ^ 1u],
                     tiles_);
}

int Engine::rebuild_lists() {
  if (use_lists_) {
    if (list_pin_[0] == nullptr) {
      for (int b = 0; b < 2; b++) {
        RF_CK(cudaHostAlloc((void **)&list_pin_[b], 4ull * (3ull + tiles_ + tasks_ + scenes_.size()),
                            cudaHostAllocDefault));
        RF_CK(cudaEventCreateWithFlags(&list_ev_[b], cudaEventDisableTiming));
      }
    }
    const uint32_t b = list_buf_;
    list_buf_ ^= 1u;
    {
      const auto w0 = std::chrono::steady_clock::now();
      RF_CK(cudaEventSynchronize(list_ev_[b]));  // the last copy out of this block is done
      list_wait_s_ += std::chrono::duration<double>(std::chrono::steady_clock::now() - w0).count();
    }
    uint32_t *blk = list_pin_[b], *tiles = blk + 3, *tasks = blk + 3 + tiles_,
             *sl = blk + 3 + tiles_ + tasks_;
    uint32_t nt = 0, nk = 0, ns = 0;
    for (uint32_t i = 0; i < scenes_.size(); i++) {
      const SceneDesc &d = scenes_[i];
      if (d.n == 0u) continue;
      for (uint32_t t = 0; t < pad_tiles(d.n); t++) tiles[nt++] = d.tile_off + t;
      for (uint32_t t = 0; t < (1u << (3u * d.sub_level)); t++) tasks[nk++] = d.task_off + t;
      sl[ns++] = i;
    }
    blk[0] = nt;
    blk[1] = nk;
    blk[2] = ns;
    if (nt != 0u)
      RF_CK(cudaMemcpyAsync(d_tile_list_, tiles, 4ull * nt, cudaMemcpyHostToDevice, stream_));
    if (nk != 0u)
      RF_CK(cudaMemcpyAsync(d_task_list_, tasks, 4ull * nk, cudaMemcpyHostToDevice, stream_));
    if (ns != 0u)
      RF_CK(cudaMemcpyAsync(d_scene_list_, sl, 4ull * ns, cudaMemcpyHostToDevice, stream_));
    RF_CK(cudaMemcpyAsync(&d_ctr_->tiles_active, blk, 12, cudaMemcpyHostToDevice, stream_));
    RF_CK(cudaEventRecord(list_ev_[b], stream_));
    return RFMM_OK;
  }
  tile_list_h_.clear();
  task_list_h_.clear();
  scene_list_h_.clear();
  for (uint32_t i = 0; i < scenes_.size(); i++) {
    const SceneDesc &d = scenes_[i];
    if (d.n == 0u) continue;
    for (uint32_t t = 0; t < pad_tiles(d.n); t++) tile_list_h_.push_back(d.tile_off + t);
    for (uint32_t t = 0; t < (1u << (3u * d.sub_level)); t++) task_list_h_.push_back(d.task_off + t);
    scene_list_h_.push_back(i);
  }
  const uint32_t counts[3] = {(uint32_t)tile_list_h_.size(), (uint32_t)task_list_h_.size(),
                              (uint32_t)scene_list_h_.size()};
  if (!tile_list_h_.empty())
    RF_CK(cudaMemcpyAsync(d_tile_list_, tile_list_h_.data(), 4 * tile_list_h_.size(),
                          cudaMemcpyHostToDevice, stream_));
  if (!task_list_h_.empty())
    RF_CK(cudaMemcpyAsync(d_task_list_, task_list_h_.data(), 4 * task_list_h_.size(),
                          cudaMemcpyHostToDevice, stream_));
  if (!scene_list_h_.empty())
    RF_CK(cudaMemcpyAsync(d_scene_list_, scene_list_h_.data(), 4 * scene_list_h_.size(),
                          cudaMemcpyHostToDevice, stream_));
  RF_CK(cudaMemcpyAsync(&d_ctr_->tiles_active, counts, sizeof(counts), cudaMemcpyHostToDevice,
                        stream_));
  return RFMM_OK;
}

int Engine::slot_desc(uint32_t scene, uint32_t n, const rfmm_params &p) {
  if (scene >= scenes_.size() || n == 0u) return RFMM_ERR_INVALID;
  SceneDesc &d = scenes_[scene];
  if (d.n != 0u) return RFMM_ERR_STATE;
  if (n > d.tile_cap * kTile) return RFMM_ERR_BUDGET;
  const uint32_t depth = p.depth ? p.depth : depth_for_particles(n);
  if (depth < 4u || depth > d.max_depth) return RFMM_ERR_BUDGET;
  d.n = n;
  d.depth = depth;
  d.cells = total_cells(depth);
  d.sub_level = depth - 3u;
  d.scale = p.fixed_point_scale > 0.0f ? p.fixed_point_scale : fixed_point_scale(n);
  d.gravity = p.gravity;
  d.softening = p.softening;
  d.dt_eff = p.dt * p.speed;
  d.n_f = (float)n;
  d.control_strength = p.control_strength;
  d.control_radius = p.control_radius;
  for (int k = 0; k < 4; k++) {
    d.control_point[k] = p.control_point[k];
    d.control_axis_mode[k] = p.control_axis_mode[k];
  }
  scenes_dirty_ = true;
  return RFMM_OK;
}

int Engine::flush_scenes() {
  if (!scenes_dirty_) return RFMM_OK;
  if (scene_pin_[0] == nullptr) {
    for (int b = 0; b < 2; b++) {
      RF_CK(cudaHostAlloc((void **)&scene_pin_[b], sizeof(SceneDesc) * scenes_.size(), cudaHostAllocDefault));
      RF_CK(cudaEventCreateWithFlags(&scene_ev_[b], cudaEventDisableTiming));
    }
  }
  const uint32_t b = scene_buf_;
  scene_buf_ ^= 1u;
  RF_CK(cudaEventSynchronize(scene_ev_[b]));  // the block's last copy is done
  std::memcpy(scene_pin_[b], scenes_.data(), sizeof(SceneDesc) * scenes_.size());
  RF_CK(cudaMemcpyAsync(d_scenes_, scene_pin_[b], sizeof(SceneDesc) * scenes_.size(),
                        cudaMemcpyHostToDevice, stream_));
  RF_CK(cudaEventRecord(scene_ev_[b], stream_));
  scenes_dirty_ = false;
  return RFMM_OK;
}

int Engine::upload_map(MapBlock &m, const std::vector<uint32_t> &scenes, uint32_t *count,
                       cudaStream_t stream, bool counts) {
  if (m.pin[0] == nullptr) {
    for (int b = 0; b < 2; b++) {
      RF_CK(cudaHostAlloc((void **)&m.pin[b], 8ull * tiles_, cudaHostAllocDefault));
      RF_CK(cudaEventCreateWithFlags(&m.ev[b], cudaEventDisableTiming));
    }
    const int st = alloc((void **)&m.dev, 8ull * tiles_);
    if (st != RFMM_OK) return st;
  }
  const uint32_t b = m.next;
  m.next ^= 1u;
  RF_CK(cudaEventSynchronize(m.ev[b]));  // the block's last copy is done
  uint32_t total = 0;
  for (uint32_t sc : scenes) total += pad_tiles(scenes_[sc].n);
  uint32_t at = 0;
  for (uint32_t sc : scenes) {
    const SceneDesc &d = scenes_[sc];
    for (uint32_t t = 0; t < pad_tiles(d.n); t++, at++) {
      m.pin[b][at] = d.tile_off + t;
      if (counts) m.pin[b][total + at] = d.n;
    }
  }
  // The previous use of m.dev is earlier on the same stream.
  RF_CK(cudaMemcpyAsync(m.dev, m.pin[b], 4ull * total * (counts ? 2u : 1u), cudaMemcpyHostToDevice, stream));
  RF_CK(cudaEventRecord(m.ev[b], stream));
  *count = total;
  return RFMM_OK;
}

int Engine::activate_many(const std::vector<Admission> &admissions) {
  if (admissions.empty()) return RFMM_OK;
  // Ascending slot order: the sort (scene rank above the Morton code) returns
  // the slots' keys in the same order, so sorted position i belongs to map
  // tile i / 256.
  std::vector<Admission> adm(admissions);
  std::sort(adm.begin(), adm.end(),
            [](const Admission &x, const Admission &y) { return x.scene < y.scene; });
  for (size_t i = 1; i < adm.size(); i++)
    if (adm[i].scene == adm[i - 1].scene) return RFMM_ERR_INVALID;
  for (const Admission &a : adm) {  // validate all before changing any slot
    if (a.scene >= scenes_.size() || a.n == 0u || a.buffer > 1u) return RFMM_ERR_INVALID;
    const SceneDesc &d = scenes_[a.scene];
    if (d.n != 0u) return RFMM_ERR_STATE;
    const uint32_t depth = a.params.depth ? a.params.depth : depth_for_particles(a.n);
    if (a.n > d.tile_cap * kTile || depth < 4u || depth > d.max_depth) return RFMM_ERR_BUDGET;
  }
  std::vector<uint32_t> slots;
  std::vector<SceneDesc> descs;
  SceneMask which{};
  for (const Admission &a : adm) {
    const int sd = slot_desc(a.scene, a.n, a.params);
    if (sd != RFMM_OK) return sd;
    slots.push_back(a.scene);
    descs.push_back(scenes_[a.scene]);
    which.bits[a.scene >> 5] |= 1u << (a.scene & 31u);
  }
  // On the admission stream (engines with lists; else the engine stream):
  // these writes touch only the admitted slots -- their descriptors (the
  // rest of the table, such as slots retiring at the end of the chunk in
  // flight, reaches the device with the next refresh_lists), bodies, ids
  // and cells -- so they may overlap the chunk in flight.  The host buffer
  // parities already describe the state after the chunks enqueued so far.
  cudaStream_t as = admit_stream_ != nullptr ? admit_stream_ : stream_;
  if (as != stream_) RF_CK(cudaStreamWaitEvent(as, refresh_ev_, 0));
  launch_write_scenes(as, d_scenes_, slots.data(), descs.data(), (uint32_t)slots.size());
  const uint32_t cur = pcur_.load(), scr = cur ^ 1u;
  for (const Admission &a : adm)
    if (a.buffer != scr)  // staged before a resort flipped the buffers
      RF_CK(cudaMemcpyAsync(slot_bodies(a.scene, scr), slot_bodies(a.scene, a.buffer), 32ull * a.n,
                            cudaMemcpyDeviceToDevice, as));
  uint32_t total = 0;
  int st = upload_map(admit_map_, slots, &total, as);
  if (st != RFMM_OK) return st;
  // Keys of the staged bodies (numbering them in caller order), one sort,
  // cleared trees, one gather with the leaf deposit into the current buffer.
  LaunchCtx L = ctx(mcur_, lpar_, scr);
  L.stream = as;
  launch_keys(L, sort_.keys[0], sort_.vals[0], d_ids_[scr], 1, total, 0u, nullptr, admit_map_.dev);
  const int r = radix_sort(as, sort_, total * kTile, key_bits_);
  launch_clear_scenes(L, (uint32_t)scenes_.size(), which, d_mom_[mcur_], d_mom_[mcur_ ^ 1u], d_src_, d_aux_);
  launch_gather(L, sort_.vals[r], d_part_[scr], d_ids_[scr], d_part_[cur], d_ids_[cur], d_mom_[mcur_],
                total, 0u, nullptr, admit_map_.dev);
  RF_CK(cudaGetLastError());
  if (as != stream_) {  // the engine stream's next kernels see the admitted slots
    RF_CK(cudaEventRecord(admit_ev_, as));
    RF_CK(cudaStreamWaitEvent(stream_, admit_ev_, 0));
  }
  for (uint32_t sc : slots) uploaded_[sc] = true;
  launches_ += 3u + 3u * ((key_bits_ + 7u) / 8u);
  committed_ = true;
  return RFMM_OK;
}

int Engine::retire_many(const std::vector<uint32_t> &slots) {
  if (slots.empty()) return RFMM_OK;
  for (uint32_t sc : slots)
    if (sc >= scenes_.size() || scenes_[sc].n == 0u) return RFMM_ERR_INVALID;
  uint32_t total = 0;
  int st = upload_map(retire_map_, slots, &total, stream_, true);
  if (st != RFMM_OK) return st;
  const uint32_t cur = pcur_.load();
  LaunchCtx L = ctx(mcur_, lpar_, cur);
  // Body counts from the map: an admission overlapping this launch does not
  // write these slots' descriptors, but the table refresh after it will.
  launch_unpermute(L, d_ids_[cur], d_part_[cur ^ 1u], 0u, total, retire_map_.dev, retire_map_.dev + total);
  RF_CK(cudaGetLastError());
  launches_ += 1;
  for (uint32_t sc : slots) scenes_[sc].n = 0u;
  scenes_dirty_ = true;
  return RFMM_OK;
}

int Engine::refresh_lists() {
  int st = flush_scenes();
  if (st == RFMM_OK) st = rebuild_lists();
  if (st == RFMM_OK && refresh_ev_ != nullptr) RF_CK(cudaEventRecord(refresh_ev_, stream_));
  return st;
}

int Engine::commit() {
  for (bool u : uploaded_)
    if (!u) return RFMM_ERR_STATE;
  LaunchCtx L = ctx(mcur_, lpar_, pcur_);
  // The key pass also numbers the bodies of scenes uploaded since the last
  // commit in caller order.
  launch_keys(L, sort_.keys[0], sort_.vals[0], d_ids_[pcur_], any_fresh_ ? 2 : 0, tiles_, 0u,
              &fresh_);
  fresh_ = SceneMask{};
  any_fresh_ = false;
  const int r = radix_sort(stream_, sort_, slots_, key_bits_);
  // The rebuilt tree starts from cleared moment, source and record buffers
  // (the upward pass skips subtrees that are empty in both moment buffers).
  RF_CK(cudaMemsetAsync(d_mom_[mcur_], 0, 16ull * cells_, stream_));
  RF_CK(cudaMemsetAsync(d_mom_[mcur_ ^ 1u], 0, 16ull * cells_, stream_));
  RF_CK(cudaMemsetAsync(d_src_, 0, 16ull * cells_, stream_));
  RF_CK(cudaMemsetAsync(d_aux_, 0, 16ull * cells_, stream_));
  launch_gather(L, sort_.vals[r], d_part_[pcur_], d_ids_[pcur_], d_part_[pcur_ ^ 1u],
                d_ids_[pcur_ ^ 1u], d_mom_[mcur_], tiles_, 0u, d_pos4_);
  launches_ += radix_sort_kernels();
  if (near_mode_ == kNearP2P) {
    launch_leaf_starts(L, sort_.keys[r], (uint32_t)scenes_.size());
    launches_ += 1;
  }
  RF_CK(cudaGetLastError());
  pcur_ ^= 1u;
  committed_ = true;
  solved_ = false;
  tree_buf_ = -1;
  since_sort_ = 0;
  return RFMM_OK;
}

void Engine::enqueue_step(uint32_t mpar, uint32_t lpar, uint32_t ppar, unsigned long long *stamps) {
  LaunchCtx L = ctx(mpar, lpar, ppar);
  L.stamps = stamps;
  K().upward(L, lpar, tasks_);
  K().m2l(L, lpar);
  K().l2l_near(L, lpar);
  if (near_mode_ == kNearP2P) K().near_p2p(L, tiles_);
  K().integrate(L, tiles_);
  if (near_mode_ == kNearP2P) enqueue_p2p_sort(mpar, lpar, ppar, d_mom_[mpar ^ 1u]);
}

void Engine::enqueue_p2p_sort(uint32_t mpar, uint32_t lpar, uint32_t ppar, uint4 *mom_into) {
  // Sorting from the caller's order makes the order inside a leaf the caller
  // order, whatever the history: the pair sums run in a fixed order.
  LaunchCtx L = ctx(mpar, lpar, ppar);
  launch_unpermute(L, d_ids_[ppar], d_part_[ppar ^ 1u], 0u, tiles_);
  LaunchCtx C = ctx(mpar, lpar, ppar ^ 1u);
  launch_keys(C, sort_.keys[0], sort_.vals[0], d_ids_[ppar ^ 1u], 1, tiles_, 0u);
  const int r = radix_sort(stream_, sort_, slots_, key_bits_);
  launch_gather(L, sort_.vals[r], d_part_[ppar ^ 1u], d_ids_[ppar ^ 1u], d_part_[ppar],
                d_ids_[ppar], mom_into, tiles_, 0u, d_pos4_);
  launch_leaf_starts(L, sort_.keys[r], (uint32_t)scenes_.size());
}

int Engine::set_near_mode(uint32_t mode) {
  if (mode != kNearReference && mode != kNearP2P) return RFMM_ERR_INVALID;
  if (use_lists_) return RFMM_ERR_INVALID;  // serving slots run the reference near field
  for (const SceneDesc &d : scenes_)
    if (d.key_level < d.depth) return RFMM_ERR_INVALID;
  if (mode == near_mode_) return RFMM_OK;
  if (mode == kNearP2P && d_pos4_ == nullptr) {
    int st = alloc((void **)&d_pos4_, 16ull * slots_);
    if (st == RFMM_OK) st = alloc((void **)&d_near4_, 16ull * slots_);
    if (st != RFMM_OK) return st;
  }
  clear_graphs();
  for (SceneDesc &d : scenes_) d.near_mode = mode;
  RF_CK(cudaMemcpyAsync(d_scenes_, scenes_.data(), sizeof(SceneDesc) * scenes_.size(),
                        cudaMemcpyHostToDevice, stream_));
  near_mode_ = mode;
  if (!committed_) return RFMM_OK;
  // Re-sort the committed bodies for the new mode, starting from the caller's order.
  LaunchCtx L = ctx(mcur_, lpar_, pcur_);
  launch_unpermute(L, d_ids_[pcur_], d_part_[pcur_ ^ 1u], 0u, tiles_);
  pcur_ ^= 1u;
  for (uint32_t i = 0; i < scenes_.size(); i++)
    if (scenes_[i].n != 0u) mark_fresh(i);  // back in caller order
  RF_CK(cudaGetLastError());
  launches_ += 1u;
  return commit();
}

int Engine::solve_fields() {
  if (!committed_) return RFMM_ERR_STATE;
  LaunchCtx L = ctx(mcur_, lpar_, pcur_);
  K().upward(L, lpar_, tasks_);
  K().m2l(L, lpar_);
  K().l2l_near(L, lpar_);
  RF_CK(cudaGetLastError());
  launches_ += 3;
  lpar_ ^= 1u;
  tree_buf_ = (int)mcur_;
  solved_ = true;
  return RFMM_OK;
}

int Engine::launch_chunk(uint32_t len, bool sort_at_end) {
  Graph *g = nullptr;
  const int st = capture_chunk(len, mcur_, lpar_, pcur_.load(), sort_at_end, &g);
  if (st != RFMM_OK) return st;
  RF_CK(cudaGraphLaunch(g->exec, stream_));
  launches_ += g->kernels;
  const uint32_t flip = len & 1u;
  tree_buf_ = (int)(mcur_ ^ ((len - 1u) & 1u));
  mcur_ ^= flip;
  lpar_ ^= flip;
  if (sort_at_end) pcur_ ^= 1u;
  return RFMM_OK;
}

int Engine::prepare_graphs(uint32_t max_len) {
  if (max_len == 0u || max_len > tuning_.graph_steps) return RFMM_ERR_INVALID;
  for (uint32_t len = 1; len <= max_len; len++)
    for (uint32_t m = 0; m < 2u; m++)
      for (uint32_t l = 0; l < 2u; l++)
        for (uint32_t p = 0; p < 2u; p++)
          for (int sort = 0; sort < (resort_interval_ > 0 ? 2 : 1); sort++) {
            Graph *g = nullptr;
            const int st = capture_chunk(len, m, l, p, sort != 0, &g);
            if (st != RFMM_OK) return st;
          }
  return RFMM_OK;
}

int Engine::capture_chunk(uint32_t len, uint32_t mcur, uint32_t lpar, uint32_t pcur, bool sort_at_end,
                          Graph **out) {
  const auto key = std::make_tuple(len, mcur, lpar, pcur, sort_at_end);
  auto it = graphs_.find(key);
  if (it == graphs_.end()) {
    // Timeline: this graph's records, cleared by its first node.
    int region = -1;
    unsigned long long *rec = nullptr;
    if (timeline_ && d_stamps_ != nullptr && stamp_regions_used_ < kStampRegions &&
        len <= kStampSteps) {
      region = (int)stamp_regions_used_++;
      rec = d_stamps_ + (size_t)region * kStampSteps * kStampWordsPerStep;
    }
    cudaGraph_t g = nullptr;
    RF_CK(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
    if (rec != nullptr)
      cudaMemsetAsync(rec, 0, 8ull * kStampSteps * kStampWordsPerStep, stream_);
    for (uint32_t j = 0; j < len; j++)
      enqueue_step(mcur ^ (j & 1u), lpar ^ (j & 1u), pcur,
                   rec != nullptr ? rec + (size_t)j * kStampWordsPerStep : nullptr);
    if (sort_at_end)
      enqueue_resort(pcur, mcur ^ (len & 1u),
                     rec != nullptr ? rec + (size_t)(len - 1u) * kStampWordsPerStep : nullptr);
    cudaError_t e = cudaStreamEndCapture(stream_, &g);
    if (e != cudaSuccess) {
      if (g != nullptr) cudaGraphDestroy(g);
      return cuda_status(e);
    }
    cudaGraphExec_t exec = nullptr;
    e = cudaGraphInstantiate(&exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_status(e);
    const uint32_t kernels = len * kernels_per_step() + (sort_at_end ? resort_kernels() : 0u);
    it = graphs_.emplace(key, Graph{exec, kernels, len, sort_at_end, region}).first;
  }
  *out = &it->second;
  return RFMM_OK;
}

int Engine::step(uint32_t steps) {
  if (!committed_) return RFMM_ERR_STATE;
  while (steps > 0 && near_mode_ == kNearP2P) {  // every step ends with its own sort
    const uint32_t len = std::min(steps, tuning_.graph_steps);
    const int st = launch_chunk(len, false);
    if (st != RFMM_OK) return st;
    steps -= len;
  }
  while (steps > 0) {
    if (resort_interval_ > 0 && since_sort_ >= resort_interval_) {
      enqueue_resort(pcur_, mcur_);
      RF_CK(cudaGetLastError());
      launches_ += resort_kernels();
      pcur_ ^= 1u;
      since_sort_ = 0;
    }
    uint32_t len = std::min(steps, tuning_.graph_steps);
    bool sort_at_end = false;
    if (resort_interval_ > 0) {
      const uint32_t until = resort_interval_ - since_sort_;
      if (len >= until) {
        len = until;
        sort_at_end = true;
      }
    }
    const int st = launch_chunk(len, sort_at_end);
    if (st != RFMM_OK) return st;
    since_sort_ = sort_at_end ? 0u : since_sort_ + len;
    steps -= len;
  }
  solved_ = true;
  return RFMM_OK;
}

// The error word is copied into pinned host memory behind the work already
// queued, so one synchronisation covers both.
int Engine::check_device_error() {
  RF_CK(cudaMemcpyAsync(h_ctr_, d_ctr_, sizeof(Counters), cudaMemcpyDeviceToHost, stream_));
  RF_CK(cudaStreamSynchronize(stream_));
  if (h_ctr_->error == kDevErrTmaTimeout) return RFMM_ERR_TIMEOUT;
  if (h_ctr_->error != 0u) return RFMM_ERR_DEVICE;
  return RFMM_OK;
}

int Engine::sync() { return check_device_error(); }

int Engine::check_wait_timeout(uint32_t polls) {
  if (polls == 0u || polls > (1u << 22)) return RFMM_ERR_INVALID;
  // The check has its own status word; the engine's error word is untouched.
  uint32_t *status = &d_ctr_->wait_check;
  RF_CK(cudaMemsetAsync(status, 0xFF, sizeof(uint32_t), stream_));
  launch_wait_check(stream_, polls, status);
  RF_CK(cudaGetLastError());
  launches_ += 1;
  uint32_t got = 0xFFFFFFFFu;
  RF_CK(cudaMemcpyAsync(&got, status, sizeof(got), cudaMemcpyDeviceToHost, stream_));
  RF_CK(cudaStreamSynchronize(stream_));
  if (got == (uint32_t)kDevErrTmaTimeout) return RFMM_ERR_TIMEOUT;
  return got == (uint32_t)kDevErrNone ? RFMM_OK : RFMM_ERR_CUDA;
}

int Engine::device_error(uint32_t *code, uint32_t *info) {
  Counters c;
  RF_CK(cudaMemcpyAsync(&c, d_ctr_, sizeof(Counters), cudaMemcpyDeviceToHost, stream_));
  RF_CK(cudaStreamSynchronize(stream_));
  if (code) *code = c.error;
  if (info) *info = c.error_info;
  return RFMM_OK;
}

size_t Engine::buffer_bytes(uint32_t scene, int which) const {
  const SceneDesc &d = scenes_[scene];
  switch (which) {
    case RFMM_BUF_PARTICLES: return 32ull * d.n;
    case RFMM_BUF_MOMENTS: return 16ull * d.cells;
    case RFMM_BUF_FIELDS: return 48ull * d.cells;
    default: return 0;
  }
}

int Engine::download(uint32_t scene, int which, void *dst, size_t bytes, cudaMemcpyKind kind) {
  if (scene >= scenes_.size() || dst == nullptr) return RFMM_ERR_INVALID;
  const size_t need = buffer_bytes(scene, which);
  if (need == 0 || bytes != need) return RFMM_ERR_INVALID;
  const SceneDesc &d = scenes_[scene];
  const void *from = nullptr;
  if (which == RFMM_BUF_PARTICLES) {
    if (!committed_) return RFMM_ERR_STATE;
    LaunchCtx L = ctx(mcur_, lpar_, pcur_);
    launch_unpermute(L, d_ids_[pcur_], d_part_[pcur_ ^ 1u], d.tile_off, pad_tiles(d.n));
    RF_CK(cudaGetLastError());
    from = d_part_[pcur_ ^ 1u] + 2ull * d.body_off;
  } else if (which == RFMM_BUF_MOMENTS) {
    if (tree_buf_ < 0) return RFMM_ERR_STATE;
    from = d_mom_[tree_buf_] + d.cell_off;
  } else {
    if (!solved_) return RFMM_ERR_STATE;
    from = d_fields_ + 12ull * d.cell_off;
  }
  RF_CK(cudaMemcpyAsync(dst, from, bytes, kind, stream_));
  return sync();
}

int Engine::download_all(int which, void *const *dst, cudaMemcpyKind kind) {
  if (dst == nullptr) return RFMM_ERR_INVALID;
  for (uint32_t s = 0; s < scenes_.size(); s++)
    if (scenes_[s].n != 0u && (dst[s] == nullptr || buffer_bytes(s, which) == 0)) return RFMM_ERR_INVALID;
  if (which == RFMM_BUF_PARTICLES) {
    if (!committed_) return RFMM_ERR_STATE;
    LaunchCtx L = ctx(mcur_, lpar_, pcur_);
    launch_unpermute(L, d_ids_[pcur_], d_part_[pcur_ ^ 1u], 0u, tiles_);  // every scene at once
    RF_CK(cudaGetLastError());
    launches_ += 1;
  } else if (which == RFMM_BUF_MOMENTS) {
    if (tree_buf_ < 0) return RFMM_ERR_STATE;
  } else if (!solved_) {
    return RFMM_ERR_STATE;
  }
  for (uint32_t s = 0; s < scenes_.size(); s++) {
    const SceneDesc &d = scenes_[s];
    if (d.n == 0u) continue;
    const void *from = which == RFMM_BUF_PARTICLES ? (const void *)(d_part_[pcur_ ^ 1u] + 2ull * d.body_off)
                       : which == RFMM_BUF_MOMENTS ? (const void *)(d_mom_[tree_buf_] + d.cell_off)
                                                   : (const void *)(d_fields_ + 12ull * d.cell_off);
    RF_CK(cudaMemcpyAsync(dst[s], from, buffer_bytes(s, which), kind, stream_));
  }
  return sync();
}

int Engine::digest(uint32_t scene, int which, uint32_t *out) {
  if (scene >= scenes_.size() || out == nullptr) return RFMM_ERR_INVALID;
  const size_t bytes = buffer_bytes(scene, which);
  if (bytes == 0) return RFMM_ERR_INVALID;
  std::vector<uint8_t> host(bytes);
  const int st = download(scene, which, host.data(), bytes, cudaMemcpyDeviceToHost);
  if (st != RFMM_OK) return st;
  uint32_t h = 2166136261u;  // FNV-1a, native/main.rs:152-163
  for (uint8_t b : host) {
    h ^= b;
    h *= 16777619u;
  }
  *out = h;
  return RFMM_OK;
}

int Engine::phase_times(float ms[7]) {
  if (!committed_ || ms == nullptr) return RFMM_ERR_INVALID;
  if (d_mom_scratch_ == nullptr) {
    const int st = alloc((void **)&d_mom_scratch_, 16ull * cells_);
    if (st != RFMM_OK) return st;
  }
  LaunchCtx L = ctx(mcur_, lpar_, pcur_);
  // Standalone P2M on a scratch tree, timed for the phase breakdown only.
  RF_CK(cudaMemsetAsync(d_mom_scratch_, 0, 16ull * cells_, stream_));
  RF_CK(cudaEventRecord(ev_[5], stream_));
  launch_deposit(L, d_mom_scratch_, tiles_);
  RF_CK(cudaEventRecord(ev_[6], stream_));
  // One instrumented frame.
  RF_CK(cudaEventRecord(ev_[0], stream_));
  K().upward(L, lpar_, tasks_);
  RF_CK(cudaEventRecord(ev_[1], stream_));
  K().m2l(L, lpar_);
  RF_CK(cudaEventRecord(ev_[2], stream_));
  K().l2l_near(L, lpar_);
  RF_CK(cudaEventRecord(ev_[3], stream_));
  if (near_mode_ == kNearP2P) K().near_p2p(L, tiles_);
  RF_CK(cudaEventRecord(ev_[7], stream_));
  K().integrate(L, tiles_);
  RF_CK(cudaEventRecord(ev_[4], stream_));
  if (near_mode_ == kNearP2P) {
    enqueue_p2p_sort(mcur_, lpar_, pcur_, d_mom_[mcur_ ^ 1u]);
    launches_ += p2p_sort_kernels();
  }
  RF_CK(cudaGetLastError());
  launches_ += 5;
  tree_buf_ = (int)mcur_;
  mcur_ ^= 1u;
  lpar_ ^= 1u;
  solved_ = true;
  since_sort_++;
  const int st = sync();
  if (st != RFMM_OK) return st;
  float t[6];
  RF_CK(cudaEventElapsedTime(&t[0], ev_[5], ev_[6]));
  RF_CK(cudaEventElapsedTime(&t[1], ev_[0], ev_[1]));
  RF_CK(cudaEventElapsedTime(&t[2], ev_[1], ev_[2]));
  RF_CK(cudaEventElapsedTime(&t[3], ev_[2], ev_[3]));
  RF_CK(cudaEventElapsedTime(&t[5], ev_[3], ev_[7]));
  RF_CK(cudaEventElapsedTime(&t[4], ev_[7], ev_[4]));
  ms[0] = 0.0f;   // clear: folded into upward
  ms[1] = t[0];   // deposit (standalone P2M; fused into integrate in the step)
  ms[2] = t[1];   // upward
  ms[3] = t[2];   // m2l
  ms[4] = t[3];   // downward (L2L fused with near)
  ms[5] = near_mode_ == kNearP2P ? t[5] : 0.0f;  // near: fused into downward, or P2P sums
  ms[6] = t[4];   // integrate (+ next deposit)
  return RFMM_OK;
}

int Engine::profile_steps(uint32_t steps, float ms[kKernelKinds], uint32_t launches[kKernelKinds]) {
  if (!committed_ || ms == nullptr || launches == nullptr) return RFMM_ERR_INVALID;
  // Every launch is enqueued back to back between its own event pair, so the
  // GPU never idles waiting for the host and each pair brackets device time.
  struct Rec {
    int kind;
    cudaEvent_t a, b;
  };
  std::vector<Rec> recs;
  int st = RFMM_OK;
  auto timed = [&](int kind, auto &&enqueue) {
    Rec r{kind, nullptr, nullptr};
    if (st != RFMM_OK) return;
    cudaError_t e = cudaEventCreate(&r.a);
    if (e == cudaSuccess) e = cudaEventCreate(&r.b);
    if (e == cudaSuccess) e = cudaEventRecord(r.a, stream_);
    if (e == cudaSuccess) enqueue();
    if (e == cudaSuccess) e = cudaEventRecord(r.b, stream_);
    if (e == cudaSuccess) e = cudaGetLastError();
    recs.push_back(r);
    if (e != cudaSuccess) st = cuda_status(e);
  };
  for (uint32_t s = 0; s < steps && st == RFMM_OK; s++) {
    if (near_mode_ == kNearReference && resort_interval_ > 0 && since_sort_ >= resort_interval_) {
      timed(kKResort, [&] { enqueue_resort(pcur_, mcur_); });
      launches_ += resort_kernels();
      pcur_ ^= 1u;
      since_sort_ = 0;
    }
    LaunchCtx L = ctx(mcur_, lpar_, pcur_);
    timed(kKUpward, [&] { K().upward(L, lpar_, tasks_); });
    timed(kKM2L, [&] { K().m2l(L, lpar_); });
    timed(kKL2LNear, [&] { K().l2l_near(L, lpar_); });
    if (near_mode_ == kNearP2P) timed(kKNearP2P, [&] { K().near_p2p(L, tiles_); });
    timed(kKIntegrate, [&] { K().integrate(L, tiles_); });
    if (near_mode_ == kNearP2P)
      timed(kKResort, [&] { enqueue_p2p_sort(mcur_, lpar_, pcur_, d_mom_[mcur_ ^ 1u]); });
    launches_ += kernels_per_step();
    tree_buf_ = (int)mcur_;
    mcur_ ^= 1u;
    lpar_ ^= 1u;
    since_sort_++;
  }
  solved_ = true;
  cudaError_t e = cudaStreamSynchronize(stream_);
  if (st == RFMM_OK && e != cudaSuccess) st = cuda_status(e);
  for (Rec &r : recs) {
    float t = 0.0f;
    if (st == RFMM_OK && r.a != nullptr && r.b != nullptr &&
        cudaEventElapsedTime(&t, r.a, r.b) == cudaSuccess) {
      ms[r.kind] += t;
      launches[r.kind] += 1u;
    }
    if (r.a != nullptr) cudaEventDestroy(r.a);
    if (r.b != nullptr) cudaEventDestroy(r.b);
  }
  if (st != RFMM_OK) return st;
  return check_device_error();
}

int Engine::diag_prepare(uint32_t scene, size_t doubles, bool all_bodies) {
  if (scene >= scenes_.size() || !committed_) return RFMM_ERR_STATE;
  if (d_accphi_ == nullptr) {
    int st = alloc((void **)&d_accphi_, 16ull * slots_);
    if (st == RFMM_OK) st = alloc((void **)&d_slot_of_, 4ull * slots_);
    if (st != RFMM_OK) return st;
  }
  if (doubles > diag_doubles_) {
    const int st = alloc((void **)&d_diag_, 8ull * doubles);
    if (st != RFMM_OK) return st;
    diag_doubles_ = doubles;
  }
  // Field solve of the current positions, then per-body acceleration and
  // potential in the caller's order, and the bodies themselves in that order.
  int st = solve_fields();
  if (st != RFMM_OK) return st;
  const SceneDesc &d = scenes_[scene];
  LaunchCtx L = ctx(tree_buf_ < 0 ? mcur_ : (uint32_t)tree_buf_, lpar_, pcur_);
  if (all_bodies) K().accel(L, d_ids_[pcur_], d_accphi_, d.tile_off, pad_tiles(d.n));
  launch_unpermute(L, d_ids_[pcur_], d_part_[pcur_ ^ 1u], d.tile_off, pad_tiles(d.n));
  RF_CK(cudaGetLastError());
  launches_ += all_bodies ? 2u : 1u;
  return RFMM_OK;
}

int Engine::accelerations(uint32_t scene, float *host_out) {
  if (host_out == nullptr) return RFMM_ERR_INVALID;
  const int st = diag_prepare(scene, 0, true);
  if (st != RFMM_OK) return st;
  const SceneDesc &d = scenes_[scene];
  RF_CK(cudaMemcpyAsync(host_out, d_accphi_ + d.body_off, 16ull * d.n, cudaMemcpyDeviceToHost,
                        stream_));
  return sync();
}

int Engine::force_error(uint32_t scene, uint32_t targets, uint64_t seed, double *rms_rel,
                        double *max_rel) {
  if (scene >= scenes_.size() || targets == 0u) return RFMM_ERR_INVALID;
  const SceneDesc &d = scenes_[scene];
  const uint32_t nt = std::min(targets, d.n);
  const uint32_t splits = 64u;
  // doubles: partial [splits][nt][3], reference [nt][3], and the target ids.
  const size_t doubles = (size_t)splits * nt * 3u + (size_t)nt * 3u + nt;
  int st = diag_prepare(scene, doubles, false);
  if (st != RFMM_OK) return st;
  // Uniform sample without replacement (splitmix64 partial Fisher-Yates).
  std::vector<uint32_t> idx(d.n);
  for (uint32_t i = 0; i < d.n; i++) idx[i] = i;
  uint64_t x = seed;
  for (uint32_t i = 0; i < nt; i++) {
    x += 0x9E3779B97F4A7C15ull;
    uint64_t z = x;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    const uint32_t j = i + (uint32_t)(z % (uint64_t)(d.n - i));
    std::swap(idx[i], idx[j]);
  }
  double *partial = d_diag_;
  double *ref = d_diag_ + (size_t)splits * nt * 3u;
  uint32_t *tgt = reinterpret_cast<uint32_t *>(ref + (size_t)nt * 3u);
  RF_CK(cudaMemcpyAsync(tgt, idx.data(), 4ull * nt, cudaMemcpyHostToDevice, stream_));
  {
    LaunchCtx L = ctx(tree_buf_ < 0 ? mcur_ : (uint32_t)tree_buf_, lpar_, pcur_);
    K().accel_targets(L, scene, d.tile_off, pad_tiles(d.n), d_ids_[pcur_], d_slot_of_, tgt, nt,
                         d_accphi_);
    launches_ += 2;
  }
  launch_direct_sum_f64(stream_, d_part_[pcur_ ^ 1u] + 2ull * d.body_off, d.n, tgt, nt,
                        (double)d.gravity, (double)d.softening, partial, splits, ref);
  RF_CK(cudaGetLastError());
  launches_ += 2;
  std::vector<double> href((size_t)nt * 3u);
  std::vector<float> acc((size_t)nt * 4u);
  RF_CK(cudaMemcpyAsync(href.data(), ref, 8ull * nt * 3u, cudaMemcpyDeviceToHost, stream_));
  RF_CK(cudaMemcpyAsync(acc.data(), d_accphi_, 16ull * nt, cudaMemcpyDeviceToHost, stream_));
  st = sync();
  if (st != RFMM_OK) return st;
  double num = 0.0, den = 0.0, mx = 0.0;
  for (uint32_t t = 0; t < nt; t++) {
    double e2 = 0.0, r2 = 0.0;
    for (int k = 0; k < 3; k++) {
      const double df = (double)acc[4u * t + k] - href[3u * t + k];
      e2 += df * df;
      r2 += href[3u * t + k] * href[3u * t + k];
    }
    num += e2;
    den += r2;
    if (r2 > 0.0) mx = std::max(mx, std::sqrt(e2 / r2));
  }
  if (rms_rel) *rms_rel = den > 0.0 ? std::sqrt(num / den) : 0.0;
  if (max_rel) *max_rel = mx;
  return RFMM_OK;
}

int Engine::render(uint32_t scene, const rfmm_render_params &p, void *dst, size_t bytes,
                   cudaMemcpyKind kind) {
  if (scene >= scenes_.size() || dst == nullptr) return RFMM_ERR_INVALID;
  if (!committed_) return RFMM_ERR_STATE;
  if (p.width == 0u || p.height == 0u || p.width > 16384u || p.height > 16384u) return RFMM_ERR_INVALID;
  if (bytes != 4ull * p.width * p.height) return RFMM_ERR_INVALID;
  const SceneDesc &d = scenes_[scene];
  RenderCamera cam{};
  cam.instances = p.instances ? p.instances : d.n;
  cam.acc_w = (p.width + 1u) / 2u;  // accumulation at half the canvas size (app.js:219-220)
  cam.acc_h = (p.height + 1u) / 2u;
  cam.canvas_w = (float)p.width;
  cam.canvas_h = (float)p.height;
  cam.cos_yaw = (float)std::cos((double)p.yaw);
  cam.sin_yaw = (float)std::sin((double)p.yaw);
  cam.cos_pitch = (float)std::cos((double)p.pitch);
  cam.sin_pitch = (float)std::sin((double)p.pitch);
  cam.zoom = p.zoom;
  cam.aspect = (float)((double)p.width / (double)std::max(1u, p.height));
  cam.exposure = p.exposure;
  cam.point_size = p.point_size;
  cam.population_scale = 0.62f * rf_powf(1048576.0f / std::max((float)cam.instances, 1.0f), 0.14f);
  const size_t texels = (size_t)cam.acc_w * cam.acc_h, pixels = (size_t)p.width * p.height;
  if (d_slot_of_ == nullptr) {
    const int st = alloc((void **)&d_slot_of_, 4ull * slots_);
    if (st != RFMM_OK) return st;
  }
  if (texels > render_texels_) {
    int st = alloc((void **)&d_render_acc_, 32ull * texels);
    if (st == RFMM_OK) st = alloc((void **)&d_render_tex_, 32ull * texels);
    if (st != RFMM_OK) return st;
    render_texels_ = texels;
  }
  uchar4 *out = reinterpret_cast<uchar4 *>(dst);
  if (kind != cudaMemcpyDeviceToDevice) {
    if (pixels > render_pixels_) {
      const int st = alloc((void **)&d_render_out_, 4ull * pixels);
      if (st != RFMM_OK) return st;
      render_pixels_ = pixels;
    }
    out = d_render_out_;
  }
  LaunchCtx L = ctx(mcur_, lpar_, pcur_);
  launch_slot_of(L, d_ids_[pcur_], d_slot_of_, d.tile_off, pad_tiles(d.n));
  launch_render(L, scene, d_slot_of_, cam, d_render_acc_, d_render_tex_, d_render_tex_ + texels, out);
  RF_CK(cudaGetLastError());
  launches_ += 5;
  if (kind != cudaMemcpyDeviceToDevice)
    RF_CK(cudaMemcpyAsync(dst, out, bytes, cudaMemcpyDeviceToHost, stream_));
  return sync();
}

int Engine::diagnostics(uint32_t scene, double out[9]) {
  if (out == nullptr) return RFMM_ERR_INVALID;
  const uint32_t blocks = 4u * (uint32_t)sms_;
  int st = diag_prepare(scene, 9u * blocks + 9u, true);
  if (st != RFMM_OK) return st;
  const SceneDesc &d = scenes_[scene];
  launch_diagnostics(stream_, d_part_[pcur_ ^ 1u] + 2ull * d.body_off, d_accphi_ + d.body_off, d.n,
                     d_diag_, blocks, d_diag_ + 9u * blocks);
  RF_CK(cudaGetLastError());
  launches_ += 2;
  RF_CK(cudaMemcpyAsync(out, d_diag_ + 9u * blocks, 9 * sizeof(double), cudaMemcpyDeviceToHost,
                        stream_));
  return sync();
}

}  // namespace rfmm
