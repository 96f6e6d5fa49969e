// Allocation-free field solve.
//
// Some hosts of this solver cannot call cudaMalloc: an engine plugin whose
// device memory is owned and budgeted by the host framework, a callback that
// runs where allocating would synchronise the device, or a process whose
// allocator is already exhausted by the host.  For them,
// rfmm_solve_fields_noalloc runs the same field solve as rfmm_solve_fields
// (deposit, upward, M2L, L2L + near) on caller-owned device buffers and keeps
// all of its intermediate data in one file-scope __device__ array of fixed
// size, so it allocates nothing.
//
// Limits and sharing:
//   * at most kMaxBodies = 131,072 bodies (planner depth 4 or 5, at most
//     37,449 cells); the array is about 7.9 MB and every GPU that loads the
//     library holds it until the process exits;
//   * every call shares the one array, which keeps the last call's contents;
//     calls that overlap on the GPU (different streams, or different host
//     threads without ordering) race on it and give wrong results;
//   * the first call on a device resolves the array's device address with
//     cudaGetSymbolAddress and encodes the TMA tensor maps; make that first
//     call before any stream capture;
//   * kernel-side errors (a bounded TMA wait that gave up, a work list over
//     its capacity) land in the array's status word, which the next call
//     clears: after synchronising, read it with rfmm_noalloc_device_error.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <atomic>
#include <cstring>
#include <mutex>

#include "rfmm.h"
#include "rfmm_internal.h"
#include "rfmm_kernels.h"
#include "rfmm_shared.h"

namespace rfmm {
namespace {

constexpr uint32_t kMaxBodies = 1u << 17;
constexpr uint32_t kMaxDepth = 5u;
constexpr uint32_t kMaxCells = 37449u;   // total_cells(5)
constexpr uint32_t kMaxParents = 4681u;  // cells of levels 0..4
constexpr uint32_t kMaxTiles = kMaxBodies / kTile;
constexpr uint32_t kMaxTasks = 64u;      // 8^(5-3) subtrees
constexpr int kMaxDevices = 64;

// Every member starts on a 16-byte boundary: the kernels read these arrays
// with 16-byte vector loads (and TMA), as they read separate allocations.
struct Scratch {
  CUtensorMap tmaps[8];                      // 64-byte aligned TMA descriptors
  alignas(16) SceneDesc scene;
  alignas(16) Counters ctr;
  alignas(16) uint32_t tickets[kTicketStride];
  alignas(16) uint32_t tile_scene[kMaxTiles];  // one scene: all zero
  alignas(16) uint32_t task_scene[kMaxTasks];  // one scene: all zero
  alignas(16) float4 part[2 * kMaxBodies];     // padded copy of the caller's bodies
  alignas(16) uint4 mom_next[kMaxCells];       // leaf level the upward pass zeroes
  alignas(16) float4 src[kMaxCells];
  alignas(16) float lfield[12 * kMaxCells];
  alignas(16) float4 aux[kMaxCells];
  alignas(16) uint32_t choice[kMaxCells];
  alignas(16) WorkItem plist[2][kMaxParents];
};
static_assert(offsetof(Scratch, lfield) % 16 == 0 && offsetof(Scratch, src) % 16 == 0 &&
                  offsetof(Scratch, part) % 16 == 0 && offsetof(Scratch, mom_next) % 16 == 0 &&
                  offsetof(Scratch, aux) % 16 == 0 && offsetof(Scratch, scene) % 16 == 0,
              "scratch arrays must be 16-byte aligned");

static __device__ __align__(256) unsigned char g_scratch[sizeof(Scratch)];

using EncodeTiledFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                   const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                   const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                   CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// `ready` is published with release order after the other fields are set,
// and read with acquire order before they are used, so a thread that sees it
// true also sees the set-up; set-up itself runs under g_setup_mutex.
struct DeviceState {
  std::atomic<bool> ready{false};
  Scratch *scratch = nullptr;  // device address of g_scratch on this device
  int sms = 0;
  uint32_t body_ctas = 0;
};

std::mutex g_setup_mutex;
DeviceState g_state[kMaxDevices];

int cuda_rc(cudaError_t e) {
  if (e == cudaSuccess) return RFMM_OK;
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver || e == cudaErrorNoKernelImageForDevice)
    return RFMM_ERR_NO_DEVICE;
  return RFMM_ERR_CUDA;
}

// Once per device, with that device current: the array's device address,
// kernel attributes and the tensor maps over the array's source records.
int setup_device(int dev, DeviceState &st) {
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (st.ready.load(std::memory_order_relaxed)) return RFMM_OK;
  cudaDeviceProp prop;
  cudaError_t e = cudaGetDeviceProperties(&prop, dev);
  if (e != cudaSuccess) return cuda_rc(e);
  if (prop.major != 10 || prop.minor != 3) return RFMM_ERR_NO_DEVICE;
  void *addr = nullptr;
  e = cudaGetSymbolAddress(&addr, g_scratch);
  if (e != cudaSuccess || addr == nullptr) return e != cudaSuccess ? cuda_rc(e) : RFMM_ERR_CUDA;
  e = configure_tree_kernels();
  if (e != cudaSuccess) return cuda_rc(e);

  void *fn = nullptr;
  cudaDriverEntryPointQueryResult q;
  e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
  if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || fn == nullptr) return RFMM_ERR_NO_DEVICE;
  EncodeTiledFn encode = reinterpret_cast<EncodeTiledFn>(fn);
  Scratch *S = static_cast<Scratch *>(addr);
  CUtensorMap maps[8];
  std::memset(maps, 0, sizeof(maps));
  for (uint32_t l = 3; l <= kMaxDepth; l++) {
    const uint64_t dim = 1ull << l;
    void *base = reinterpret_cast<char *>(S->src) + 16ull * level_offset(l);
    const cuuint64_t gdim[3] = {4 * dim, dim, dim};
    const cuuint64_t gstride[2] = {16 * dim, 16 * dim * dim};
    const cuuint32_t box[3] = {24, 6, 6};
    const cuuint32_t estride[3] = {1, 1, 1};
    if (encode(&maps[l], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, base, gdim, gstride, box, estride,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
               CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return RFMM_ERR_CUDA;
  }
  e = cudaMemcpy(S->tmaps, maps, sizeof(maps), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_rc(e);
  st.scratch = S;
  st.sms = prop.multiProcessorCount;
  st.body_ctas = (uint32_t)st.sms * body_ctas_per_sm();
  st.ready.store(true, std::memory_order_release);
  return RFMM_OK;
}

// The current device's state, set up on first use.
int device_state(DeviceState **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_rc(e);
  if (dev < 0 || dev >= kMaxDevices) return RFMM_ERR_NO_DEVICE;
  DeviceState &st = g_state[dev];
  if (!st.ready.load(std::memory_order_acquire)) {
    const int rc = setup_device(dev, st);
    if (rc != RFMM_OK) return rc;
  }
  *out = &st;
  return RFMM_OK;
}

}  // namespace
}  // namespace rfmm

extern "C" int rfmm_solve_fields_noalloc(const void *device_particles, uint32_t n,
                                         const rfmm_params *params, void *device_moments,
                                         void *device_fields, void *stream) {
  using namespace rfmm;
  if (device_particles == nullptr || device_moments == nullptr || device_fields == nullptr ||
      n == 0u || n > kMaxBodies)
    return RFMM_ERR_INVALID;
  if ((reinterpret_cast<uintptr_t>(device_particles) | reinterpret_cast<uintptr_t>(device_moments) |
       reinterpret_cast<uintptr_t>(device_fields)) % 16u != 0u)
    return RFMM_ERR_INVALID;
  rfmm_params p;
  if (params != nullptr) {
    p = *params;
  } else {
    rfmm_default_params(&p);
  }
  const uint32_t depth = p.depth ? p.depth : depth_for_particles(n);
  if (depth < 4u || depth > kMaxDepth || !(p.fixed_point_scale >= 0.0f)) return RFMM_ERR_INVALID;

  DeviceState *stp = nullptr;
  {
    const int rc = device_state(&stp);
    if (rc != RFMM_OK) return rc;
  }
  const DeviceState &st = *stp;
  Scratch *S = st.scratch;
  cudaError_t e = cudaSuccess;
  cudaStream_t s = static_cast<cudaStream_t>(stream);

  SceneDesc d{};
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
  d.key_level = 10u;
  d.max_depth = depth;
  d.tile_cap = (n + kTile - 1u) / kTile;
  const uint32_t tiles = (n + kTile - 1u) / kTile;
  const uint32_t tasks = 1u << (3u * d.sub_level);

  // Clear what must start at zero: counters, tickets, scene maps, outputs.
  e = cudaMemcpyAsync(&S->scene, &d, sizeof(d), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(&S->ctr, 0, sizeof(Counters), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(S->tickets, 0, sizeof(S->tickets), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(S->tile_scene, 0, sizeof(S->tile_scene), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(S->task_scene, 0, sizeof(S->task_scene), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(device_moments, 0, 16ull * d.cells, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(device_fields, 0, 48ull * d.cells, s);
  // The upward pass trusts that subtrees empty in both moment buffers have
  // cleared sources: start every call from cleared scratch.
  if (e == cudaSuccess) e = cudaMemsetAsync(S->mom_next, 0, sizeof(S->mom_next), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(S->src, 0, sizeof(S->src), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(S->aux, 0, sizeof(S->aux), s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(S->part, device_particles, 32ull * n, cudaMemcpyDeviceToDevice, s);
  if (e != cudaSuccess) return cuda_rc(e);

  LaunchCtx L{};
  L.stream = s;
  L.scenes = &S->scene;
  L.tile_scene = S->tile_scene;
  L.task_scene = S->task_scene;
  L.part = S->part;
  L.mom = static_cast<uint4 *>(device_moments);
  L.mom_next = S->mom_next;
  L.src = S->src;
  L.aux = S->aux;
  L.choice = S->choice;
  L.lfield = S->lfield;
  L.fields = static_cast<float *>(device_fields);
  L.plist = S->plist[0];
  L.plist_prev = S->plist[1];
  L.plist_cap = kMaxParents;
  L.ctr = &S->ctr;
  L.tickets = S->tickets;
  L.tmaps = S->tmaps;
  L.body_ctas = st.body_ctas;
  L.tree_ctas = (uint32_t)st.sms * 6u;
  L.m2l_ctas = (uint32_t)st.sms * 6u;
  L.l2l_ctas = (uint32_t)st.sms * 5u;
  L.integrate_dynamic = false;
  L.tile_list = nullptr;
  L.task_list = nullptr;
  L.pdl = false;

  launch_deposit(L, L.mom, tiles);
  launch_upward(L, 0u, tasks);
  launch_m2l(L, 0u);
  launch_l2l_near(L, 0u);
  return cuda_rc(cudaGetLastError());
}

extern "C" int rfmm_noalloc_device_error(uint32_t *code, uint32_t *info, void *stream) {
  using namespace rfmm;
  DeviceState *st = nullptr;
  const int rc = device_state(&st);
  if (rc != RFMM_OK) return rc;
  // Read behind the work queued on `stream`; the copy goes to a local and
  // the stream is synchronised before it is read.
  Counters c{};
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaMemcpyAsync(&c, &st->scratch->ctr, sizeof(Counters), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_rc(e);
  if (code != nullptr) *code = c.error;
  if (info != nullptr) *info = c.error_info;
  if (c.error == kDevErrTmaTimeout) return RFMM_ERR_TIMEOUT;
  return c.error != 0u ? RFMM_ERR_DEVICE : RFMM_OK;
}
