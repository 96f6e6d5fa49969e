// Kernel launch interface used by the host engine.
#pragma once

#include <cstddef>
#include <cstdint>

#include <cuda.h>
#include <cuda_runtime.h>

#include "rfmm_shared.h"

namespace rfmm {

// Most scenes one engine holds (the scene rank sits above an 18-bit Morton
// code in the sort key).
constexpr uint32_t kMaxSceneCount = 1u << 14;

// One bit per scene, passed to kernels by value.
struct SceneMask {
  uint32_t bits[kMaxSceneCount / 32u];
};

// Caller device buffers of up to kUploadChunk scenes for one bulk upload
// launch (null: the scene is skipped), passed by value.
constexpr uint32_t kUploadChunk = 1024u;
struct UploadSources {
  const float4 *p[kUploadChunk];
};

// Device pointers one launch needs; filled by the engine for each step parity.
struct LaunchCtx {
  cudaStream_t stream;
  const SceneDesc *scenes;
  const uint32_t *tile_scene;  // body tile -> scene
  const uint32_t *task_scene;  // upward task -> scene
  float4 *part;                // current particle slots (2 float4 per body)
  uint4 *mom;                  // moments of the current positions (leaf level valid)
  uint4 *mom_next;             // leaf level receives the integrate deposit
  float4 *src;                 // per-cell (com, G*m)
  float4 *aux;                 // per-cell (G*(count-1)/N, density pulse, count) for integrate
  uint32_t *choice;            // per-leaf sample cell of integrate's descent
  float *lfield;               // per-cell M2L result (12 floats)
  float *fields;               // per-cell final field (12 floats, reference layout)
  WorkItem *plist;             // parent list written this step
  const WorkItem *plist_prev;  // parent list of the previous step
  uint32_t plist_cap;
  Counters *ctr;
  uint32_t *tickets;
  const CUtensorMap *tmaps;    // 8 per scene (levels 0..7; 3..6 used)
  uint32_t sms;                // multiprocessors of the device
  uint32_t body_ctas;          // persistent grid of the body passes (resident CTAs)
  uint32_t tree_ctas;          // persistent grid of the upward pass
  uint32_t m2l_ctas;           // persistent grid of the M2L pass
  uint32_t l2l_ctas;           // persistent grid of the L2L + near pass
  bool integrate_dynamic;      // integrate CTAs grab tiles from a counter
  bool m2l_compact;            // M2L variant that lists contributing slots first
  uint32_t m2l_lanes;          // M2L with one lane per target: 0 never, 1 always, 2 long lists
  uint32_t l2l_lanes;          // L2L + near with one lane per target: the same
  uint32_t upward_warps;       // upward with one warp (not one CTA) per subtree: the same
  bool many_scenes;            // the engine holds more than one scene
  const uint32_t *tile_list;   // active body tiles (null: every tile)
  const uint32_t *task_list;   // active upward tasks (null: every task)
  const uint32_t *scene_list;  // active scenes (null: every scene)
  bool pdl;                    // launch step kernels with programmatic stream serialization
  bool p2p;                    // near field by exact pair sums (every scene in kNearP2P)
  float4 *pos4;                // leaf-sorted position snapshot (kNearP2P)
  float4 *near4;               // per-slot P2P pair sums of the step (kNearP2P)
  uint32_t *starts_out;        // per-leaf start table (kNearP2P)
  // Timeline records of this step (2 words per kernel kind, upward, M2L,
  // L2L + near, integrate, resort, P2P near field), or null: no stamps.
  unsigned long long *stamps;
};

// Record of kernel kind `kind` (0..5) within a step's timeline, or null.
inline unsigned long long *stamp_rec(const LaunchCtx &L, uint32_t kind) {
  return L.stamps != nullptr ? L.stamps + 2u * kind : nullptr;
}

// Launch `kernel` on L.stream, with programmatic dependent launch when L.pdl:
// the kernel may start while its predecessor drains and waits for it with
// griddepcontrol.wait before touching shared data.
template <typename... K, typename... A>
inline void launch_step_kernel(const LaunchCtx &L, void (*kernel)(K...), dim3 grid, dim3 block,
                               size_t smem, A &&...args) {
  if (!L.pdl) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = L.stream;
    cudaLaunchKernelEx(&cfg, kernel, static_cast<A &&>(args)...);
    return;
  }
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = L.stream;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, kernel, static_cast<A &&>(args)...);
}

// Tree passes (kernels_tree.cu).
void launch_upward(const LaunchCtx &L, uint32_t list_par, uint32_t tasks);
void launch_m2l(const LaunchCtx &L, uint32_t list_par);
void launch_l2l_near(const LaunchCtx &L, uint32_t list_par);
cudaError_t configure_tree_kernels();

// Body passes (kernels_body.cu).
void launch_integrate(const LaunchCtx &L, uint32_t tiles);
// kNearP2P: exact near-field pair sums of every body into L.near4.
void launch_near_p2p(const LaunchCtx &L, uint32_t tiles);
void launch_deposit(const LaunchCtx &L, uint4 *moments, uint32_t tiles);
// keys/vals of tiles [tile_base, tile_base + tiles), written from index 0.
// Body ids (caller order) are written too for every scene (fresh_ids 1) or
// for the scenes set in *fresh (fresh_ids 2).
// With `tile_map` (device, `tiles` entries) the tiles are tile_map[0 ..]
// instead of [tile_base, tile_base + tiles).
void launch_keys(const LaunchCtx &L, uint32_t *keys, uint32_t *vals, uint32_t *ids, int fresh_ids,
                 uint32_t tiles, uint32_t tile_base, const SceneMask *fresh = nullptr,
                 const uint32_t *tile_map = nullptr);
// Permute the bodies of tiles [tile_base, tile_base + tiles) (perm from index 0),
// or of the tiles tile_map[0 ..] (each scene's tiles among themselves).
// With `pos_out`, also writes each permuted body's position float4 there.
void launch_gather(const LaunchCtx &L, const uint32_t *perm, const float4 *part_in,
                   const uint32_t *ids_in, float4 *part_out, uint32_t *ids_out, uint4 *deposit_into,
                   uint32_t tiles, uint32_t tile_base, float4 *pos_out = nullptr,
                   const uint32_t *tile_map = nullptr);
// Leaf start tables of every kNearP2P scene from the sorted keys.
void launch_leaf_starts(const LaunchCtx &L, const uint32_t *sorted_keys, uint32_t scenes);
// Bodies of tiles [tile_base, tile_base + tiles) (or tile_map[0 ..]) back to
// caller order: out[body_off + id] = part[slot].
void launch_unpermute(const LaunchCtx &L, const uint32_t *ids, float4 *out, uint32_t tile_base,
                      uint32_t tiles, const uint32_t *tile_map = nullptr,
                      const uint32_t *tile_count = nullptr);
// Scene descriptors desc[i] into scenes[index[i]] on `stream` (other entries untouched).
void launch_write_scenes(cudaStream_t stream, SceneDesc *scenes, const uint32_t *index,
                         const SceneDesc *desc, uint32_t count);
// Cleared moments (both buffers), sources and records of the scenes in `which`.
void launch_clear_scenes(const LaunchCtx &L, uint32_t nscenes, const SceneMask &which, uint4 *mom0,
                         uint4 *mom1, float4 *src, float4 *aux);
void launch_initialize(const LaunchCtx &L, float4 *part_out, uint32_t tile_base, uint32_t tiles);
// Bodies of the scenes whose tiles are [tile_base, tile_base + tiles) copied
// from src.p[scene - scene_base] (caller order, 16-byte aligned) into their slots.
void launch_upload_scenes(const LaunchCtx &L, float4 *part, uint32_t tile_base, uint32_t tiles,
                          uint32_t scene_base, const UploadSources &src);
// Self-check of the bounded kernel wait: *status (device) receives
// kDevErrTmaTimeout when a wait that cannot complete gives up after `polls`.
void launch_wait_check(cudaStream_t stream, uint32_t polls, uint32_t *status);
uint32_t body_ctas_per_sm();  // resident 256-thread CTAs per SM of the persistent body passes
// FMM acceleration + potential per body of tiles [tile_base, +tiles), caller order.
void launch_accel(const LaunchCtx &L, const uint32_t *ids, float4 *out, uint32_t tile_base,
                  uint32_t tiles);
// The same for `nt` bodies of one scene given by caller id (out[t] for
// targets[t]); slot_of (one entry per slot) receives the id -> slot map.
void launch_accel_targets(const LaunchCtx &L, uint32_t scene, uint32_t tile_base, uint32_t tiles,
                          const uint32_t *ids, uint32_t *slot_of, const uint32_t *targets,
                          uint32_t nt, float4 *out);

// Headless point-splat renderer (kernels_render.cu).  The camera terms the
// reference's render plan stores in its parameter slots (app.js:141-185).
struct RenderCamera {
  uint32_t instances;        // points drawn (render count)
  uint32_t acc_w, acc_h;     // accumulation texture (half the canvas, rounded up)
  float canvas_w, canvas_h;  // canvas (viewport) size
  float cos_yaw, sin_yaw, cos_pitch, sin_pitch;
  float zoom;                // camera distance in half-extents (Params.speed)
  float aspect;              // canvas width / height
  float exposure;
  float point_size;          // outer blur radius in canvas pixels
  float population_scale;    // 0.62 * (2^20 / instances)^0.14
};
void launch_render(const LaunchCtx &L, uint32_t scene, const uint32_t *slot_of, const RenderCamera &cam,
                   unsigned long long *acc, float4 *tex_a, float4 *tex_b, uchar4 *out);
// slot_of[body_off + id] = resident slot, for the bodies of tiles [tile_base, +tiles).
void launch_slot_of(const LaunchCtx &L, const uint32_t *ids, uint32_t *slot_of, uint32_t tile_base,
                    uint32_t tiles);

// FP64 diagnostics (kernels_diag.cu).
void launch_direct_sum_f64(cudaStream_t stream, const float4 *part_caller, uint32_t n,
                           const uint32_t *targets, uint32_t nt, double gravity, double eps,
                           double *partial, uint32_t splits, double *out);
void launch_diagnostics(cudaStream_t stream, const float4 *part_caller, const float4 *accphi,
                        uint32_t n, double *partial, uint32_t blocks, double *out);

// The step kernels of the fast float variant (kernels_tree.cu and
// kernels_body.cu compiled a second time with RFMM_FAST_FLOAT: contraction
// on, approximate division and square root, hardware reciprocal square root
// for WGSL inverseSqrt).  Same signatures and launch shapes as above.
namespace fast {
void launch_upward(const LaunchCtx &L, uint32_t list_par, uint32_t tasks);
void launch_m2l(const LaunchCtx &L, uint32_t list_par);
void launch_l2l_near(const LaunchCtx &L, uint32_t list_par);
void launch_integrate(const LaunchCtx &L, uint32_t tiles);
void launch_near_p2p(const LaunchCtx &L, uint32_t tiles);
void launch_accel(const LaunchCtx &L, const uint32_t *ids, float4 *out, uint32_t tile_base,
                  uint32_t tiles);
void launch_accel_targets(const LaunchCtx &L, uint32_t scene, uint32_t tile_base, uint32_t tiles,
                          const uint32_t *ids, uint32_t *slot_of, const uint32_t *targets,
                          uint32_t nt, float4 *out);
cudaError_t configure_tree_kernels();
uint32_t body_ctas_per_sm();
}  // namespace fast

// LSD radix sort of (key, value) pairs, 8-bit digits (kernels_sort.cu).
struct SortScratch {
  uint32_t *keys[2];
  uint32_t *vals[2];
  uint32_t *hist;     // 256 * sort tiles
  uint32_t *totals;   // 256
  uint32_t capacity;  // elements
};
uint32_t sort_tiles(uint32_t n);
// Sorts keys[0]/vals[0] over `bits` low bits; returns which buffer holds the result.
int radix_sort(cudaStream_t stream, SortScratch &s, uint32_t n, uint32_t bits);
// Leaf counting sort of every scene's bodies (part_in/ids_in -> part_out/
// ids_out) from the leaf counts in `counts` (moments of the current
// positions).  block_scratch: leaf_sort_blocks(max_depth) words per scene;
// starts: one word per tree cell (left holding each leaf's end slot).
uint32_t leaf_sort_blocks(uint32_t max_depth);
void leaf_counting_sort(const LaunchCtx &L, uint32_t scenes, uint32_t max_depth, const uint4 *counts,
                        uint32_t *block_scratch, uint32_t *starts, const float4 *part_in,
                        const uint32_t *ids_in, float4 *part_out, uint32_t *ids_out, uint32_t tiles);

}  // namespace rfmm
