// Structures shared by host code and kernels.
#pragma once

#include <cstdint>

namespace rfmm {

// Bodies are processed in tiles of this many slots; every scene's slot range
// starts on a tile boundary, so a tile (one integrate CTA) never mixes scenes.
constexpr uint32_t kTile = 256u;

// Near-field modes.  Reference: 26 neighbour-cell monopoles at each adaptive
// leaf's centre plus the self-cell monopole (wgsl:521-572, 646-657).  P2P:
// neither; instead every body sums the exact softened pair forces of the
// bodies in the 3x3x3 block of cells around its sample cell (an accuracy
// mode without a reference counterpart).
// Completion tickets of the upward pass, per scene: word 0 counts finished
// groups of kTicketGroup subtrees, words 1.. count each group's finished
// subtrees (two levels, so no single word takes an atomic from every CTA).
constexpr uint32_t kTicketGroup = 64u;
constexpr uint32_t kTicketStride = 16u;  // 1 + up to 8 groups (512 subtrees at depth 6)

constexpr uint32_t kNearReference = 0u;
constexpr uint32_t kNearP2P = 1u;

// One independent scene (a plain solve is a batch of one scene).
struct alignas(16) SceneDesc {
  uint32_t n;          // bodies (particle_count, wgsl:19)
  uint32_t depth;      // leaf level (wgsl:20)
  uint32_t body_off;   // first slot of this scene in the particle arrays
  uint32_t tile_off;   // first body tile of this scene
  uint32_t cell_off;   // first cell of this scene's tree in moments/fields
  uint32_t cells;      // total_cells(depth)
  uint32_t sub_level;  // root level of the 8x8x8-leaf subtrees of the upward pass
  uint32_t task_off;   // first upward task of this scene
  float scale;         // fixed-point deposit scale (control_settings.z)
  float gravity;       // wgsl:30
  float softening;     // wgsl:31
  float dt_eff;        // dt * speed (wgsl:693)
  float n_f;           // f32(particle_count)
  float control_strength;  // control_settings.x
  float control_radius;    // control_settings.y
  uint32_t key_base;   // scene rank shifted above the 3*key_level Morton bits (sort key)
  float control_point[4];      // wgsl:45
  float control_axis_mode[4];  // wgsl:47
  uint32_t key_level;  // level of the fine Morton cells uploads sort by (>= depth)
  uint32_t max_depth;  // deepest tree this scene's buffers hold (serving slots)
  uint32_t tile_cap;   // body tiles reserved for this scene
  uint32_t near_mode;  // kNearReference or kNearP2P
};
static_assert(sizeof(SceneDesc) == 112, "SceneDesc layout");

// Device-side counters and status words of one engine.
struct Counters {
  uint32_t parents[2];   // length of the parent work list, per step parity
  uint32_t error;        // first error code raised by a kernel (0 = none)
  uint32_t error_info;   // kernel-specific detail for `error`
  uint32_t tiles_active; // entries of the active body-tile list (when one is used)
  uint32_t tasks_active; // entries of the active upward-task list (when one is used)
  uint32_t scenes_active; // entries of the active scene list (when one is used)
  uint32_t tile_cursor;  // next body tile for dynamically scheduled integrate CTAs
  uint32_t p2p_cursor;   // next body tile for the near-field pair-sum CTAs
  uint32_t wait_check;   // status word of the bounded-wait self-check
};

enum DeviceError : uint32_t {
  kDevErrNone = 0,
  kDevErrTmaTimeout = 1,     // an mbarrier wait for a bulk tensor copy gave up
  kDevErrListOverflow = 2,   // a work list exceeded its capacity
};

// One M2L/L2L work item: a parent cell whose count exceeds the adaptive leaf
// capacity; its non-empty children are the on-path targets (wgsl:472-476).
struct WorkItem {
  uint32_t scene;
  uint32_t cell;  // local cell index in the scene's tree (level offset included)
};

}  // namespace rfmm
