// Host engine: device buffers, scene table, step sequencing and CUDA graphs
// for one or more independent scenes on one GPU.
//
// A plain solve is an engine with one scene; the batched form packs many
// scenes into the same buffers so every kernel covers all of them in one
// launch (per-scene slot ranges aligned to body tiles, per-scene tree cell
// ranges, and one parent work list shared by all scenes).
#pragma once

#include <cstdint>
#include <atomic>
#include <map>
#include <tuple>
#include <vector>

#include <cuda.h>
#include <cuda_runtime.h>

#include "rfmm.h"
#include "rfmm_kernels.h"
#include "rfmm_shared.h"

namespace rfmm {

// Kernel kinds reported by profile_steps.
enum KernelKind { kKUpward = 0, kKM2L, kKL2LNear, kKIntegrate, kKResort, kKNearP2P, kKernelKinds };
static_assert(kKernelKinds == RFMM_KERNEL_KINDS, "kernel kinds of the C ABI");

// Launchers of the kernels whose arithmetic differs between the exact
// contract and the fast float variant.
struct StepLaunchers {
  void (*upward)(const LaunchCtx &, uint32_t, uint32_t);
  void (*m2l)(const LaunchCtx &, uint32_t);
  void (*l2l_near)(const LaunchCtx &, uint32_t);
  void (*integrate)(const LaunchCtx &, uint32_t);
  void (*near_p2p)(const LaunchCtx &, uint32_t);
  void (*accel)(const LaunchCtx &, const uint32_t *, float4 *, uint32_t, uint32_t);
  void (*accel_targets)(const LaunchCtx &, uint32_t, uint32_t, uint32_t, const uint32_t *,
                        uint32_t *, const uint32_t *, uint32_t, float4 *);
};

struct SceneSpec {
  uint32_t n;          // bodies (or, for a slot, the capacity)
  rfmm_params params;  // for a slot: params.depth = deepest tree it must hold (0 = planner)
  bool slot = false;   // reserve buffers but start empty (serving slots)
};

class Engine {
 public:
  // Allocates every buffer for `specs`; returns an RFMM status.
  static int create(const std::vector<SceneSpec> &specs, Engine **out);
  ~Engine();

  int set_stream(cudaStream_t s);
  cudaStream_t stream() const { return stream_; }
  int set_params(uint32_t scene, const rfmm_params &p);
  int set_resort_interval(uint32_t steps);
  int get_tuning(rfmm_tuning *out) const;
  int set_tuning(const rfmm_tuning &t);
  int autotune(uint32_t steps_per_trial, rfmm_tuning *best);

  // Copy a scene's bodies (caller order) into the resident buffer; the new
  // bodies take effect at the next commit().
  int upload(uint32_t scene, const void *src, size_t bytes, cudaMemcpyKind kind);
  // Runs a bounded wait that cannot complete; RFMM_ERR_TIMEOUT when it gave up.
  int check_wait_timeout(uint32_t polls);
  // Every scene's bodies from one device buffer per scene (caller order).
  int upload_all_device(const void *const *src);
  // Every scene's buffer `which` to dst[scene]: one reorder launch, one copy
  // per scene, one synchronisation.
  int download_all(int which, void *const *dst, cudaMemcpyKind kind);
  int seed_galaxy(uint32_t scene);
  // Sort every scene into leaf order and deposit the leaf moments.
  int commit();

  int solve_fields();
  int step(uint32_t steps);

  // Serving slots.  Requests are staged into empty slots of the scratch
  // particle buffer (slot_bodies(slot, scratch_buffer()) as read at staging
  // time) and admitted together: one scene-table copy, one key pass, one
  // radix sort, one tree clear and one gather with deposit into the current
  // buffer for all of them (their keys concatenated in slot order); a slot
  // staged before a resort flipped the buffers is copied across first.
  // Lists are left for refresh_lists().
  struct Admission {
    uint32_t scene, n;
    rfmm_params params;
    uint32_t buffer;  // particle buffer the bodies were staged in
  };
  int activate_many(const std::vector<Admission> &admissions);
  // Finished slots: their bodies back to caller order in their scratch-buffer
  // range (one launch for all), then the slots are emptied; the emptied
  // descriptors reach the device with the next refresh_lists() or admission,
  // which must come before the next step.
  int retire_many(const std::vector<uint32_t> &slots);
  int refresh_lists();
  // Captures the step graphs of every chunk length up to max_len and every
  // buffer parity ahead of time (serving: no capture while requests wait).
  int prepare_graphs(uint32_t max_len);
  // Seconds refresh_lists spent waiting for a pinned list block's last copy.
  double list_wait_seconds() const { return list_wait_s_; }
  // Serving: a slot's bodies in particle buffer `buffer`.  Stage-in writes
  // an empty slot in scratch_buffer() as read at the time (a resort may flip
  // the buffers before admission, which then copies the slot across); a
  // retired slot's result lies in scratch_buffer() as read right after
  // retire_many().  Kernels never touch an inactive slot's range in either
  // buffer.
  float4 *slot_bodies(uint32_t scene, uint32_t buffer) const {
    return d_part_[buffer] + 2ull * scenes_[scene].body_off;
  }
  uint32_t particle_buffer() const { return pcur_.load(); }
  uint32_t scratch_buffer() const { return pcur_.load() ^ 1u; }
  uint32_t capacity(uint32_t scene) const { return scenes_[scene].tile_cap * kTile; }
  bool active(uint32_t scene) const { return scenes_[scene].n != 0u; }
  int sync();

  int download(uint32_t scene, int which, void *dst, size_t bytes, cudaMemcpyKind kind);
  int digest(uint32_t scene, int which, uint32_t *out);
  int phase_times(float ms[7]);
  // Runs `steps` frames with direct launches and CUDA events around every
  // kernel; adds per-kind device time (ms) and launch counts.
  int profile_steps(uint32_t steps, float ms[kKernelKinds], uint32_t launches[kKernelKinds]);
  uint64_t launch_count() const { return launches_; }
  // Timeline mode: graphs captured from now on stamp every step kernel's
  // first-CTA begin and last-CTA end (see rfmm_timeline).
  int set_timeline(bool on);
  int get_timeline(rfmm_timeline *out);
  int device_error(uint32_t *code, uint32_t *info);

  // Diagnostics on the current positions (each runs a field solve first).
  int accelerations(uint32_t scene, float *host_out);  // n x (ax, ay, az, phi), caller order
  int force_error(uint32_t scene, uint32_t targets, uint64_t seed, double *rms_rel, double *max_rel);
  int diagnostics(uint32_t scene, double out[9]);
  // Headless render of a scene's current bodies into an RGBA8 image.
  int render(uint32_t scene, const rfmm_render_params &p, void *dst, size_t bytes, cudaMemcpyKind kind);

  uint32_t num_scenes() const { return (uint32_t)scenes_.size(); }
  const SceneDesc &scene(uint32_t s) const { return scenes_[s]; }
  size_t buffer_bytes(uint32_t scene, int which) const;
  size_t device_bytes() const { return device_bytes_; }
  uint32_t kernels_per_step() const { return near_mode_ == kNearP2P ? 5u + p2p_sort_kernels() : 4u; }
  // Near-field mode of every scene (kNearReference / kNearP2P); a committed
  // state is re-sorted for the new mode.
  int set_near_mode(uint32_t mode);
  uint32_t near_mode() const { return near_mode_; }
  // RFMM_FLOAT_EXACT (the oracle's contract) or RFMM_FLOAT_FAST.
  int set_float_mode(uint32_t mode);
  uint32_t float_mode() const { return float_mode_; }
  uint32_t total_tiles() const { return tiles_; }

 private:
  Engine() = default;
  int alloc(void **p, size_t bytes);
  int build_tensor_maps();
  LaunchCtx ctx(uint32_t mpar, uint32_t lpar, uint32_t ppar) const;
  void enqueue_step(uint32_t mpar, uint32_t lpar, uint32_t ppar,
                    unsigned long long *stamps = nullptr);
  // Refresh of the resident leaf order: bodies of particle buffer `ppar` are
  // bucketed by leaf into the other buffer using the leaf counts of
  // moments buffer `count_par` (the deposit of the current positions).
  void enqueue_resort(uint32_t ppar, uint32_t count_par, unsigned long long *stamps = nullptr);
  uint32_t radix_sort_kernels() const;  // keys + radix sort + gather (uploads)
  uint32_t max_depth_ = 0;
  uint32_t *d_leaf_blocks_ = nullptr;  // leaf counting sort: per-block sums
  // kNearP2P end of step: bodies back to caller order, leaf-key sort, gather
  // with the deposit into `mom_into`, position snapshot and leaf starts.
  void enqueue_p2p_sort(uint32_t mpar, uint32_t lpar, uint32_t ppar, uint4 *mom_into);
  uint32_t p2p_sort_kernels() const { return 4u + 3u * ((key_bits_ + 7u) / 8u); }
  uint32_t near_mode_ = kNearReference;
  uint32_t float_mode_ = RFMM_FLOAT_EXACT;
  const StepLaunchers &K() const;
  float4 *d_pos4_ = nullptr;      // kNearP2P: leaf-sorted positions
  float4 *d_near4_ = nullptr;     // kNearP2P: per-slot pair sums of the step
  uint32_t *d_starts_ = nullptr;  // per-leaf start slots (leaf sorts)
  int launch_chunk(uint32_t len, bool sort_at_end);
  int slot_desc(uint32_t scene, uint32_t n, const rfmm_params &p);  // fill a free slot's descriptor (host)
  // Serving: the host scene table goes to the device whole (from two pinned
  // blocks used in turn) when slot changes made it stale.
  int flush_scenes();
  bool scenes_dirty_ = false;
  SceneDesc *scene_pin_[2] = {nullptr, nullptr};
  cudaEvent_t scene_ev_[2] = {nullptr, nullptr};
  uint32_t scene_buf_ = 0;
  // Tile maps of admissions and retirements: pinned blocks used in turn, each
  // with an event marking its last copy, and their device copies.
  struct MapBlock {
    uint32_t *pin[2] = {nullptr, nullptr};
    cudaEvent_t ev[2] = {nullptr, nullptr};
    uint32_t *dev = nullptr;
    uint32_t next = 0;
  };
  MapBlock admit_map_, retire_map_;
  // Copies the tiles of `scenes` (each slot's padded tiles, in order) into
  // the map's next pinned block and to the device on `stream`; with
  // `counts`, each tile's scene body count follows the tiles (at dev +
  // count).  Returns the tile count.
  int upload_map(MapBlock &m, const std::vector<uint32_t> &scenes, uint32_t *count, cudaStream_t stream,
                 bool counts = false);
  // Serving admissions run on their own stream, overlapping the chunk in
  // flight (they touch only the admitted slots' bodies and cells); the engine
  // stream waits for them before its next kernels.
  cudaStream_t admit_stream_ = nullptr;
  cudaEvent_t admit_ev_ = nullptr;
  // Recorded on the engine stream after each refresh_lists: an admission
  // waits for it, so the whole-table copy of a refresh never lands on top of
  // the admitted slots' descriptors.
  cudaEvent_t refresh_ev_ = nullptr;
  int rebuild_lists();
  int check_device_error();

  int device_ = 0;
  int sms_ = 0;
  uint32_t body_ctas_ = 0;
  uint32_t tree_ctas_ = 0;
  uint32_t body_limit_ = 1;   // resident integrate CTAs per SM
  rfmm_tuning tuning_{};
  void clear_graphs();
  bool use_lists_ = false;  // serving: kernels walk the active tile/task lists
  cudaStream_t stream_ = nullptr;
  cudaStream_t own_stream_ = nullptr;

  std::vector<SceneDesc> scenes_;
  std::vector<uint32_t> tile_scene_h_;
  std::vector<uint32_t> task_scene_h_;
  uint32_t slots_ = 0, tiles_ = 0, cells_ = 0, tasks_ = 0, plist_cap_ = 0, key_bits_ = 18;

  SceneDesc *d_scenes_ = nullptr;
  uint32_t *d_tile_scene_ = nullptr, *d_task_scene_ = nullptr;
  float4 *d_part_[2] = {nullptr, nullptr};
  uint32_t *d_ids_[2] = {nullptr, nullptr};
  SceneMask fresh_{};       // scenes uploaded since the last commit (ids still to number)
  bool any_fresh_ = false;
  void mark_fresh(uint32_t scene) {
    fresh_.bits[scene >> 5] |= 1u << (scene & 31u);
    any_fresh_ = true;
  }
  uint4 *d_mom_[2] = {nullptr, nullptr};
  uint4 *d_mom_scratch_ = nullptr;
  float4 *d_accphi_ = nullptr;    // diagnostics: per-body acceleration + potential
  double *d_diag_ = nullptr;      // diagnostics: FP64 partial sums
  size_t diag_doubles_ = 0;
  uint32_t *d_slot_of_ = nullptr;  // diagnostics / render: caller id -> resident slot
  unsigned long long *d_render_acc_ = nullptr;  // render: fixed-point accumulation
  float4 *d_render_tex_ = nullptr;              // render: two blur textures
  uchar4 *d_render_out_ = nullptr;              // render: staging for host copies
  size_t render_texels_ = 0, render_pixels_ = 0;
  int diag_prepare(uint32_t scene, size_t doubles, bool all_bodies);
  float4 *d_src_ = nullptr;
  float4 *d_aux_ = nullptr;
  uint32_t *d_tile_list_ = nullptr, *d_task_list_ = nullptr, *d_scene_list_ = nullptr;
  std::vector<uint32_t> tile_list_h_, task_list_h_, scene_list_h_;
  // Serving engines refresh the active lists often and while kernels are
  // queued: the lists go to the device from two pinned blocks used in turn
  // ([counts of tiles, tasks, scenes | tiles_ tiles | tasks_ tasks | scenes]), each
  // with an event marking when its last copy finished.  A pageable source
  // would make the copy wait for the queued kernels once it outgrows the
  // driver's staging buffer.
  uint32_t *list_pin_[2] = {nullptr, nullptr};
  cudaEvent_t list_ev_[2] = {nullptr, nullptr};
  uint32_t list_buf_ = 0;
  double list_wait_s_ = 0.0;
  uint32_t *d_choice_ = nullptr;
  float *d_lfield_ = nullptr, *d_fields_ = nullptr;
  WorkItem *d_plist_[2] = {nullptr, nullptr};
  Counters *h_ctr_ = nullptr;  // pinned host copy of the counters (status reads)
  Counters *d_ctr_ = nullptr;
  uint32_t *d_tickets_ = nullptr;
  CUtensorMap *d_tmaps_ = nullptr;
  SortScratch sort_{};
  std::vector<void *> allocations_;
  size_t device_bytes_ = 0;

  // Host-side sequencing state.
  // Particle buffer holding the resident bodies; flipped by the thread that
  // enqueues work, read by serving stage-in threads (particle_buffer()).
  std::atomic<uint32_t> pcur_{0};
  uint32_t mcur_ = 0;    // moment buffer whose leaf level holds the current deposit
  uint32_t lpar_ = 0;    // parent list to write next
  int tree_buf_ = -1;    // moment buffer holding the last complete tree
  bool committed_ = false;
  bool solved_ = false;  // fields hold a solution
  uint32_t resort_interval_ = 16, since_sort_ = 0;
  bool pdl_ = true;  // programmatic dependent launch between step kernels
  std::vector<bool> uploaded_;

  struct Graph {
    cudaGraphExec_t exec;
    uint32_t kernels;  // kernel launches per graph launch
    uint32_t len;      // steps per graph launch
    bool sort_at_end;  // ends with a resort
    int region;        // timeline region (-1: captured without stamps)
  };
  // Timeline records: per captured graph one region of kStampSteps steps x
  // kKernelKinds kinds x 2 words, cleared by the graph's first node.
  static constexpr uint32_t kStampSteps = 64u, kStampRegions = 32u;
  static constexpr uint32_t kStampWordsPerStep = 2u * kKernelKinds;
  bool timeline_ = false;
  uint32_t stamp_regions_used_ = 0;
  unsigned long long *d_stamps_ = nullptr;
  std::map<std::tuple<uint32_t, uint32_t, uint32_t, uint32_t, bool>, Graph> graphs_;
  // The step graph of `len` steps from the given buffer parities (captured
  // and instantiated on first use).
  int capture_chunk(uint32_t len, uint32_t mcur, uint32_t lpar, uint32_t pcur, bool sort_at_end, Graph **out);
  uint64_t launches_ = 0;  // kernels this engine has launched (graph nodes included)
  uint32_t resort_kernels() const { return 4u; }
  cudaEvent_t ev_[8] = {};
};

const char *status_string(int status);
int cuda_status(cudaError_t e);

}  // namespace rfmm
