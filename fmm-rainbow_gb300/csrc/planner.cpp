// Octree planner: C++ restatement of the reference planner
// (iskamag/fmm-rainbow src/lib.rs:10-157).
//
// The dense linear octree stores level l at cell offset (8^l - 1) / 7, cells
// of a level in x-fastest order (x + dim * (y + dim * z)).  Depth is the
// smallest d in [4, 6] with 8^d >= ceil(N / 8); the fixed-point deposit scale
// is the largest power of two keeping N * 1.6 * scale below 0.82 * INT32_MAX.
//
// The exported `rainbow_*` symbols keep the reference's names and clamping
// (src/lib.rs:88-157).  The `*_unclamped` helpers expose the reference's
// `pub fn`s, which its native harness calls directly (native/main.rs:90-92).

#include <cmath>
#include <cstdint>

#include "rainbow_fmm.h"
#include "rfmm_internal.h"

namespace rfmm {

uint32_t level_cells(uint32_t level) { return 1u << (3u * level); }  // lib.rs:26-28

uint32_t level_offset(uint32_t level) { return (level_cells(level) - 1u) / 7u; }  // lib.rs:31-33

uint32_t total_cells(uint32_t depth) { return level_offset(depth + 1u); }  // lib.rs:36-38

uint32_t depth_for_particles(uint32_t particles) {  // lib.rs:45-52
  const uint32_t target_cells =
      particles / RAINBOW_TARGET_PARTICLES_PER_LEAF +
      (particles % RAINBOW_TARGET_PARTICLES_PER_LEAF != 0u ? 1u : 0u);
  uint32_t depth = RAINBOW_MIN_DEPTH;
  while (depth < RAINBOW_MAX_DEPTH && level_cells(depth) < target_cells) ++depth;
  return depth;
}

float fixed_point_scale(uint32_t particles) {  // lib.rs:59-69
  const double headroom = 0.82;
  const double worst = static_cast<double>(particles) *
                       static_cast<double>(RAINBOW_WORLD_HALF_EXTENT);
  const double max_scale = headroom * 2147483647.0 / (worst > 1.0 ? worst : 1.0);
  const double exponent = std::floor(std::log2(max_scale));
  return static_cast<float>(std::pow(2.0, exponent));
}

uint32_t clamp_particle_count(uint32_t requested) {  // lib.rs:71-79
  if (requested < RAINBOW_MIN_PARTICLES) return RAINBOW_MIN_PARTICLES;
  if (requested > RAINBOW_MAX_PARTICLES) return RAINBOW_MAX_PARTICLES;
  return requested;
}

uint64_t linear_work_bound(uint32_t particles, uint32_t depth) {  // lib.rs:83-86
  const uint64_t cells = total_cells(depth);
  return static_cast<uint64_t>(particles) * 3u + cells * (189u + 8u + 2u);
}

static uint32_t clamp_depth(uint32_t depth) {
  return depth < RAINBOW_MIN_DEPTH ? RAINBOW_MIN_DEPTH
                                   : (depth > RAINBOW_MAX_DEPTH ? RAINBOW_MAX_DEPTH : depth);
}

}  // namespace rfmm

namespace {
const char kAlgorithm[] = "Sparse p=1 Cartesian FMM / BLDTT-inspired adaptive hierarchy";
}

extern "C" {

uint32_t rainbow_api_version(void) { return 1u; }

const uint8_t *rainbow_shader_ptr(void) {
  return reinterpret_cast<const uint8_t *>(rfmm::kernel_source_text());
}

size_t rainbow_shader_len(void) { return rfmm::kernel_source_len(); }

const uint8_t *rainbow_algorithm_ptr(void) {
  return reinterpret_cast<const uint8_t *>(kAlgorithm);
}

size_t rainbow_algorithm_len(void) { return sizeof(kAlgorithm) - 1u; }

uint32_t rainbow_depth_for_particles(uint32_t particles) {
  return rfmm::depth_for_particles(rfmm::clamp_particle_count(particles));
}

uint32_t rainbow_level_cells(uint32_t level) {
  return level <= RAINBOW_MAX_DEPTH ? rfmm::level_cells(level) : 0u;
}

uint32_t rainbow_level_offset(uint32_t level) {
  return level <= RAINBOW_MAX_DEPTH + 1u ? rfmm::level_offset(level) : 0u;
}

uint32_t rainbow_total_cells(uint32_t depth) {
  return rfmm::total_cells(rfmm::clamp_depth(depth));
}

uint32_t rainbow_clamp_particle_count(uint32_t requested) {
  return rfmm::clamp_particle_count(requested);
}

float rainbow_fixed_point_scale(uint32_t particles) {
  return rfmm::fixed_point_scale(rfmm::clamp_particle_count(particles));
}

uint32_t rainbow_linear_work_lo(uint32_t particles, uint32_t depth) {
  return static_cast<uint32_t>(rfmm::linear_work_bound(
      rfmm::clamp_particle_count(particles), rfmm::clamp_depth(depth)));
}

uint32_t rainbow_plan_depth_unclamped(uint32_t particles) {
  return rfmm::depth_for_particles(particles);
}

float rainbow_plan_scale_unclamped(uint32_t particles) {
  return rfmm::fixed_point_scale(particles);
}

uint64_t rainbow_plan_work_bound_unclamped(uint32_t particles, uint32_t depth) {
  return rfmm::linear_work_bound(particles, depth);
}

}  // extern "C"
