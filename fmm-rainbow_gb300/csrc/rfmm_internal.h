// Host-side helpers shared between the planner, the engine and the C ABI.
#pragma once

#include <cstddef>
#include <cstdint>

namespace rfmm {

// Planner (planner.cpp), unclamped, src/lib.rs:26-86.
uint32_t level_cells(uint32_t level);
uint32_t level_offset(uint32_t level);
uint32_t total_cells(uint32_t depth);
uint32_t depth_for_particles(uint32_t particles);
float fixed_point_scale(uint32_t particles);
uint32_t clamp_particle_count(uint32_t requested);
uint64_t linear_work_bound(uint32_t particles, uint32_t depth);

// Embedded kernel source text (generated at build time).
const char *kernel_source_text();
size_t kernel_source_len();

}  // namespace rfmm
