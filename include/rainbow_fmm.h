/*
 * rainbow_fmm.h -- octree planner C ABI.
 *
 * These are the twelve `#[no_mangle] extern "C"` exports of the reference
 * planner (iskamag/fmm-rainbow src/lib.rs:88-157), restated in C++ with the
 * same symbol names, argument meaning and clamping behaviour, so a host that
 * binds the reference's wasm/cdylib exports binds this library unchanged.
 *
 * Every function is pure and thread-safe and never fails: out-of-range
 * arguments are clamped or mapped to 0 exactly as the reference does.
 * Static strings are owned by the library and are not NUL-terminated in the
 * length they report (the reference returns Rust &str pointer/length pairs).
 */
#ifndef RAINBOW_FMM_H
#define RAINBOW_FMM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Planner constants, src/lib.rs:10-23 and src/rainbow_fmm.wgsl:10-16. */
#define RAINBOW_MIN_DEPTH 4u
#define RAINBOW_MAX_DEPTH 6u
#define RAINBOW_MIN_PARTICLES (1u << 14)
#define RAINBOW_MAX_PARTICLES (1u << 23)
#define RAINBOW_TARGET_PARTICLES_PER_LEAF 8u
#define RAINBOW_WORLD_HALF_EXTENT 1.60f
#define RAINBOW_ADAPTIVE_LEAF_CAPACITY 16u

/* src/lib.rs:88-91 -- always 1. */
uint32_t rainbow_api_version(void);

/* src/lib.rs:93-101 -- the "shader" payload. In this build it is the CUDA
 * source text of the solver kernels (embedded at build time), so the ABI
 * stays complete; the reference returns its WGSL text here. */
const uint8_t *rainbow_shader_ptr(void);
size_t rainbow_shader_len(void);

/* src/lib.rs:103-111 -- the algorithm description string. */
const uint8_t *rainbow_algorithm_ptr(void);
size_t rainbow_algorithm_len(void);

/* src/lib.rs:113-116 -- depth_for_particles(clamp_particle_count(n)). */
uint32_t rainbow_depth_for_particles(uint32_t particles);

/* src/lib.rs:118-125 -- 8^level, or 0 when level > 6. */
uint32_t rainbow_level_cells(uint32_t level);

/* src/lib.rs:127-134 -- (8^level - 1) / 7, or 0 when level > 7. */
uint32_t rainbow_level_offset(uint32_t level);

/* src/lib.rs:136-139 -- total cells of levels 0..=depth, depth clamped to
 * [4, 6]. */
uint32_t rainbow_total_cells(uint32_t depth);

/* src/lib.rs:141-144 -- clamp to [2^14, 2^23]. */
uint32_t rainbow_clamp_particle_count(uint32_t requested);

/* src/lib.rs:146-149 -- power-of-two i32-safe deposit scale of the clamped
 * count. */
float rainbow_fixed_point_scale(uint32_t particles);

/* src/lib.rs:151-157 -- low 32 bits of 3*N + 199*C for the clamped count
 * and clamped depth. */
uint32_t rainbow_linear_work_lo(uint32_t particles, uint32_t depth);

/* Unclamped planner functions (src/lib.rs:26-86 `pub fn`s). The reference's
 * native harness calls these directly (native/main.rs:90-92), which is how
 * scenes below 2^14 bodies get a plan; the exported functions above clamp. */
uint32_t rainbow_plan_depth_unclamped(uint32_t particles);
float rainbow_plan_scale_unclamped(uint32_t particles);
uint64_t rainbow_plan_work_bound_unclamped(uint32_t particles, uint32_t depth);

#ifdef __cplusplus
}
#endif

#endif /* RAINBOW_FMM_H */
