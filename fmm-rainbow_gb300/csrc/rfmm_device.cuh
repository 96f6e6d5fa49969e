// Device-side definitions shared by the solver kernels.
//
// Buffer layouts are the reference's (src/rainbow_fmm.wgsl:52-73):
//   Particle 32 B = float4 (x, y, z, hue) + float4 (vx, vy, vz, excitation)
//   Moment   16 B = (count u32, sum_x i32, sum_y i32, sum_z i32), fixed point
//   Field    48 B = (ax, ay, az, phi) (Jxx, Jxy, Jxz, Jyy) (Jyz, Jzz, 0, 0)
//
// Floating-point contract: every kernel translation unit is compiled with
// -fmad=false, IEEE division and IEEE square root, so each expression below
// rounds exactly like the CPU oracle (binary32, round-to-nearest, no
// contraction).  The expression trees follow the WGSL source left to right;
// changing an association here changes results bit-wise.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "rfmm_shared.h"

namespace rfmm {

constexpr float kHalf = 1.60f;           // WORLD_HALF_EXTENT, wgsl:12
constexpr uint32_t kAdaptive = 16u;      // ADAPTIVE_LEAF_CAPACITY, wgsl:10

__host__ __device__ __forceinline__ uint32_t level_offset_d(uint32_t l) {
  return ((1u << (3u * l)) - 1u) / 7u;
}

__device__ __forceinline__ float clampf_d(float x, float lo, float hi) {
  return fminf(fmaxf(x, lo), hi);
}

// i32(round(x)): ties-to-even, saturating, NaN -> 0 (cvt.rni.s32.f32).
__device__ __forceinline__ int32_t f2i_rn_sat(float x) { return __float2int_rn(x); }

// (x - y) etc. kept as plain operators: -fmad=false forbids contraction.

// Normalised position u = clamp(p / 1.6, -0.99999, 0.99999) * 0.5 + 0.5 of
// position_cell (wgsl:144-152); the cell at side `dim` is floor(u * dim).
// u * 2^l is exact, so computing u once and scaling per level is bit-identical
// to calling position_cell per level.
__device__ __forceinline__ float unit_coord(float p) {
  float n = clampf_d(p / kHalf, -0.99999f, 0.99999f);
  return n * 0.5f + 0.5f;
}

__device__ __forceinline__ uint32_t cell_of_unit(float u, uint32_t dim) {
  return (uint32_t)floorf(u * (float)dim);
}

// cell_center (wgsl:136-142) for one axis.
__device__ __forceinline__ float cell_center_axis(uint32_t c, uint32_t dim) {
  float w = 2.0f / (float)dim;
  return (((float)c + 0.5f) * w - 1.0f) * kHalf;
}

__device__ __forceinline__ uint32_t lin3(uint32_t x, uint32_t y, uint32_t z, uint32_t dim) {
  return x + dim * (y + dim * z);
}

// Level containing local tree cell g (g >= 1), as level_of (wgsl:380-392).
__device__ __forceinline__ uint32_t level_of_d(uint32_t g) {
  uint32_t level = 1u, start = 1u;
  while (g >= start + (1u << (3u * level))) {
    start += 1u << (3u * level);
    ++level;
  }
  return level;
}

struct Pair10 {
  float v[10];  // ax ay az phi Jxx Jxy Jxz Jyy Jyz Jzz
};

// pair_field (wgsl:170-203) for a source cell whose centre of mass `src`
// and gravity-times-mass `gm` were precomputed exactly as the reference
// computes them per pair (moment_com_read and G * count / N).
__device__ __forceinline__ void pair_field_d(float4 src, float tx, float ty, float tz, float eps,
                                             float out[10]) {
  const float gm = src.w;
  const float rx = src.x - tx, ry = src.y - ty, rz = src.z - tz;
  const float r2 = (rx * rx + ry * ry) + rz * rz + eps * eps;
  const float inv_r = 1.0f / sqrtf(r2);
  const float inv_r3 = inv_r * inv_r * inv_r;
  const float inv_r5 = inv_r3 * inv_r * inv_r;
  const float diagonal = -gm * inv_r3;
  const float tidal = 3.0f * gm * inv_r5;
  out[0] = gm * rx * inv_r3;
  out[1] = gm * ry * inv_r3;
  out[2] = gm * rz * inv_r3;
  out[3] = -gm * inv_r;
  out[4] = diagonal + tidal * rx * rx;
  out[5] = tidal * rx * ry;
  out[6] = tidal * rx * rz;
  out[7] = diagonal + tidal * ry * ry;
  out[8] = tidal * ry * rz;
  out[9] = diagonal + tidal * rz * rz;
}

// Source record of a cell: centre of mass and G * mass (0 for empty cells).
// com = f32(sum) * (1 / (scale * f32(count))), mass = f32(count) / f32(N)
// (wgsl:163-168, 182-183).
__device__ __forceinline__ float4 make_source(uint4 m, float scale, float gravity, float n_f) {
  if (m.x == 0u) return make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  const float inv = 1.0f / (scale * (float)m.x);
  const float mass = (float)m.x / n_f;
  return make_float4((float)(int32_t)m.y * inv, (float)(int32_t)m.z * inv,
                     (float)(int32_t)m.w * inv, gravity * mass);
}

// Warp-level segmented reduction of (count, qx, qy, qz) over runs of equal
// key, followed by one set of 32-bit reductions into `moments` per run.  The
// sums are exact modulo 2^32, so the result equals the reference's per-body
// atomics (wgsl:418-421) bit for bit, whatever the body order.
__device__ __forceinline__ void deposit_segmented(uint32_t key, bool active, int32_t qx, int32_t qy,
                                                  int32_t qz, uint4 *moments) {
  const unsigned lane = threadIdx.x & 31u;
  if (!active) key = 0xFFFFFFFFu;
  uint32_t c = active ? 1u : 0u;
  uint32_t sx = active ? (uint32_t)qx : 0u, sy = active ? (uint32_t)qy : 0u,
           sz = active ? (uint32_t)qz : 0u;
  const uint32_t prev_key = __shfl_up_sync(0xFFFFFFFFu, key, 1);
  const uint32_t next_key = __shfl_down_sync(0xFFFFFFFFu, key, 1);
  const bool head = lane == 0u || prev_key != key;
  const bool tail = lane == 31u || next_key != key;
  const uint32_t heads = __ballot_sync(0xFFFFFFFFu, head);
  const uint32_t le_mask = 0xFFFFFFFFu >> (31u - lane);
  const uint32_t seg_start = 31u - __clz(heads & le_mask);
#pragma unroll
  for (uint32_t off = 1u; off < 32u; off <<= 1) {
    const uint32_t uc = __shfl_up_sync(0xFFFFFFFFu, c, off);
    const uint32_t ux = __shfl_up_sync(0xFFFFFFFFu, sx, off);
    const uint32_t uy = __shfl_up_sync(0xFFFFFFFFu, sy, off);
    const uint32_t uz = __shfl_up_sync(0xFFFFFFFFu, sz, off);
    if (lane >= seg_start + off) {
      c += uc;
      sx += ux;
      sy += uy;
      sz += uz;
    }
  }
  if (tail && key != 0xFFFFFFFFu) {
    uint32_t *m = reinterpret_cast<uint32_t *>(moments + key);
    atomicAdd(m + 0, c);
    atomicAdd(m + 1, sx);
    atomicAdd(m + 2, sy);
    atomicAdd(m + 3, sz);
  }
}

}  // namespace rfmm
