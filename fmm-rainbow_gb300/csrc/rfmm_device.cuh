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
//
// The fast float variant (RFMM_FAST_FLOAT, namespace rfmm::fast) compiles the
// tree and body kernels a second time with contraction on, approximate
// division and square root, and WGSL inverseSqrt as the hardware reciprocal
// square root: the latitude WGSL itself gives these operations.  The leaf and
// fixed-point arithmetic (unit_coord, cell_of_unit, the deposit rounding) is
// written with explicit round-to-nearest intrinsics or exact scalings, so
// leaf assignment and every integer result are the same in both variants.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "rfmm_shared.h"

#ifdef RFMM_FAST_FLOAT
#define RFMM_KERNEL_NS_BEGIN \
  namespace rfmm {           \
  namespace fast {
#define RFMM_KERNEL_NS_END \
  }                        \
  }
#else
#define RFMM_KERNEL_NS_BEGIN namespace rfmm {
#define RFMM_KERNEL_NS_END }
#endif

RFMM_KERNEL_NS_BEGIN

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
// x / c, correctly rounded, for a constant divisor c with z = RN(1/c): the
// estimate q0 = RN(x z) is corrected once with the exact remainder
// r = fma(-q0, c, x), q = fma(r, z, q0) (Markstein's correction step;
// Brisebarre, Muller & Raina, IEEE Trans. Comput. 53(8), 2004, for known
// divisors).  For the two divisors used (1.6f and 0.70f - 0.30f) the result
// equals IEEE x / c for every binary32 x with |x| >= 2^-100 (checked
// exhaustively by tests/native/const_div_check.c); smaller |x|, where the
// remainder is not exact, take the division, and non-finite estimates are
// already the quotient.
__device__ __forceinline__ float div_by_const(float x, float c, float z) {
  if (fabsf(x) < 0x1p-100f) return x / c;
  const float q0 = __fmul_rn(x, z);
  if (!(fabsf(q0) < __int_as_float(0x7f800000))) return q0;
  const float r = __fmaf_rn(-q0, c, x);
  return __fmaf_rn(r, z, q0);
}
constexpr float kHalfRcp = 0.625f;  // RN(1 / 1.6f)

__device__ __forceinline__ float unit_coord(float p) {
  float n = clampf_d(div_by_const(p, kHalf, kHalfRcp), -0.99999f, 0.99999f);
  return n * 0.5f + 0.5f;
}

__device__ __forceinline__ uint32_t cell_of_unit(float u, uint32_t dim) {
  return (uint32_t)floorf(u * (float)dim);
}

// 2^-l, exact (0 <= l <= 126).
__device__ __forceinline__ float pow2_neg(uint32_t l) { return __int_as_float((int)(127u - l) << 23); }

// cell_center (wgsl:136-142) for one axis at level l: 2.0 / f32(2^l) is
// exactly 2^(1-l), so it is formed from its exponent instead of a division.
__device__ __forceinline__ float cell_center_lv(uint32_t c, uint32_t l) {
  const float w = __int_as_float((int)(128u - l) << 23);
  return (((float)c + 0.5f) * w - 1.0f) * kHalf;
}

// Linear index x + dim * (y + dim * z) for dim = 2^l (wgsl:120-122).
__device__ __forceinline__ uint32_t lin3_lv(uint32_t x, uint32_t y, uint32_t z, uint32_t l) {
  return x | (y << l) | (z << (2u * l));
}

__device__ __forceinline__ uint32_t lin3(uint32_t x, uint32_t y, uint32_t z, uint32_t dim) {
  return x + dim * (y + dim * z);
}

// Level containing local tree cell g (g >= 1), as level_of (wgsl:380-392).
// Level l holds the cells g with (8^l - 1) / 7 <= g < (8^(l+1) - 1) / 7, i.e.
// 8^l <= 7g + 1 < 8^(l+1): l = floor(log2(7g + 1) / 3) (g < 2^28).
__device__ __forceinline__ uint32_t level_of_d(uint32_t g) {
  return (31u - (uint32_t)__clz((int)(7u * g + 1u))) / 3u;
}

// Coordinates of local cell index `i` at level l (x | y << l | z << 2l).
__device__ __forceinline__ void cell_coords_lv(uint32_t i, uint32_t l, uint32_t &x, uint32_t &y,
                                               uint32_t &z) {
  const uint32_t mask = (1u << l) - 1u;
  x = i & mask;
  y = (i >> l) & mask;
  z = i >> (2u * l);
}

// Programmatic dependent launch: a kernel launched with the programmatic
// stream-serialization attribute may start while its predecessor drains;
// grid_dependency_wait() blocks until the predecessor grid has completed and
// its writes are visible, so every kernel calls it before touching data the
// predecessor produced or consumed.  Without the attribute both are no-ops.
__device__ __forceinline__ void grid_dependency_wait() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
}
__device__ __forceinline__ void grid_dependents_may_launch() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Optional per-launch timeline record, two 64-bit words: rec[0] holds the
// largest ~t_begin over the launch's CTAs (so ~rec[0] is the earliest begin)
// and rec[1] the latest t_end, in %globaltimer nanoseconds; both start at 0.
// t_begin is taken after the dependency wait (when the CTA can work), t_end
// when the CTA is done.  A null record costs one predicated branch.
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void stamp_begin(unsigned long long *rec) {
  if (rec != nullptr && threadIdx.x == 0) atomicMax(rec, ~global_ns());
}
// Every thread of the CTA calls it: with a record it waits for the CTA's
// other threads before stamping.
__device__ __forceinline__ void stamp_end(unsigned long long *rec) {
  if (rec != nullptr) {
    __syncthreads();
    if (threadIdx.x == 0) atomicMax(rec + 1, global_ns());
  }
}

// WGSL inverseSqrt (wgsl:179, 654, 670): IEEE 1 / sqrt in the exact
// contract, the hardware reciprocal square root in the fast variant.
#ifdef RFMM_FAST_FLOAT
__device__ __forceinline__ float inv_sqrt(float x) { return rsqrtf(x); }
#else
__device__ __forceinline__ float inv_sqrt(float x) { return 1.0f / sqrtf(x); }
#endif

// pair_field (wgsl:170-203) for a source cell whose centre of mass `src`
// and gravity-times-mass `gm` were precomputed exactly as the reference
// computes them per pair (moment_com_read and G * count / N), in two steps:
// pair_setup forms the offset and 1/r (the long square-root and division
// chain), pair_terms the ten field terms from them.  Callers that keep two
// pairs in flight run both setups before either's terms.
struct PairSetup {
  float rx, ry, rz, gm, inv_r;
};

__device__ __forceinline__ PairSetup pair_setup(float4 src, float tx, float ty, float tz, float eps) {
  PairSetup p;
  p.gm = src.w;
  p.rx = src.x - tx;
  p.ry = src.y - ty;
  p.rz = src.z - tz;
  const float r2 = (p.rx * p.rx + p.ry * p.ry) + p.rz * p.rz + eps * eps;
  p.inv_r = inv_sqrt(r2);
  return p;
}

__device__ __forceinline__ void pair_terms(const PairSetup &p, float out[10]) {
  const float gm = p.gm, rx = p.rx, ry = p.ry, rz = p.rz, inv_r = p.inv_r;
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

__device__ __forceinline__ void pair_field_d(float4 src, float tx, float ty, float tz, float eps,
                                             float out[10]) {
  pair_terms(pair_setup(src, tx, ty, tz, eps), out);
}

// Per-cell terms of integrate's self-leaf and excitation update that depend
// only on the cell's count: (G * f32(count - 1) / f32(N), clamp((f32(count) -
// 16) / 72, 0, 1), count bits, 0) (wgsl:646-656, 703-707), evaluated once per
// cell with the reference's expressions.
__device__ __forceinline__ float4 make_aux(uint32_t count, float gravity, float n_f) {
  const float self_mass = count > 1u ? (float)(count - 1u) / n_f : 0.0f;
  return make_float4(gravity * self_mass,
                     clampf_d(((float)count - (float)kAdaptive) / 72.0f, 0.0f, 1.0f),
                     __uint_as_float(count), 0.0f);
}

// The cell integrate samples for bodies of one leaf (wgsl:625-639) depends
// only on the counts of the leaf's ancestors, so it is resolved once per leaf:
// (level << 28) | local cell index, or kChoiceUnresolved when the leaf's
// subtree root holds at most 16 bodies (then an ancestor above the subtree
// may be the sampled cell and integrate descends itself).
constexpr uint32_t kChoiceUnresolved = 0xFFFFFFFFu;

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

// Per-CTA deposit accumulator: an open-addressing hash table in shared
// memory keyed by global leaf cell.  A CTA reduces the leaf-sorted tiles it
// walks into it and flushes each touched leaf with one set of 32-bit
// reductions, so a leaf holding tens of thousands of bodies receives a few
// global reductions instead of one per warp.  All sums are integers
// modulo 2^32, so the result is independent of order and equals the
// reference's per-body atomics (wgsl:418-421) bit for bit.
struct DepositTable {
  static constexpr uint32_t kSlots = 1024u;
  static constexpr uint32_t kEmpty = 0xFFFFFFFFu;
  static constexpr uint32_t kProbes = 32u;
  uint32_t key[kSlots];
  uint32_t val[4][kSlots];

  __device__ __forceinline__ void clear() {
    for (uint32_t i = threadIdx.x; i < kSlots; i += blockDim.x) {
      key[i] = kEmpty;
      val[0][i] = val[1][i] = val[2][i] = val[3][i] = 0u;
    }
  }

  __device__ __forceinline__ void insert(uint32_t k, uint32_t c, uint32_t sx, uint32_t sy,
                                         uint32_t sz, uint4 *moments) {
    uint32_t h = (k * 2654435761u) >> 22;  // 10-bit multiplicative hash
    for (uint32_t probe = 0; probe < kProbes; probe++) {
      const uint32_t prev = atomicCAS(&key[h], kEmpty, k);
      if (prev == kEmpty || prev == k) {
        atomicAdd(&val[0][h], c);
        atomicAdd(&val[1][h], sx);
        atomicAdd(&val[2][h], sy);
        atomicAdd(&val[3][h], sz);
        return;
      }
      h = (h + 1u) & (kSlots - 1u);
    }
    uint32_t *m = reinterpret_cast<uint32_t *>(moments + k);  // table crowded: go direct
    atomicAdd(m + 0, c);
    atomicAdd(m + 1, sx);
    atomicAdd(m + 2, sy);
    atomicAdd(m + 3, sz);
  }

  __device__ __forceinline__ void flush(uint4 *moments) {
    for (uint32_t i = threadIdx.x; i < kSlots; i += blockDim.x) {
      const uint32_t k = key[i];
      if (k == kEmpty) continue;
      uint32_t *m = reinterpret_cast<uint32_t *>(moments + k);
      atomicAdd(m + 0, val[0][i]);
      atomicAdd(m + 1, val[1][i]);
      atomicAdd(m + 2, val[2][i]);
      atomicAdd(m + 3, val[3][i]);
    }
  }
};

// One body's deposit into the CTA table: lanes with the same leaf are
// grouped (__match_any_sync), their values summed with __reduce_add_sync, and
// the group's lowest lane inserts the totals.
__device__ __forceinline__ void deposit_body(DepositTable &T, uint32_t key, bool active, int32_t qx,
                                             int32_t qy, int32_t qz, uint4 *moments) {
  if (!active) key = DepositTable::kEmpty;
  const uint32_t peers = __match_any_sync(0xFFFFFFFFu, key);
  const uint32_t c = __reduce_add_sync(peers, active ? 1u : 0u);
  const uint32_t sx = __reduce_add_sync(peers, active ? (uint32_t)qx : 0u);
  const uint32_t sy = __reduce_add_sync(peers, active ? (uint32_t)qy : 0u);
  const uint32_t sz = __reduce_add_sync(peers, active ? (uint32_t)qz : 0u);
  if (active && (threadIdx.x & 31u) == (uint32_t)(__ffs(peers) - 1)) T.insert(key, c, sx, sy, sz, moments);
}

// Contiguous range of body tiles handled by this CTA of a persistent grid.
__device__ __forceinline__ void cta_tile_range(uint32_t tiles, uint32_t &t0, uint32_t &t1) {
  const uint32_t per = (tiles + gridDim.x - 1u) / gridDim.x;
  t0 = min(blockIdx.x * per, tiles);
  t1 = min(t0 + per, tiles);
}

// Stage a scene descriptor in shared memory (all threads of the CTA call it).
__device__ __forceinline__ void load_scene(SceneDesc &dst, const SceneDesc *scenes, uint32_t s) {
  __syncthreads();
  if (threadIdx.x < sizeof(SceneDesc) / 4u)
    reinterpret_cast<uint32_t *>(&dst)[threadIdx.x] =
        reinterpret_cast<const uint32_t *>(scenes + s)[threadIdx.x];
  __syncthreads();
}

RFMM_KERNEL_NS_END
