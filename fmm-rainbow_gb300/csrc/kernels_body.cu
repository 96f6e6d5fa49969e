// Body passes: integrate (L2P + self leaf + kick/drift) fused with the next
// step's deposit, the sort-key and gather passes that keep bodies resident in
// leaf (Morton) order, the standalone deposit, and the galaxy seed.
//
// Reference passes (iskamag/fmm-rainbow src/rainbow_fmm.wgsl):
//   deposit     408-422   leaf cell + i32(round(pos * scale)) atomics
//   integrate   613-771   adaptive descent, local expansion, self leaf,
//                         control field, symplectic Euler, soft wall, hue
//   initialize  232-374   seeded galaxy
//
// Bodies live in HBM in leaf-key order (a permutation of the caller's order,
// undone on download).  Every result is independent of that order: each
// body's update reads only its own state and the tree, and the moment sums
// are exact integers.  Sorted order makes a warp's bodies share leaves, so
// the tree gathers broadcast and the deposit is one reduction per run.
#include <cuda_runtime.h>

#include "rfmm_device.cuh"
#include "rfmm_kernels.h"
#include "rfmm_math.h"

RFMM_KERNEL_NS_BEGIN

// Leaf (level `depth`) cell of a position, local to the scene's tree.
__device__ __forceinline__ uint32_t leaf_cell(float x, float y, float z, uint32_t depth) {
  const uint32_t dim = 1u << depth;
  return level_offset_d(depth) + lin3_lv(cell_of_unit(unit_coord(x), dim),
                                         cell_of_unit(unit_coord(y), dim),
                                         cell_of_unit(unit_coord(z), dim), depth);
}

// 3-D Morton interleave of leaf coordinates (x in bit 0).
__device__ __forceinline__ uint32_t spread3(uint32_t v) {
  v &= 0x3FFu;
  v = (v | (v << 16)) & 0x030000FFu;
  v = (v | (v << 8)) & 0x0300F00Fu;
  v = (v | (v << 4)) & 0x030C30C3u;
  v = (v | (v << 2)) & 0x09249249u;
  return v;
}

__device__ __forceinline__ uint32_t morton3(uint32_t x, uint32_t y, uint32_t z) {
  return spread3(x) | (spread3(y) << 1) | (spread3(z) << 2);
}

__device__ __forceinline__ float length3(float x, float y, float z) {
  return sqrtf((x * x + y * y) + z * z);
}

// Soft absorbing band and last-resort clamp for one axis (wgsl:740-751).
__device__ __forceinline__ void soft_wall(float &p, float &v, float world_edge, float edge_band) {
  const float over = fabsf(p) - (world_edge - edge_band);
  if (over > 0.0f) {
    const float absorb = clampf_d(over / edge_band, 0.0f, 1.0f);
    v = v * (1.0f - absorb * 0.16f);
  }
  if (fabsf(p) > world_edge) {
    p = clampf_d(p, -world_edge, world_edge);
    v = v * -0.55f;
  }
}

// Near-field P2P inputs: the leaf-sorted position snapshot, the per-leaf
// start table (Morton order, absolute slots, 8^depth + 1 entries per scene at
// the scene's cell offset), the body's own slot, and (integrate) the pair
// sums k_near_p2p already formed for every slot, or null: form them here.
struct P2PView {
  const float4 *pos;
  const uint32_t *starts;
  uint32_t self;
  const float4 *near = nullptr;
};

// The cell a body samples its field from (wgsl:625-639): the first level
// whose cell holds at most 16 bodies, else the leaf level.  Resolved once per
// leaf by the upward pass; bodies of unresolved leaves (sparse subtrees)
// descend here.  Returns the global cell index; `level` and the leaf
// coordinates (lx, ly, lz) describe it (coordinates at the level are the
// leaf coordinates shifted right by depth - level).
__device__ __forceinline__ uint32_t sample_cell(const SceneDesc &S, float px, float py, float pz,
                                                const uint4 *__restrict__ mom,
                                                const uint32_t *__restrict__ choice,
                                                uint32_t &level, uint32_t &lx, uint32_t &ly,
                                                uint32_t &lz) {
  const uint32_t D = S.depth;
  // Leaf coordinates; floor(u * 2^l) == floor(u * 2^D) >> (D - l).
  const uint32_t dimD = 1u << D;
  lx = cell_of_unit(unit_coord(px), dimD);
  ly = cell_of_unit(unit_coord(py), dimD);
  lz = cell_of_unit(unit_coord(pz), dimD);
  uint32_t chosen = D, cell_index = 0u;
  const uint32_t pick = __ldg(&choice[S.cell_off + level_offset_d(D) + lin3_lv(lx, ly, lz, D)]);
  if (pick != kChoiceUnresolved) {
    chosen = pick >> 28;
    cell_index = S.cell_off + (pick & 0x0FFFFFFFu);
  } else {
#pragma unroll
    for (uint32_t l = 6u; l >= 1u; l--) {
      if (l <= D) {
        const uint32_t sh = D - l;
        const uint32_t idx = S.cell_off + level_offset_d(l) + lin3_lv(lx >> sh, ly >> sh, lz >> sh, l);
        const uint32_t c = __ldg(&mom[idx].x);
        if ((int32_t)c <= (int32_t)kAdaptive || l == D) {
          chosen = l;
          cell_index = idx;
        }
      }
    }
  }
  level = chosen;
  return cell_index;
}

// Softened pair sums over the bodies of the 3x3x3 cells (level `l`) around
// cell (cx, cy, cz): cells z-, y-, x-major from -1 to +1, bodies of a cell in
// (leaf Morton code, caller id) order, the body itself skipped.
template <bool kPhi>
__device__ __forceinline__ void p2p_sums(const SceneDesc &S, const P2PView &V, uint32_t l,
                                         uint32_t cx, uint32_t cy, uint32_t cz, float px, float py,
                                         float pz, float &sx, float &sy, float &sz, float &sp) {
  const int dim = 1 << l;
  const uint32_t sh3 = 3u * (S.depth - l);
  const float eps2 = S.softening * S.softening;
  sx = 0.0f;
  sy = 0.0f;
  sz = 0.0f;
  sp = 0.0f;
  for (int oz = -1; oz <= 1; oz++) {
    const int nz = (int)cz + oz;
    if (nz < 0 || nz >= dim) continue;
    for (int oy = -1; oy <= 1; oy++) {
      const int ny = (int)cy + oy;
      if (ny < 0 || ny >= dim) continue;
      for (int ox = -1; ox <= 1; ox++) {
        const int nx = (int)cx + ox;
        if (nx < 0 || nx >= dim) continue;
        const uint32_t m = morton3((uint32_t)nx, (uint32_t)ny, (uint32_t)nz);
        const uint32_t lo = __ldg(&V.starts[S.cell_off + (m << sh3)]);
        const uint32_t hi = __ldg(&V.starts[S.cell_off + ((m + 1u) << sh3)]);
        for (uint32_t j = lo; j < hi; j++) {
          if (j == V.self) continue;
          const float4 q = __ldg(&V.pos[j]);
          const float dx = q.x - px, dy = q.y - py, dz = q.z - pz;
          const float r2 = ((dx * dx + dy * dy) + dz * dz) + eps2;
          const float inv = inv_sqrt(r2);
          const float w = (inv * inv) * inv;
          sx = sx + dx * w;
          sy = sy + dy * w;
          sz = sz + dz * w;
          if (kPhi) sp = sp + inv;
        }
      }
    }
  }
}

// FMM acceleration at a body (wgsl:619-657): adaptive descent to the sample
// cell, local expansion about its centre, softened self-leaf monopole (or,
// with kP2P, the exact near-field pair sums instead).  With `phi`, also the
// potential of the same expansion (diagnostics only; integrate never
// evaluates it).  Returns the sample cell's count.
template <bool kPhi, bool kP2P = false>
__device__ __forceinline__ uint32_t body_acceleration(const SceneDesc &S, float px, float py, float pz,
                                                      const uint4 *__restrict__ mom,
                                                      const float4 *__restrict__ src,
                                                      const float4 *__restrict__ aux,
                                                      const uint32_t *__restrict__ choice,
                                                      const float *__restrict__ fields, float &ax,
                                                      float &ay, float &az, float &pulse,
                                                      float *phi, const P2PView *V = nullptr) {
    const uint32_t D = S.depth;
    uint32_t chosen, lx, ly, lz;
    const uint32_t cell_index = sample_cell(S, px, py, pz, mom, choice, chosen, lx, ly, lz);
    const float4 ax4 = __ldg(&aux[cell_index]);
    const uint32_t count = __float_as_uint(ax4.z);
    const uint32_t csh = D - chosen;
    const float cx = cell_center_lv(lx >> csh, chosen);
    const float cy = cell_center_lv(ly >> csh, chosen);
    const float cz = cell_center_lv(lz >> csh, chosen);

    const float4 *fp = reinterpret_cast<const float4 *>(fields + (size_t)cell_index * 12u);
    const float4 fa = __ldg(fp), fj0 = __ldg(fp + 1), fj1 = __ldg(fp + 2);
    const float rx = px - cx, ry = py - cy, rz = pz - cz;
    ax = fa.x + (fj0.x * rx + fj0.y * ry + fj0.z * rz);
    ay = fa.y + (fj0.y * rx + fj0.w * ry + fj1.x * rz);
    az = fa.z + (fj0.z * rx + fj1.x * ry + fj1.y * rz);

    if (kP2P) {
      float sx, sy, sz, sp = 0.0f;
      if (!kPhi && V->near != nullptr) {
        const float4 nr = V->near[V->self];
        sx = nr.x;
        sy = nr.y;
        sz = nr.z;
      } else {
        p2p_sums<kPhi>(S, *V, chosen, lx >> csh, ly >> csh, lz >> csh, px, py, pz, sx, sy, sz, sp);
      }
      const float gm = S.gravity / S.n_f;
      ax = ax + gm * sx;
      ay = ay + gm * sy;
      az = az + gm * sz;
      if (kPhi) *phi = (fa.w - ((fa.x * rx + fa.y * ry) + fa.z * rz)) - gm * sp;
      pulse = ax4.y;
      return count;
    }

    // Self leaf: softened monopole of the other count-1 bodies (wgsl:646-657).
    // x / 2^l == x * 2^-l exactly, so the eps division is a scaling.
    if (count > 1u) {
      const float4 s = __ldg(&src[cell_index]);
      const float dx = s.x - px, dy = s.y - py, dz = s.z - pz;
      const float eps = fmaxf(S.softening, (0.62f * kHalf) * pow2_neg(chosen));
      const float inv_r = inv_sqrt((dx * dx + dy * dy) + dz * dz + eps * eps);
      const float gsm = ax4.x;  // G * f32(count - 1) / f32(N)
#ifdef RFMM_FAST_FLOAT
      // One weight for the three components (reassociated: fast variant only).
      const float w = gsm * ((inv_r * inv_r) * inv_r);
      ax = ax + dx * w;
      ay = ay + dy * w;
      az = az + dz * w;
#else
      ax = ax + gsm * dx * inv_r * inv_r * inv_r;
      ay = ay + gsm * dy * inv_r * inv_r * inv_r;
      az = az + gsm * dz * inv_r * inv_r * inv_r;
#endif
    }

    if (kPhi) {
      float p = fa.w - ((fa.x * rx + fa.y * ry) + fa.z * rz);
      if (count > 1u) {
        const float4 s = __ldg(&src[cell_index]);
        const float dx = s.x - px, dy = s.y - py, dz = s.z - pz;
        const float eps = fmaxf(S.softening, (0.62f * kHalf) * pow2_neg(chosen));
        p = p - ax4.x / sqrtf((dx * dx + dy * dy) + dz * dz + eps * eps);
      }
      *phi = p;
    }
    pulse = ax4.y;  // clamp((f32(count) - 16) / 72, 0, 1)
    return count;
}

// One body's integrate (wgsl:613-771).  Writes the new state into p0/p1 and
// the new position's leaf cell and fixed-point coordinates (the next deposit).
template <bool kP2P>
__device__ __forceinline__ void integrate_body(const SceneDesc &S, float4 &p0, float4 &p1,
                                               const uint4 *__restrict__ mom,
                                               const float4 *__restrict__ src,
                                               const float4 *__restrict__ aux,
                                               const uint32_t *__restrict__ choice,
                                               const float *__restrict__ fields, uint32_t &key,
                                               int32_t &qx, int32_t &qy, int32_t &qz,
                                               const P2PView *V) {
    float px = p0.x, py = p0.y, pz = p0.z;
    float vx = p1.x, vy = p1.y, vz = p1.z;
    const uint32_t D = S.depth;
    float ax, ay, az, density_pulse;
    body_acceleration<false, kP2P>(S, px, py, pz, mom, src, aux, choice, fields, ax, ay, az,
                                   density_pulse, nullptr, V);

    // Interactive control field (wgsl:659-689); off unless control_point.w > 0.5.
    float control_influence = 0.0f;
    if (S.control_point[3] > 0.5f) {
      const float cdx = S.control_point[0] - px, cdy = S.control_point[1] - py,
                  cdz = S.control_point[2] - pz;
      const float d2 = (cdx * cdx + cdy * cdy) + cdz * cdz;
      const float cr = fmaxf(S.control_radius, 0.02f);
      control_influence = rf_expf(-2.0f * d2 / (cr * cr));
      const float strength = S.control_strength;
      const float inv = inv_sqrt(d2 + cr * cr * 0.018f);
      const float dirx = cdx * inv, diry = cdy * inv, dirz = cdz * inv;
      const float mode = S.control_axis_mode[3];
      if (mode < 1.5f) {
        ax = ax + dirx * strength * control_influence;
        ay = ay + diry * strength * control_influence;
        az = az + dirz * strength * control_influence;
      } else if (mode < 2.5f) {
        ax = ax - dirx * strength * control_influence;
        ay = ay - diry * strength * control_influence;
        az = az - dirz * strength * control_influence;
      } else {
        const float al = length3(S.control_axis_mode[0], S.control_axis_mode[1], S.control_axis_mode[2]);
        const float nx = S.control_axis_mode[0] / al, ny = S.control_axis_mode[1] / al,
                    nz = S.control_axis_mode[2] / al;
        const float tx = ny * cdz - nz * cdy, ty = nz * cdx - nx * cdz, tz = nx * cdy - ny * cdx;
        const float tl = length3(tx, ty, tz);
        if (tl > 0.00001f) {
          ax = ax + tx / tl * strength * control_influence;
          ay = ay + ty / tl * strength * control_influence;
          az = az + tz / tl * strength * control_influence;
        }
      }
    }

    // Symplectic Euler with excitation and hue state (wgsl:691-769).
    const float dt = S.dt_eff;
    const float radius = fmaxf(length3(px, py, pz), 0.0001f);
    const float vlen = fmaxf(length3(vx, vy, vz), 0.0001f);
    const float pv = (px * vx + py * vy) + pz * vz;
    const float signed_radial = clampf_d(pv / (radius * vlen), -1.0f, 1.0f);
    const float rf = fabsf(signed_radial);
    const float radial_shock = rf * rf * rf;
    const float field_strength = clampf_d(length3(ax, ay, az) * (radius + 0.12f) * 0.58f, 0.0f, 1.0f);
    const float target_exc = clampf_d(0.025f + radial_shock * 0.56f + density_pulse * 0.26f +
                                          field_strength * 0.13f + control_influence * 0.42f,
                                      0.0f, 1.0f);
    float exc = p1.w;
    const float response = target_exc > exc ? 10.0f : 1.05f;
    const float t = clampf_d(dt * response, 0.0f, 1.0f);
    exc = exc * (1.0f - t) + target_exc * t;

    vx = vx + ax * dt;
    vy = vy + ay * dt;
    vz = vz + az * dt;
    px = px + vx * dt;
    py = py + vy * dt;
    pz = pz + vz * dt;

    const float world_edge = kHalf * 0.985f;
    const float edge_band = 0.12f * kHalf;
    soft_wall(px, vx, world_edge, edge_band);
    soft_wall(py, vy, world_edge, edge_band);
    soft_wall(pz, vz, world_edge, edge_band);
    constexpr float kWidth = 0.70f - 0.30f, kWidthRcp = 0x1.400002p+1f;  // RN(1 / kWidth)
    const float st = clampf_d(div_by_const(exc - 0.30f, kWidth, kWidthRcp), 0.0f, 1.0f);
    const float hue_drift = 1.0f - st * st * (3.0f - 2.0f * st);
    const float hsum = p0.w + dt * hue_drift *
                                  (0.012f + signed_radial * 0.030f + exc * 0.036f +
                                   control_influence * 0.080f);
    const float hue = hsum - floorf(hsum);
    p0 = make_float4(px, py, pz, hue);
    p1 = make_float4(vx, vy, vz, exc);

    // The next step's deposit (wgsl:414-421 on the new position).
    key = S.cell_off + leaf_cell(px, py, pz, D);
    qx = f2i_rn_sat(px * S.scale);
    qy = f2i_rn_sat(py * S.scale);
    qz = f2i_rn_sat(pz * S.scale);
}

// Persistent integrate: CTA c of G walks body tiles c, c + G, c + 2G, ...
// (each tile is 256 leaf-sorted, spatially compact bodies; interleaving the
// tiles spreads dense and sparse regions, whose per-body costs differ, evenly
// over the CTAs), integrates every body and accumulates the next step's
// deposit in a shared-memory table flushed once at the end.
//
// kP2P: near field by exact pair sums over the leaf-sorted position snapshot;
// no deposit (the end-of-step sort deposits the new positions).
// Six resident CTAs per SM (40 registers): more warps to cover the latency of
// the per-body dependent chain (measured: 6 CTAs beat 4 and 8).
template <bool kP2P>
__global__ void __launch_bounds__(256, 6) k_integrate(const SceneDesc *__restrict__ scenes,
                                                   const uint32_t *__restrict__ tile_scene,
                                                   float4 *__restrict__ part,
                                                   const uint4 *__restrict__ mom,
                                                   const float4 *__restrict__ src,
                                                   const float4 *__restrict__ aux,
                                                   const uint32_t *__restrict__ choice,
                                                   const float *__restrict__ fields,
                                                   uint4 *__restrict__ mom_next, uint32_t tiles,
                                                   const uint32_t *__restrict__ tile_list,
                                                   Counters *__restrict__ ctr, int dynamic,
                                                   const float4 *__restrict__ pos4,
                                                   const uint32_t *__restrict__ starts,
                                                   const float4 *__restrict__ near4,
                                                   unsigned long long *__restrict__ stamp) {
  __shared__ DepositTable T;
  __shared__ SceneDesc S;
  __shared__ uint32_t s_next;
  if (!kP2P) T.clear();
  grid_dependency_wait();  // fields of this step are complete
  stamp_begin(stamp);
  const uint32_t ntiles = tile_list != nullptr ? min(ctr->tiles_active, tiles) : tiles;
  // Static schedule: interleaved tiles.  Dynamic: tiles are taken one at a
  // time from a counter (reset by this step's upward pass).
  auto grab = [&]() -> uint32_t {
    __syncthreads();
    if (threadIdx.x == 0) s_next = atomicAdd(&ctr->tile_cursor, 1u);
    __syncthreads();
    return s_next;
  };
  // Static schedule: runs of `run` consecutive tiles, interleaved over the
  // CTAs (CTA c takes runs c, c + G, ...).  Single tiles balance best; with
  // at least 16 tiles per CTA (many scenes, whose tiles are contiguous) runs
  // of 4 make the tile's scene change, and its descriptor reload, rarer.
  const uint32_t end = ntiles;
  const uint32_t run_log2 = end >= 16u * gridDim.x ? 2u : 0u;
  uint32_t k = 0u;  // this CTA's static tile count so far
  auto static_tile = [&](uint32_t kk) {
    return (((kk >> run_log2) * gridDim.x + blockIdx.x) << run_log2) + (kk & ((1u << run_log2) - 1u));
  };
  uint32_t i = dynamic ? grab() : static_tile(k);
  uint32_t cur = 0xFFFFFFFFu;
  // The next tile's bodies are loaded one iteration ahead.
  float4 n0 = make_float4(0.f, 0.f, 0.f, 0.f), n1 = n0;
  uint32_t next_tile = i < end ? (tile_list != nullptr ? tile_list[i] : i) : 0u;
  if (i < end) {
    n0 = part[2u * (next_tile * kTile + threadIdx.x)];
    n1 = part[2u * (next_tile * kTile + threadIdx.x) + 1u];
  }
  while (i < end) {
    const uint32_t tile = next_tile;
    const uint32_t slot = tile * kTile + threadIdx.x;
    float4 p0 = n0, p1 = n1;
    const uint32_t ni = dynamic ? grab() : static_tile(++k);
    if (ni < end) {
      next_tile = tile_list != nullptr ? tile_list[ni] : ni;
      n0 = part[2u * (next_tile * kTile + threadIdx.x)];
      n1 = part[2u * (next_tile * kTile + threadIdx.x) + 1u];
    }
    i = ni;
    // The CTA's last tile: the next step's upward pass may launch now (it
    // waits for this whole grid before reading anything); its CTAs take SM
    // slots as this grid's CTAs leave.
    if (ni >= end) grid_dependents_may_launch();
    const uint32_t sc = tile_scene[tile];
    if (sc != cur) {
      load_scene(S, scenes, sc);
      cur = sc;
    }
    const bool active = slot - S.body_off < S.n;
    uint32_t key = DepositTable::kEmpty;
    int32_t qx = 0, qy = 0, qz = 0;
    if (active) {
      const P2PView V{pos4, starts, slot, near4};
      integrate_body<kP2P>(S, p0, p1, mom, src, aux, choice, fields, key, qx, qy, qz, &V);
      part[2u * slot] = p0;
      part[2u * slot + 1u] = p1;
    }
    if (!kP2P) deposit_body(T, key, active, qx, qy, qz, mom_next);
  }
  if (!kP2P) {
    __syncthreads();
    T.flush(mom_next);
  }
  stamp_end(stamp);
  grid_dependents_may_launch();
}

// ------------------------------------------------------------ P2P near field
//
// Exact softened pair sums of every body over the bodies of the 3x3x3 cells
// around its sample cell (kNearP2P), written per slot for the integrate that
// follows.  Persistent CTAs walk interleaved tiles of 256 leaf-sorted bodies.
// A tile whose bodies all share one sample cell (the common case: a dense
// leaf holds thousands of bodies) stages its 27 cells' sources as coalesced
// float4 chunks in shared memory and every thread reads each source by
// broadcast; otherwise each warp whose bodies share a sample cell does the
// same with its own 32-source slice, and the remaining bodies gather their
// sources themselves.  Every thread sums in the same fixed order (cells z-,
// y-, x-major, bodies in slot order, itself skipped) whichever way its
// sources arrive, so the sums equal p2p_sums bit for bit under the exact
// contract.

// One source's contribution (the expression p2p_sums evaluates).
__device__ __forceinline__ void p2p_pair(float4 q, float px, float py, float pz, float eps2,
                                         float &sx, float &sy, float &sz) {
  const float dx = q.x - px, dy = q.y - py, dz = q.z - pz;
  const float r2 = ((dx * dx + dy * dy) + dz * dz) + eps2;
  const float inv = inv_sqrt(r2);
  const float w = (inv * inv) * inv;
  sx = sx + dx * w;
  sy = sy + dy * w;
  sz = sz + dz * w;
}

// Sources [lo, hi) through a staging buffer of kWidth float4 shared by the
// kWidth threads of a group (a CTA or a warp); `sync` orders the group.
template <uint32_t kWidth, typename Sync>
__device__ __forceinline__ void p2p_staged_range(const float4 *__restrict__ pos, uint32_t lo,
                                                 uint32_t hi, float4 *buf, uint32_t rank,
                                                 uint32_t self, float px, float py, float pz,
                                                 float eps2, float &sx, float &sy, float &sz,
                                                 Sync sync) {
  for (uint32_t base = lo; base < hi; base += kWidth) {
    sync();  // the previous chunk is consumed
    if (base + rank < hi) buf[rank] = __ldg(&pos[base + rank]);
    sync();
    const uint32_t m = min(kWidth, hi - base);
    if (self - base < m) {  // this chunk holds the body itself: skip it
      for (uint32_t k = 0; k < m; k++)
        if (base + k != self) p2p_pair(buf[k], px, py, pz, eps2, sx, sy, sz);
    } else {
#ifdef RFMM_FAST_FLOAT
      // Two partial sums (even and odd sources) give each thread two
      // independent chains; the fast variant does not keep the reference
      // summation order.
      float ax = 0.0f, ay = 0.0f, az = 0.0f, bx = 0.0f, by = 0.0f, bz = 0.0f;
      uint32_t k = 0;
#pragma unroll 2
      for (; k + 1u < m; k += 2u) {
        p2p_pair(buf[k], px, py, pz, eps2, ax, ay, az);
        p2p_pair(buf[k + 1u], px, py, pz, eps2, bx, by, bz);
      }
      if (k < m) p2p_pair(buf[k], px, py, pz, eps2, ax, ay, az);
      sx = sx + (ax + bx);
      sy = sy + (ay + by);
      sz = sz + (az + bz);
#else
#pragma unroll 4
      for (uint32_t k = 0; k < m; k++) p2p_pair(buf[k], px, py, pz, eps2, sx, sy, sz);
#endif
    }
  }
}

// Slot range [lo, hi) of neighbour j (0..26, in the reference's z-, y-,
// x-major order) of cell (cx, cy, cz) at level l; false when j lies outside
// the grid.
__device__ __forceinline__ bool neighbour_range(const SceneDesc &S, const uint32_t *starts,
                                                uint32_t l, uint32_t cx, uint32_t cy, uint32_t cz,
                                                uint32_t j, uint32_t &lo, uint32_t &hi) {
  const int dim = 1 << l;
  const int nx = (int)cx + (int)(j % 3u) - 1, ny = (int)cy + (int)((j / 3u) % 3u) - 1,
            nz = (int)cz + (int)(j / 9u) - 1;
  if (nx < 0 || ny < 0 || nz < 0 || nx >= dim || ny >= dim || nz >= dim) return false;
  const uint32_t sh3 = 3u * (S.depth - l);
  const uint32_t m = morton3((uint32_t)nx, (uint32_t)ny, (uint32_t)nz);
  lo = __ldg(&starts[S.cell_off + (m << sh3)]);
  hi = __ldg(&starts[S.cell_off + ((m + 1u) << sh3)]);
  return true;
}

struct CtaSync {
  __device__ __forceinline__ void operator()() const { __syncthreads(); }
};
struct WarpSync {
  __device__ __forceinline__ void operator()() const { __syncwarp(); }
};

__global__ void __launch_bounds__(256, 4) k_near_p2p(const SceneDesc *__restrict__ scenes,
                                                  const uint32_t *__restrict__ tile_scene,
                                                  const float4 *__restrict__ pos4,
                                                  const uint32_t *__restrict__ starts,
                                                  const uint4 *__restrict__ mom,
                                                  const uint32_t *__restrict__ choice,
                                                  uint32_t tiles,
                                                  const uint32_t *__restrict__ tile_list,
                                                  Counters *__restrict__ ctr,
                                                  float4 *__restrict__ near_out,
                                                  unsigned long long *__restrict__ stamp) {
  __shared__ float4 buf[kTile];
  __shared__ SceneDesc S;
  __shared__ uint32_t s_cell[5];  // tid 0's sample cell: key, level, x, y, z
  __shared__ uint32_t s_next;
  const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
  grid_dependency_wait();  // the upward pass resolved this step's sample cells
  stamp_begin(stamp);
  const uint32_t ntiles = tile_list != nullptr ? min(ctr->tiles_active, tiles) : tiles;
  // Tiles are taken one at a time from a counter (reset by this step's
  // upward pass): a tile's cost is its bodies times the sources around their
  // sample cell, which spans two orders of magnitude between sparse and
  // core leaves, so a static share leaves most SMs idle behind the heaviest.
  auto grab = [&]() -> uint32_t {
    __syncthreads();
    if (tid == 0) s_next = atomicAdd(&ctr->p2p_cursor, 1u);
    __syncthreads();
    return s_next;
  };
  uint32_t cur = 0xFFFFFFFFu;
  for (uint32_t i = grab(); i < ntiles; i = grab()) {
    const uint32_t tile = tile_list != nullptr ? tile_list[i] : i;
    const uint32_t sc = tile_scene[tile];
    if (sc != cur) {
      load_scene(S, scenes, sc);  // barriers inside: the previous tile's buffer is free
      cur = sc;
    } else {
      __syncthreads();
    }
    const uint32_t slot = tile * kTile + tid;
    const bool active = slot - S.body_off < S.n;
    float px = 0.0f, py = 0.0f, pz = 0.0f;
    uint32_t level = 0u, lx = 0u, ly = 0u, lz = 0u, key = 0xFFFFFFFFu;
    if (active) {
      const float4 p = pos4[slot];
      px = p.x;
      py = p.y;
      pz = p.z;
      key = sample_cell(S, px, py, pz, mom, choice, level, lx, ly, lz);
    }
    const uint32_t csh = S.depth - level;
    if (tid == 0) {  // slot 0 of a tile always holds a body
      s_cell[0] = key;
      s_cell[1] = level;
      s_cell[2] = lx >> csh;
      s_cell[3] = ly >> csh;
      s_cell[4] = lz >> csh;
    }
    __syncthreads();
    const float eps2 = S.softening * S.softening;
    float sx = 0.0f, sy = 0.0f, sz = 0.0f;
    const bool tile_uniform = __syncthreads_and(!active || key == s_cell[0]) != 0;
    if (tile_uniform) {
      // Every thread takes the same branches: tid 0's cell drives the loops.
      for (uint32_t j = 0; j < 27u; j++) {
        uint32_t lo, hi;
        if (neighbour_range(S, starts, s_cell[1], s_cell[2], s_cell[3], s_cell[4], j, lo, hi))
          p2p_staged_range<kTile>(pos4, lo, hi, buf, tid, slot, px, py, pz, eps2, sx, sy, sz,
                                  CtaSync());
      }
    } else {
      // Warps whose active bodies share a cell stage their own 32-source slice.
      const uint32_t amask = __ballot_sync(0xFFFFFFFFu, active);
      const uint32_t lead = amask != 0u ? (uint32_t)__ffs(amask) - 1u : 0u;
      const uint32_t wkey = __shfl_sync(0xFFFFFFFFu, key, lead);
      const bool warp_uniform = __all_sync(0xFFFFFFFFu, !active || key == wkey);
      if (amask == 0u) {
        // Padding only: nothing to sum.
      } else if (warp_uniform) {
        const uint32_t wl = __shfl_sync(0xFFFFFFFFu, level, lead);
        const uint32_t wx = __shfl_sync(0xFFFFFFFFu, lx >> csh, lead);
        const uint32_t wy = __shfl_sync(0xFFFFFFFFu, ly >> csh, lead);
        const uint32_t wz = __shfl_sync(0xFFFFFFFFu, lz >> csh, lead);
        float4 *wbuf = buf + 32u * warp;
        for (uint32_t j = 0; j < 27u; j++) {
          uint32_t lo, hi;
          if (neighbour_range(S, starts, wl, wx, wy, wz, j, lo, hi))
            p2p_staged_range<32u>(pos4, lo, hi, wbuf, lane, slot, px, py, pz, eps2, sx, sy, sz,
                                  WarpSync());
        }
      } else if (active) {
        const P2PView V{pos4, starts, slot};
        float sp;
        p2p_sums<false>(S, V, level, lx >> csh, ly >> csh, lz >> csh, px, py, pz, sx, sy, sz, sp);
      }
    }
    if (active) near_out[slot] = make_float4(sx, sy, sz, 0.0f);
  }
  stamp_end(stamp);
  grid_dependents_may_launch();
}

// Standalone P2M: deposit the current positions into `moments` (leaf level
// must be zero).  Persistent like k_integrate.
__global__ void __launch_bounds__(256) k_deposit(const SceneDesc *__restrict__ scenes,
                                                 const uint32_t *__restrict__ tile_scene,
                                                 const float4 *__restrict__ part,
                                                 uint4 *__restrict__ moments, uint32_t tiles,
                                                 const uint32_t *__restrict__ tile_list,
                                                 const Counters *__restrict__ ctr) {
  __shared__ DepositTable T;
  __shared__ SceneDesc S;
  const uint32_t ntiles = tile_list != nullptr ? min(ctr->tiles_active, tiles) : tiles;
  uint32_t t0, t1;
  cta_tile_range(ntiles, t0, t1);
  T.clear();
  uint32_t cur = 0xFFFFFFFFu;
  for (uint32_t i = t0; i < t1; i++) {
    const uint32_t tile = tile_list != nullptr ? tile_list[i] : i;
    const uint32_t slot = tile * kTile + threadIdx.x;
    const float4 p = part[2u * slot];
    const uint32_t sc = tile_scene[tile];
    if (sc != cur) {
      load_scene(S, scenes, sc);
      cur = sc;
    }
    const bool active = slot - S.body_off < S.n;
    uint32_t key = DepositTable::kEmpty;
    int32_t qx = 0, qy = 0, qz = 0;
    if (active) {
      key = S.cell_off + leaf_cell(p.x, p.y, p.z, S.depth);
      qx = f2i_rn_sat(p.x * S.scale);
      qy = f2i_rn_sat(p.y * S.scale);
      qz = f2i_rn_sat(p.z * S.scale);
    }
    deposit_body(T, key, active, qx, qy, qz, moments);
  }
  __syncthreads();
  T.flush(moments);
}

// FMM acceleration and potential of every body of one scene, written in the
// caller's body order (diagnostics and force-error checks; not on the step).
__global__ void __launch_bounds__(256) k_accel(const SceneDesc *__restrict__ scenes,
                                               const uint32_t *__restrict__ tile_scene,
                                               const float4 *__restrict__ part,
                                               const uint32_t *__restrict__ ids,
                                               const uint4 *__restrict__ mom,
                                               const float4 *__restrict__ src,
                                               const float4 *__restrict__ aux,
                                               const uint32_t *__restrict__ choice,
                                               const float *__restrict__ fields,
                                               float4 *__restrict__ out, uint32_t tile_base,
                                               const float4 *__restrict__ pos4,
                                               const uint32_t *__restrict__ starts) {
  const uint32_t tile = tile_base + blockIdx.x;
  const SceneDesc &S = scenes[tile_scene[tile]];
  const uint32_t slot = tile * kTile + threadIdx.x;
  if (slot - S.body_off >= S.n) return;
  const uint32_t id = ids[slot];
  if (id >= S.n) return;
  const float4 p = part[2u * slot];
  float ax, ay, az, pulse, phi;
  if (S.near_mode == kNearP2P) {
    const P2PView V{pos4, starts, slot};
    body_acceleration<true, true>(S, p.x, p.y, p.z, mom, src, aux, choice, fields, ax, ay, az, pulse,
                                  &phi, &V);
  } else {
    body_acceleration<true>(S, p.x, p.y, p.z, mom, src, aux, choice, fields, ax, ay, az, pulse, &phi);
  }
  out[S.body_off + id] = make_float4(ax, ay, az, phi);
}

// Resident slot of every body of one scene: slot_of[body_off + id] = slot.
__global__ void __launch_bounds__(256) k_slot_of(const SceneDesc *__restrict__ scenes,
                                                 const uint32_t *__restrict__ tile_scene,
                                                 const uint32_t *__restrict__ ids,
                                                 uint32_t *__restrict__ slot_of, uint32_t tile_base) {
  const uint32_t tile = tile_base + blockIdx.x;
  const SceneDesc &S = scenes[tile_scene[tile]];
  const uint32_t slot = tile * kTile + threadIdx.x;
  if (slot - S.body_off >= S.n) return;
  const uint32_t id = ids[slot];
  if (id < S.n) slot_of[S.body_off + id] = slot;
}

// FMM acceleration + potential of selected bodies (caller ids) of one scene.
__global__ void __launch_bounds__(256) k_accel_targets(
    const SceneDesc *__restrict__ scenes, uint32_t scene, const float4 *__restrict__ part,
    const uint32_t *__restrict__ slot_of, const uint32_t *__restrict__ targets, uint32_t nt,
    const uint4 *__restrict__ mom, const float4 *__restrict__ src, const float4 *__restrict__ aux,
    const uint32_t *__restrict__ choice, const float *__restrict__ fields, float4 *__restrict__ out,
    const float4 *__restrict__ pos4, const uint32_t *__restrict__ starts) {
  const SceneDesc &S = scenes[scene];
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nt || targets[t] >= S.n) return;
  const uint32_t slot = slot_of[S.body_off + targets[t]];
  const float4 p = part[2u * slot];
  float ax, ay, az, pulse, phi;
  if (S.near_mode == kNearP2P) {
    const P2PView V{pos4, starts, slot};
    body_acceleration<true, true>(S, p.x, p.y, p.z, mom, src, aux, choice, fields, ax, ay, az, pulse,
                                  &phi, &V);
  } else {
    body_acceleration<true>(S, p.x, p.y, p.z, mom, src, aux, choice, fields, ax, ay, az, pulse, &phi);
  }
  out[t] = make_float4(ax, ay, az, phi);
}

void launch_slot_of(const LaunchCtx &L, const uint32_t *ids, uint32_t *slot_of, uint32_t tile_base,
                    uint32_t tiles) {
  k_slot_of<<<tiles, kTile, 0, L.stream>>>(L.scenes, L.tile_scene, ids, slot_of, tile_base);
}

void launch_accel_targets(const LaunchCtx &L, uint32_t scene, uint32_t tile_base, uint32_t tiles,
                          const uint32_t *ids, uint32_t *slot_of, const uint32_t *targets,
                          uint32_t nt, float4 *out) {
  k_slot_of<<<tiles, kTile, 0, L.stream>>>(L.scenes, L.tile_scene, ids, slot_of, tile_base);
  k_accel_targets<<<(nt + 255u) / 256u, 256, 0, L.stream>>>(
      L.scenes, scene, L.part, slot_of, targets, nt, L.mom, L.src, L.aux, L.choice, L.fields, out,
      L.pos4, L.starts_out);
}

void launch_accel(const LaunchCtx &L, const uint32_t *ids, float4 *out, uint32_t tile_base,
                  uint32_t tiles) {
  k_accel<<<tiles, kTile, 0, L.stream>>>(L.scenes, L.tile_scene, L.part, ids, L.mom, L.src, L.aux,
                                         L.choice, L.fields, out, tile_base, L.pos4, L.starts_out);
}

__global__ void __launch_bounds__(256) k_keys(const SceneDesc *__restrict__ scenes,
                                              const uint32_t *__restrict__ tile_scene,
                                              const float4 *__restrict__ part,
                                              uint32_t *__restrict__ keys, uint32_t *__restrict__ vals,
                                              uint32_t *__restrict__ ids, int fresh_ids,
                                              uint32_t tile_base,
                                              const __grid_constant__ SceneMask fresh,
                                              const uint32_t *__restrict__ tile_map) {
  const uint32_t tile = tile_map != nullptr ? tile_map[blockIdx.x] : tile_base + blockIdx.x;
  const uint32_t sc = tile_scene[tile];
  const SceneDesc &S = scenes[sc];
  const uint32_t slot = tile * kTile + threadIdx.x;
  const uint32_t out = blockIdx.x * kTile + threadIdx.x;  // keys/vals are relative to tile_base
  const uint32_t local = slot - S.body_off;
  const uint32_t F = S.key_level;
  uint32_t key = S.key_base | ((1u << (3u * F)) - 1u);  // padding sorts after its scene's bodies
  if (local < S.n && S.near_mode == kNearP2P) {
    // Leaf key only: bodies of a leaf keep their input (caller) order.
    const float4 p = part[2u * slot];
    const uint32_t dim = 1u << S.depth;
    key = S.key_base | (morton3(cell_of_unit(unit_coord(p.x), dim), cell_of_unit(unit_coord(p.y), dim),
                                cell_of_unit(unit_coord(p.z), dim))
                        << (3u * (F - S.depth)));
  } else if (local < S.n) {
    const float4 p = part[2u * slot];
    const uint32_t dim = 1u << F;
    // floor(u * 2^F) >> (F - depth) == floor(u * 2^depth): the fine key refines the leaf key.
    key = S.key_base | (spread3(cell_of_unit(unit_coord(p.x), dim)) |
                        (spread3(cell_of_unit(unit_coord(p.y), dim)) << 1) |
                        (spread3(cell_of_unit(unit_coord(p.z), dim)) << 2));
  }
  keys[out] = key;
  vals[out] = slot;
  if (fresh_ids == 1 || (fresh_ids == 2 && ((fresh.bits[sc >> 5] >> (sc & 31u)) & 1u))) ids[slot] = local;
}

// Apply a permutation to the resident bodies (and their caller ids).  With
// `deposit_into`, the permuted bodies are also deposited (persistent grid,
// per-CTA deposit table); otherwise one CTA per tile.
__global__ void __launch_bounds__(256) k_gather(const SceneDesc *__restrict__ scenes,
                                                const uint32_t *__restrict__ tile_scene,
                                                const uint32_t *__restrict__ perm,
                                                const float4 *__restrict__ part_in,
                                                const uint32_t *__restrict__ ids_in,
                                                float4 *__restrict__ part_out,
                                                uint32_t *__restrict__ ids_out,
                                                uint4 *__restrict__ deposit_into, uint32_t tiles,
                                                uint32_t tile_base, float4 *__restrict__ pos_out,
                                                const uint32_t *__restrict__ tile_map) {
  __shared__ DepositTable T;
  __shared__ SceneDesc S;
  // Slots [tile_base * 256, (tile_base + tiles) * 256) are permuted among
  // themselves; perm is relative to tile_base and holds absolute slots.  With
  // a tile map, output tile i is tile_map[i] and each scene's tiles are
  // permuted among themselves.
  const uint32_t lo = tile_base * kTile, hi = (tile_base + tiles) * kTile;
  uint32_t t0 = blockIdx.x, t1 = blockIdx.x + 1u;
  if (deposit_into != nullptr) {
    cta_tile_range(tiles, t0, t1);
    T.clear();
  }
  uint32_t cur = 0xFFFFFFFFu;
  for (uint32_t i = t0; i < t1; i++) {
    const uint32_t tile = tile_map != nullptr ? tile_map[i] : tile_base + i;
    const uint32_t slot = tile * kTile + threadIdx.x;
    uint32_t from = perm[i * kTile + threadIdx.x];
    // Defensive: a permutation never leaves its range (or its scene).
    if (tile_map != nullptr ? tile_scene[from / kTile] != tile_scene[tile] : (from < lo || from >= hi))
      from = slot;
    const float4 p0 = part_in[2u * from], p1 = part_in[2u * from + 1u];
    part_out[2u * slot] = p0;
    part_out[2u * slot + 1u] = p1;
    ids_out[slot] = ids_in[from];
    if (pos_out != nullptr) pos_out[slot] = p0;
    if (deposit_into != nullptr) {
      const uint32_t sc = tile_scene[tile];
      if (sc != cur) {
        load_scene(S, scenes, sc);
        cur = sc;
      }
      const bool active = slot - S.body_off < S.n;
      uint32_t key = DepositTable::kEmpty;
      int32_t qx = 0, qy = 0, qz = 0;
      if (active) {
        key = S.cell_off + leaf_cell(p0.x, p0.y, p0.z, S.depth);
        qx = f2i_rn_sat(p0.x * S.scale);
        qy = f2i_rn_sat(p0.y * S.scale);
        qz = f2i_rn_sat(p0.z * S.scale);
      }
      deposit_body(T, key, active, qx, qy, qz, deposit_into);
    }
  }
  if (deposit_into != nullptr) {
    __syncthreads();
    T.flush(deposit_into);
  }
}

// Scatter bodies back to the caller's order: out[body_off + id] = part[slot].
__global__ void __launch_bounds__(256) k_unpermute(const SceneDesc *__restrict__ scenes,
                                                   const uint32_t *__restrict__ tile_scene,
                                                   const float4 *__restrict__ part,
                                                   const uint32_t *__restrict__ ids,
                                                   float4 *__restrict__ out, uint32_t tile_base,
                                                   const uint32_t *__restrict__ tile_map,
                                                   const uint32_t *__restrict__ tile_count) {
  const uint32_t tile = tile_map != nullptr ? tile_map[blockIdx.x] : tile_base + blockIdx.x;
  const SceneDesc &S = scenes[tile_scene[tile]];
  // The scene's body count: from the caller when given (a retiring serving
  // slot's descriptor may already read empty), else from the descriptor.
  const uint32_t n = tile_count != nullptr ? tile_count[blockIdx.x] : S.n;
  const uint32_t slot = tile * kTile + threadIdx.x;
  if (slot - S.body_off >= n) return;
  const uint32_t id = ids[slot];
  if (id >= n) return;  // defensive: ids are a permutation of 0..n-1
  const uint32_t dst = S.body_off + id;
  out[2u * dst] = part[2u * slot];
  out[2u * dst + 1u] = part[2u * slot + 1u];
}

// ------------------------------------------------------ galaxy seeding

__device__ __forceinline__ uint32_t hash32(uint32_t x) {  // wgsl:205-210
  x = ((x >> 16) ^ x) * 0x45d9f3bu;
  x = ((x >> 16) ^ x) * 0x45d9f3bu;
  return (x >> 16) ^ x;
}

__device__ __forceinline__ float random01(uint32_t seed) {
  return (float)hash32(seed) * (1.0f / 4294967296.0f);
}

__device__ float seeded_enclosed_mass(float radius) {  // wgsl:216-230
  const float bulge = 0.05f * rf_powf(clampf_d(radius / 0.11f, 0.0f, 1.0f), 3.0f);
  const float halo = 0.70f * rf_powf(clampf_d(radius / 0.70f, 0.0f, 1.0f), 3.0f);
  const float disc = 0.18f * rf_powf(clampf_d((radius - 0.055f) / 0.60f, 0.0f, 1.0f), 1.0f / 0.72f);
  const float polar = 0.07f * rf_powf(clampf_d((radius - 0.22f) / 0.31f, 0.0f, 1.0f), 1.0f / 0.86f);
  return fmaxf(bulge + halo + disc + polar, 0.0001f);
}

__device__ __forceinline__ void cross3(const float a[3], const float b[3], float o[3]) {
  o[0] = a[1] * b[2] - a[2] * b[1];
  o[1] = a[2] * b[0] - a[0] * b[2];
  o[2] = a[0] * b[1] - a[1] * b[0];
}

__global__ void __launch_bounds__(256) k_initialize(const SceneDesc *__restrict__ scenes,
                                                    const uint32_t *__restrict__ tile_scene,
                                                    float4 *__restrict__ out, uint32_t tile_base) {
  constexpr float kTau = 6.28318530718f;
  const uint32_t tile = tile_base + blockIdx.x;
  const SceneDesc &S = scenes[tile_scene[tile]];
  const uint32_t slot = tile * kTile + threadIdx.x;
  const uint32_t i = slot - S.body_off;
  if (i >= S.n) return;
  const float u0 = random01(i * 11u + 1u), u1 = random01(i * 11u + 2u), u2 = random01(i * 11u + 3u);
  const float u3 = random01(i * 11u + 4u), u4 = random01(i * 11u + 5u), u5 = random01(i * 11u + 6u);
  float pos[3], vel[3], excitation;
  if (u5 < 0.75f) {
    const float z = u0 * 2.0f - 1.0f, phi = kTau * u1;
    const float outer = u5 < 0.05f ? 0.11f : 0.70f;
    const float radius = outer * rf_powf(u2, 0.3333333f);
    const float ring = sqrtf(fmaxf(0.0f, 1.0f - z * z));
    const float rd[3] = {ring * rf_cosf(phi), z, ring * rf_sinf(phi)};
    for (int k = 0; k < 3; k++) pos[k] = radius * rd[k];
    const float tz = u3 * 2.0f - 1.0f, tphi = kTau * u4;
    const float tring = sqrtf(fmaxf(0.0f, 1.0f - tz * tz));
    const float rnd[3] = {tring * rf_cosf(tphi), tz, tring * rf_sinf(tphi)};
    float tangent[3];
    cross3(rd, rnd, tangent);
    if (length3(tangent[0], tangent[1], tangent[2]) < 0.001f) {
      const float up[3] = {0.0f, 1.0f, 0.0f};
      cross3(rd, up, tangent);
    }
    if (length3(tangent[0], tangent[1], tangent[2]) < 0.001f) {
      const float ex[3] = {1.0f, 0.0f, 0.0f};
      cross3(rd, ex, tangent);
    }
    const float orbital = 0.985f * sqrtf(S.gravity * seeded_enclosed_mass(radius) / (radius + 0.018f));
    const float tl = length3(tangent[0], tangent[1], tangent[2]);
    for (int k = 0; k < 3; k++) vel[k] = orbital * (tangent[k] / tl);
    excitation = u5 < 0.05f ? 0.09f : 0.025f + u4 * 0.025f;
  } else if (u5 < 0.93f) {
    const float radius = 0.055f + 0.60f * rf_powf(u0, 0.72f);
    const float arm = (float)(i & 3u) * (kTau / 4.0f);
    const float angle = arm + radius * 7.8f + (u1 - 0.5f) * (0.045f + radius * 0.055f);
    const float thickness = (u2 + u3 + u4 - 1.5f) * (0.0035f + radius * 0.010f);
    const float flat[3] = {radius * rf_cosf(angle), radius * rf_sinf(angle) * 0.72f, thickness};
    const float tilt = 0.20f;
    pos[0] = flat[0];
    pos[1] = flat[1] * rf_cosf(tilt) - flat[2] * rf_sinf(tilt);
    pos[2] = flat[1] * rf_sinf(tilt) + flat[2] * rf_cosf(tilt);
    const float orbital = 0.99f * sqrtf(S.gravity * seeded_enclosed_mass(radius) / (radius + 0.018f));
    const float tangent[3] = {-rf_sinf(angle), rf_cosf(angle) * 0.72f * rf_cosf(tilt),
                              rf_cosf(angle) * 0.72f * rf_sinf(tilt)};
    const float pl = length3(pos[0], pos[1], pos[2]);
    const float tl = length3(tangent[0], tangent[1], tangent[2]);
    const float sw = rf_sinf(angle * 3.0f - radius * 13.0f);
    for (int k = 0; k < 3; k++) vel[k] = orbital * (tangent[k] / tl) + (pos[k] / pl) * orbital * 0.035f * sw;
    excitation = 0.08f + u3 * 0.05f;
  } else {
    const float lineage = (float)(i & 3u);
    const float radius = 0.22f + 0.31f * rf_powf(u0, 0.86f) + (lineage - 1.5f) * 0.007f;
    const float angle = kTau * u1 + radius * 3.5f;
    const float thickness = (u2 + u3 + u4 - 1.5f) * (0.004f + radius * 0.009f);
    const float flat[3] = {radius * rf_cosf(angle), thickness, radius * rf_sinf(angle)};
    const float tilt = -0.54f + lineage * 0.36f;
    pos[0] = flat[0] * rf_cosf(tilt) - flat[1] * rf_sinf(tilt);
    pos[1] = flat[0] * rf_sinf(tilt) + flat[1] * rf_cosf(tilt);
    pos[2] = flat[2];
    const float tangent[3] = {-rf_sinf(angle) * rf_cosf(tilt), -rf_sinf(angle) * rf_sinf(tilt), rf_cosf(angle)};
    const float orbital = 0.99f * sqrtf(S.gravity * seeded_enclosed_mass(radius) / (radius + 0.018f));
    const float tl = length3(tangent[0], tangent[1], tangent[2]);
    for (int k = 0; k < 3; k++) vel[k] = -orbital * (tangent[k] / tl);
    excitation = 0.20f + u4 * 0.08f;
  }
  float hue = 0.0f;
  if (u5 >= 0.75f) {
    const float speed = fmaxf(length3(vel[0], vel[1], vel[2]), 0.0001f);
    const float radius = fmaxf(length3(pos[0], pos[1], pos[2]), 0.0001f);
    const float pv = (pos[0] * vel[0] + pos[1] * vel[1]) + pos[2] * vel[2];
    const float radial_motion = clampf_d(pv / (radius * speed), -1.0f, 1.0f);
    float am[3];
    cross3(pos, vel, am);
    const float spin = am[1] / fmaxf(length3(am[0], am[1], am[2]), 0.0001f);
    const float h = rf_atan2f(vel[1], vel[0]) / kTau + (vel[2] / speed) * 0.14f + spin * 0.075f +
                    radial_motion * 0.065f + excitation * 0.085f + (float)(i & 3u) * 0.018f;
    hue = h - floorf(h);
  }
  out[2u * slot] = make_float4(pos[0], pos[1], pos[2], hue);
  out[2u * slot + 1u] = make_float4(vel[0], vel[1], vel[2], excitation);
}

// --------------------------------------------------------------- launches

uint32_t body_ctas_per_sm() {
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_integrate<false>, kTile, 0) != cudaSuccess || n < 1)
    n = 1;
  return (uint32_t)n;
}

// Persistent body-pass grid: whole waves of resident CTAs, at most one per tile.
static uint32_t body_grid(const LaunchCtx &L, uint32_t tiles) {
  return tiles < L.body_ctas ? tiles : L.body_ctas;
}

void launch_integrate(const LaunchCtx &L, uint32_t tiles) {
  launch_step_kernel(L, L.p2p ? k_integrate<true> : k_integrate<false>, dim3(body_grid(L, tiles)),
                     dim3(kTile), 0, L.scenes, L.tile_scene, L.part, (const uint4 *)L.mom,
                     (const float4 *)L.src, (const float4 *)L.aux, (const uint32_t *)L.choice,
                     (const float *)L.fields, L.mom_next, tiles, L.tile_list, L.ctr,
                     L.integrate_dynamic ? 1 : 0, L.pos4, (const uint32_t *)L.starts_out,
                     (const float4 *)L.near4, stamp_rec(L, 3u));
}

// The P2P grid: one wave of this kernel's resident CTAs (its register
// budget allows fewer per SM than integrate's), at most one per tile.
static uint32_t near_p2p_grid(const LaunchCtx &L, uint32_t tiles) {
  static const uint32_t per_sm = [] {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_near_p2p, kTile, 0) != cudaSuccess || n < 1)
      n = 1;
    return (uint32_t)n;
  }();
  const uint32_t grid = (L.sms ? L.sms : 1u) * per_sm;
  return tiles < grid ? tiles : grid;
}

void launch_near_p2p(const LaunchCtx &L, uint32_t tiles) {
  launch_step_kernel(L, k_near_p2p, dim3(near_p2p_grid(L, tiles)), dim3(kTile), 0, L.scenes,
                     L.tile_scene, (const float4 *)L.pos4, (const uint32_t *)L.starts_out,
                     (const uint4 *)L.mom, (const uint32_t *)L.choice, tiles, L.tile_list, L.ctr,
                     L.near4, stamp_rec(L, 5u));
}

void launch_deposit(const LaunchCtx &L, uint4 *moments, uint32_t tiles) {
  k_deposit<<<body_grid(L, tiles), kTile, 0, L.stream>>>(L.scenes, L.tile_scene, L.part, moments,
                                                         tiles, L.tile_list, L.ctr);
}

void launch_keys(const LaunchCtx &L, uint32_t *keys, uint32_t *vals, uint32_t *ids, int fresh_ids,
                 uint32_t tiles, uint32_t tile_base, const SceneMask *fresh,
                 const uint32_t *tile_map) {
  static const SceneMask kNone{};
  k_keys<<<tiles, kTile, 0, L.stream>>>(L.scenes, L.tile_scene, L.part, keys, vals, ids, fresh_ids,
                                        tile_base, fresh != nullptr ? *fresh : kNone, tile_map);
}

void launch_gather(const LaunchCtx &L, const uint32_t *perm, const float4 *part_in,
                   const uint32_t *ids_in, float4 *part_out, uint32_t *ids_out, uint4 *deposit_into,
                   uint32_t tiles, uint32_t tile_base, float4 *pos_out, const uint32_t *tile_map) {
  const uint32_t grid = deposit_into != nullptr ? body_grid(L, tiles) : tiles;
  k_gather<<<grid, kTile, 0, L.stream>>>(L.scenes, L.tile_scene, perm, part_in, ids_in, part_out,
                                         ids_out, deposit_into, tiles, tile_base, pos_out, tile_map);
}

// Per-leaf body ranges of the leaf-sorted scenes (kNearP2P): entry m of a
// scene's table (at its cell offset) is the first slot whose leaf Morton code
// is >= m, for m in [0, 8^depth]; found by binary search in the sorted keys.
__global__ void __launch_bounds__(256) k_leaf_starts(const SceneDesc *__restrict__ scenes,
                                                     const uint32_t *__restrict__ keys,
                                                     uint32_t *__restrict__ starts) {
  const SceneDesc &S = scenes[blockIdx.y];
  if (S.n == 0u || S.near_mode != kNearP2P) return;
  const uint32_t leaves = 1u << (3u * S.depth);
  for (uint32_t m = blockIdx.x * blockDim.x + threadIdx.x; m <= leaves; m += gridDim.x * blockDim.x) {
    uint32_t lo = m < leaves ? 0u : S.n, hi = S.n;  // entry 8^depth ends the last leaf
    if (m < leaves) {
      const uint32_t target = S.key_base | (m << (3u * (S.key_level - S.depth)));
      while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (keys[S.body_off + mid] < target) {
          lo = mid + 1u;
        } else {
          hi = mid;
        }
      }
    }
    starts[S.cell_off + m] = S.body_off + lo;
  }
}

void launch_leaf_starts(const LaunchCtx &L, const uint32_t *sorted_keys, uint32_t scenes) {
  k_leaf_starts<<<dim3(64, scenes), 256, 0, L.stream>>>(L.scenes, sorted_keys, L.starts_out);
}

void launch_unpermute(const LaunchCtx &L, const uint32_t *ids, float4 *out, uint32_t tile_base,
                      uint32_t tiles, const uint32_t *tile_map, const uint32_t *tile_count) {
  k_unpermute<<<tiles, kTile, 0, L.stream>>>(L.scenes, L.tile_scene, L.part, ids, out, tile_base,
                                             tile_map, tile_count);
}

// Scene descriptors written from kernel parameters (a few at a time, on the
// caller's stream, without touching the other entries of the table).
struct SceneWrites {
  static constexpr uint32_t kMax = 16u;
  uint32_t count;
  uint32_t index[kMax];
  SceneDesc desc[kMax];
};

__global__ void __launch_bounds__(32) k_write_scenes(SceneDesc *__restrict__ scenes,
                                                     const __grid_constant__ SceneWrites w) {
  for (uint32_t i = 0; i < w.count; i++) {
    const uint32_t *src = reinterpret_cast<const uint32_t *>(&w.desc[i]);
    uint32_t *dst = reinterpret_cast<uint32_t *>(scenes + w.index[i]);
    for (uint32_t k = threadIdx.x; k < sizeof(SceneDesc) / 4u; k += blockDim.x) dst[k] = src[k];
  }
}

void launch_write_scenes(cudaStream_t stream, SceneDesc *scenes, const uint32_t *index,
                         const SceneDesc *desc, uint32_t count) {
  for (uint32_t at = 0; at < count; at += SceneWrites::kMax) {
    SceneWrites w{};
    w.count = count - at < SceneWrites::kMax ? count - at : SceneWrites::kMax;
    for (uint32_t i = 0; i < w.count; i++) {
      w.index[i] = index[at + i];
      w.desc[i] = desc[at + i];
    }
    k_write_scenes<<<1, 32, 0, stream>>>(scenes, w);
  }
}

// Zero the moments (both buffers), sources and records of every cell of the
// scenes set in `which` (a rebuilt scene starts from cleared trees: the
// upward pass skips subtrees that are empty in both moment buffers).  Every
// CTA takes a share of each scene's cells.
__global__ void __launch_bounds__(256) k_clear_scenes(const SceneDesc *__restrict__ scenes, uint32_t nscenes,
                                                      const __grid_constant__ SceneMask which,
                                                      uint4 *__restrict__ mom0, uint4 *__restrict__ mom1,
                                                      float4 *__restrict__ src, float4 *__restrict__ aux) {
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t w = 0; w < (nscenes + 31u) / 32u; w++) {
    for (uint32_t bits = which.bits[w]; bits != 0u; bits &= bits - 1u) {
      const SceneDesc &S = scenes[32u * w + (uint32_t)(__ffs(bits) - 1)];
      for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < S.cells; c += stride) {
        const uint32_t i = S.cell_off + c;
        mom0[i] = make_uint4(0u, 0u, 0u, 0u);
        mom1[i] = make_uint4(0u, 0u, 0u, 0u);
        src[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        aux[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      }
    }
  }
}

void launch_clear_scenes(const LaunchCtx &L, uint32_t nscenes, const SceneMask &which, uint4 *mom0,
                         uint4 *mom1, float4 *src, float4 *aux) {
  k_clear_scenes<<<4u * L.sms, 256, 0, L.stream>>>(L.scenes, nscenes, which, mom0, mom1, src, aux);
}

void launch_initialize(const LaunchCtx &L, float4 *part_out, uint32_t tile_base, uint32_t tiles) {
  k_initialize<<<tiles, kTile, 0, L.stream>>>(L.scenes, L.tile_scene, part_out, tile_base);
}

// Bulk upload, one CTA per 256-slot tile: two 16-byte loads and stores per body.
__global__ void __launch_bounds__(256) k_upload_scenes(const SceneDesc *__restrict__ scenes,
                                                       const uint32_t *__restrict__ tile_scene,
                                                       float4 *__restrict__ part, uint32_t tile_base,
                                                       uint32_t scene_base,
                                                       const __grid_constant__ UploadSources src) {
  const uint32_t tile = tile_base + blockIdx.x;
  const uint32_t sc = tile_scene[tile];
  const float4 *from = src.p[sc - scene_base];
  const SceneDesc &S = scenes[sc];
  const uint32_t slot = tile * kTile + threadIdx.x, local = slot - S.body_off;
  if (from != nullptr && local < S.n) {
    part[2u * slot] = from[2u * local];
    part[2u * slot + 1u] = from[2u * local + 1u];
  }
}

void launch_upload_scenes(const LaunchCtx &L, float4 *part, uint32_t tile_base, uint32_t tiles,
                          uint32_t scene_base, const UploadSources &src) {
  k_upload_scenes<<<tiles, kTile, 0, L.stream>>>(L.scenes, L.tile_scene, part, tile_base, scene_base,
                                                 src);
}

RFMM_KERNEL_NS_END
