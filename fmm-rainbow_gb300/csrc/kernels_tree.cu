// Tree passes of the FMM step: upward (M2M), M2L, and L2L fused with the
// adaptive-leaf near field.
//
// Reference passes (iskamag/fmm-rainbow src/rainbow_fmm.wgsl):
//   upward   424-455   one dispatch per level, 8-child integer sums
//   m2l_all  457-519   <= 189 pair_field terms per on-path cell
//   downward 574-611   parent field translated to the child centre
//   near_all 521-572   26 neighbour cell monopoles per adaptive leaf
//
// GB300 structure:
//   k_upward     one 256-thread CTA per 8x8x8-leaf subtree reduces four levels
//                in shared memory and takes a completion ticket as soon as
//                its root is known; the last CTA of a scene finishes the top
//                levels.  It also writes each cell's source record (centre
//                of mass, G*m), appends every parent with more than 16 bodies
//                to the work list, zeroes the leaf level the next integrate
//                deposits into, and resolves each leaf's sample cell; a few
//                extra CTAs clear the fields of the previous step's targets
//                (fields are zero off the M2L path).
//   k_m2l        one CTA per listed parent: the 6x6x6 source tile of the
//                parent's 3x3x3 neighbourhood is staged in shared memory by a
//                TMA tensor copy; warp w evaluates child w's contributing
//                stencil slots in parallel and 80 threads (8 children x 10
//                components) sum them in the reference's loop order (excluded
//                and empty slots contribute +0, which leaves an accumulation
//                that starts at +0 unchanged).
//   k_l2l_near   one warp per target: the top-down L2L chain is recomputed
//                from the M2L results of the target's ancestors (so levels
//                need no ordering), then adaptive leaves add their 26 near
//                terms in loop order.
//   k_upward_warps, and the lane paths of k_m2l and k_l2l_near
//                the same passes with one warp per subtree and one lane per
//                target (its sums in its own registers, in the same order):
//                fewer instructions and barriers per term, for work lists
//                long enough to fill the GPU (many scenes).
#include <cuda.h>
#include <cuda_runtime.h>

#include <type_traits>
#include <utility>

#include "rfmm_device.cuh"
#include "rfmm_kernels.h"

RFMM_KERNEL_NS_BEGIN

// ----------------------------------------------------------------- upward

__device__ __forceinline__ uint4 add_moment(uint4 a, uint4 b) {
  return make_uint4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w);
}

__device__ __forceinline__ void store_cell(const SceneDesc &S, uint32_t local_cell, uint4 m,
                                           uint4 *mom, float4 *src, float4 *aux) {
  const uint32_t g = S.cell_off + local_cell;
  mom[g] = m;
  src[g] = make_source(m, S.scale, S.gravity, S.n_f);
  aux[g] = make_aux(m.x, S.gravity, S.n_f);
}

// atomicAdd with acquire-release semantics at GPU scope: this thread's earlier
// writes are visible to whoever observes the new value, and writes released
// by earlier adders are visible to this thread afterwards.
__device__ __forceinline__ uint32_t atomic_add_acq_rel(uint32_t *p, uint32_t v) {
  uint32_t old;
  asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
}

// Sum of the 8 children (2x, 2y, 2z) + {0,1}^3 of cell (x, y, z) in a
// child level of side cdim held in shared memory.
__device__ __forceinline__ uint4 sum_children(const uint4 *c, uint32_t x, uint32_t y, uint32_t z,
                                              uint32_t cdim) {
  uint4 acc = make_uint4(0u, 0u, 0u, 0u);
#pragma unroll
  for (uint32_t dz = 0; dz < 2u; dz++)
#pragma unroll
    for (uint32_t dy = 0; dy < 2u; dy++)
#pragma unroll
      for (uint32_t dx = 0; dx < 2u; dx++)
        acc = add_moment(acc, c[(2u * x + dx) + cdim * ((2u * y + dy) + cdim * (2u * z + dz))]);
  return acc;
}

// Body of one upward task: the 8x8x8-leaf subtree `sub` of scene `scene`.
// The completion ticket needs only the subtree root's moment, so the
// reduction runs first in shared memory, thread 0 writes the root and takes
// the ticket, and the other writes of the subtree (sources and records of its
// cells, the cleared next-deposit leaves, the listed parents, the leaves'
// sample cells) follow the ticket, off the path to the scene's last CTA.
__device__ __forceinline__ void upward_task(
    const SceneDesc &S, uint32_t scene, uint32_t sub, uint4 *__restrict__ mom,
    uint4 *__restrict__ mom_next, float4 *__restrict__ src, float4 *__restrict__ aux,
    uint32_t *__restrict__ choice, WorkItem *__restrict__ plist, uint32_t plist_cap,
    Counters *__restrict__ ctr, uint32_t list_par, uint32_t *__restrict__ tickets, uint4 *s0,
    uint4 *s1, uint4 *s2, uint4 *s_top, WorkItem *s_items, uint32_t &s_nitems, uint32_t &s_base,
    uint32_t &s_last, bool trigger) {
  const uint32_t tid = threadIdx.x;
  const uint32_t D = S.depth, r = S.sub_level;  // r = D - 3
  uint32_t sx, sy, sz;
  cell_coords_lv(sub, r, sx, sy, sz);
  if (tid == 0) s_nitems = 0;

  // Leaves of this subtree: 8x8x8 block, x fastest (rows of 128 B); two per
  // thread.  Also read: the subtree root in both moment buffers.
  const uint32_t dim = 1u << D;
  uint32_t seen = 0u;
  uint4 m[2];
#pragma unroll
  for (uint32_t h = 0; h < 2u; h++) {
    const uint32_t t = tid + h * 256u;
    const uint32_t lx = t & 7u, ly = (t >> 3) & 7u, lz = t >> 6;
    const uint32_t leaf = level_offset_d(D) + lin3(sx * 8u + lx, sy * 8u + ly, sz * 8u + lz, dim);
    m[h] = mom[S.cell_off + leaf];
    seen |= m[h].x;
  }
  // Upper cell `tid` < 73 of the subtree: 64 of level D-1, 8 of D-2, the root.
  const uint32_t ul = tid < 64u ? D - 1u : (tid < 72u ? D - 2u : r);
  const uint32_t uw = tid < 64u ? 4u : (tid < 72u ? 2u : 1u);
  const uint32_t ui = tid < 64u ? tid : (tid < 72u ? tid - 64u : 0u);
  const uint32_t ucell = level_offset_d(ul) + lin3(sx * uw + ui % uw, sy * uw + (ui / uw) % uw,
                                                   sz * uw + ui / (uw * uw), 1u << ul);
  // A buffer's subtree-root count is the count of its leaves as of the last
  // upward pass that built that buffer's tree (counts never wrap), and a
  // zero count means zero sums and records in every cell of the subtree.
  // The next-deposit buffer's tree was built by the previous step's upward
  // pass from the leaves it still holds, so its root count is zero exactly
  // when those leaves are; the current buffer's root is that of the pass
  // before, so a zero root means its upper cells hold nothing stale.
  if (tid == 72u) seen |= mom[S.cell_off + ucell].x | mom_next[S.cell_off + ucell].x;
  // Empty now, empty in the previous deposit and nothing stale above the
  // leaves: the subtree's moments, sources and next-deposit leaves are all
  // zero already (induction over steps; every rebuild of the moments clears
  // both buffers), so it only takes part in the ticket count.  Bodies never
  // sit in its leaves, so their sample cells are never read.
  const bool live = __syncthreads_or(seen != 0u);
  if (live) {
    s0[tid] = m[0];
    s0[tid + 256u] = m[1];
    __syncthreads();
    if (tid < 64u) s1[tid] = sum_children(s0, tid & 3u, (tid >> 2) & 3u, tid >> 4, 8u);
    __syncthreads();
    if (tid < 8u) s2[tid] = sum_children(s1, tid & 1u, (tid >> 1) & 1u, tid >> 2, 4u);
    __syncthreads();
    if (tid == 0) {
      uint4 acc = make_uint4(0u, 0u, 0u, 0u);
      for (uint32_t k = 0; k < 8u; k++) acc = add_moment(acc, s2[k]);
      s2[8] = acc;
      // The level-r cell the last CTA reads.
      mom[S.cell_off + level_offset_d(r) + lin3(sx, sy, sz, 1u << r)] = acc;
    }
  }

  // The scene's last finished subtree reduces levels r-1 .. 0.  Only thread 0
  // wrote the level-r cell that reduction reads; its tickets release that
  // write (and acquire the earlier subtrees' ones) on the way to the last CTA,
  // whose other threads are ordered after thread 0 by the barrier below.
  if (tid == 0) {
    const uint32_t ntasks = 1u << (3u * r);
    const uint32_t ngroups = (ntasks + kTicketGroup - 1u) / kTicketGroup;
    const uint32_t group = sub / kTicketGroup;
    const uint32_t gsize = min(kTicketGroup, ntasks - group * kTicketGroup);
    uint32_t *t = tickets + scene * kTicketStride;
    uint32_t last = 0u;
    // A live subtree releases its root write; an empty one has nothing to
    // release and takes its ticket relaxed.  The group's last CTA acquires
    // the group's releases (fence after observing the final count) before
    // its scene ticket.
    const uint32_t g_old = live ? atomic_add_acq_rel(&t[1u + group], 1u) : atomicAdd(&t[1u + group], 1u);
    if (g_old == gsize - 1u) {  // last subtree of its group
      if (!live) __threadfence();
      t[1u + group] = 0u;
      if (atomic_add_acq_rel(&t[0], 1u) == ngroups - 1u) {  // last group of the scene
        t[0] = 0u;
        last = 1u;
      }
    }
    s_last = last;
  }
  __syncthreads();
  // The CTA's last task is past its ticket: let the next pass launch, so its
  // launch overlaps the writes below and the last CTA's top levels (the
  // next pass still waits for this whole grid before it reads anything).
  if (trigger) grid_dependents_may_launch();

  if (live) {
    // Leaves: source records and the cleared next-deposit leaf.
#pragma unroll
    for (uint32_t h = 0; h < 2u; h++) {
      const uint32_t t = tid + h * 256u;
      const uint32_t lx = t & 7u, ly = (t >> 3) & 7u, lz = t >> 6;
      const uint32_t leaf = S.cell_off + level_offset_d(D) + lin3(sx * 8u + lx, sy * 8u + ly, sz * 8u + lz, dim);
      src[leaf] = make_source(m[h], S.scale, S.gravity, S.n_f);
      aux[leaf] = make_aux(m[h].x, S.gravity, S.n_f);
      mom_next[leaf] = make_uint4(0u, 0u, 0u, 0u);
    }
    // Upper cells.
    if (tid < 73u) {
      const uint4 acc = tid < 64u ? s1[tid] : (tid < 72u ? s2[tid - 64u] : s2[8]);
      store_cell(S, ucell, acc, mom, src, aux);
      if ((int32_t)acc.x > (int32_t)kAdaptive) s_items[atomicAdd(&s_nitems, 1u)] = {scene, ucell};
    }
    // Sample cell of each leaf.  Counts never shrink towards the root, so
    // when this subtree's root holds more than 16 bodies every level <= r is
    // skipped by the descent and the choice lies within the subtree: the
    // first of levels D-2, D-1 with count <= 16, else the leaf.
    const uint32_t root_count = s2[8].x;
#pragma unroll
    for (uint32_t h = 0; h < 2u; h++) {
      const uint32_t t = tid + h * 256u;
      const uint32_t lx = t & 7u, ly = (t >> 3) & 7u, lz = t >> 6;
      uint32_t v = kChoiceUnresolved;
      if ((int32_t)root_count > (int32_t)kAdaptive) {
        const uint32_t c2 = s2[(lx >> 2) + 2u * ((ly >> 2) + 2u * (lz >> 2))].x;
        const uint32_t c1 = s1[(lx >> 1) + 4u * ((ly >> 1) + 4u * (lz >> 1))].x;
        if ((int32_t)c2 <= (int32_t)kAdaptive) {
          v = ((D - 2u) << 28) | (level_offset_d(D - 2u) +
                                  lin3_lv(sx * 2u + (lx >> 2), sy * 2u + (ly >> 2), sz * 2u + (lz >> 2), D - 2u));
        } else if ((int32_t)c1 <= (int32_t)kAdaptive) {
          v = ((D - 1u) << 28) | (level_offset_d(D - 1u) +
                                  lin3_lv(sx * 4u + (lx >> 1), sy * 4u + (ly >> 1), sz * 4u + (lz >> 1), D - 1u));
        } else {
          v = (D << 28) | (level_offset_d(D) + lin3_lv(sx * 8u + lx, sy * 8u + ly, sz * 8u + lz, D));
        }
      }
      choice[S.cell_off + level_offset_d(D) + lin3_lv(sx * 8u + lx, sy * 8u + ly, sz * 8u + lz, D)] = v;
    }
  }

  if (s_last) {
    // Level r has at most 512 cells: stage it (written by other CTAs) via L2.
    const uint32_t nr = 1u << (3u * r);
    for (uint32_t i = tid; i < nr; i += blockDim.x)
      s0[i] = __ldcg(&mom[S.cell_off + level_offset_d(r) + i]);
    __syncthreads();
    // Sums of levels r-1 .. 0 into s_top (level l at level_offset(l)), then
    // their records in one pass.
    for (int l = (int)r - 1; l >= 0; l--) {
      const uint32_t nl = 1u << (3u * l);
      if (tid < nl) {
        uint32_t x, y, z;
        cell_coords_lv(tid, (uint32_t)l, x, y, z);
        const uint4 *child = l + 1 == (int)r ? s0 : s_top + level_offset_d((uint32_t)l + 1u);
        s_top[level_offset_d((uint32_t)l) + tid] = sum_children(child, x, y, z, 2u << l);
      }
      __syncthreads();
    }
    if (tid < level_offset_d(r)) {  // every cell of levels 0 .. r-1
      const uint4 acc = s_top[tid];
      store_cell(S, tid, acc, mom, src, aux);
      if ((int32_t)acc.x > (int32_t)kAdaptive) s_items[atomicAdd(&s_nitems, 1u)] = {scene, tid};
    }
  }
  __syncthreads();
  // Publish the parents listed by this subtree (and, in the scene's last
  // CTA, by the top levels).
  if (tid == 0 && s_nitems != 0u) {
    uint32_t base = atomicAdd(&ctr->parents[list_par], s_nitems);
    if (base + s_nitems > plist_cap) {
      atomicCAS(&ctr->error, 0u, (uint32_t)kDevErrListOverflow);
      s_nitems = base < plist_cap ? plist_cap - base : 0u;
    }
    s_base = base;
  }
  __syncthreads();
  for (uint32_t i = tid; i < s_nitems; i += blockDim.x) plist[s_base + i] = s_items[i];
  __syncthreads();
}

// The clearing CTAs of the upward pass: each warp takes 32 of the previous
// step's listed parents at a time (one per lane), then clears their 8
// children's 48-byte fields with one 16-byte store per lane (fields are zero
// off the M2L path).
__device__ __forceinline__ void clear_previous_fields(const SceneDesc *__restrict__ scenes,
                                                      float *__restrict__ fields,
                                                      const WorkItem *__restrict__ plist_prev,
                                                      Counters *__restrict__ ctr, uint32_t list_par,
                                                      uint32_t plist_cap, uint32_t clear_ctas,
                                                      unsigned long long *__restrict__ stamp) {
  const uint32_t tid = threadIdx.x;
  grid_dependency_wait();  // the previous integrate read the fields
  stamp_begin(stamp);
  if (blockIdx.x == 0 && tid == 0) {  // for this step's integrate and pair sums
    ctr->tile_cursor = 0u;
    ctr->p2p_cursor = 0u;
  }
  const uint32_t prev_n = min(ctr->parents[list_par ^ 1u], plist_cap);
  const uint32_t wpb = blockDim.x >> 5, lane = tid & 31u;
  const uint32_t ch = lane / 3u, part = lane % 3u;  // lanes 0..23: child, float4 of its field
  const uint32_t choff_x = ch & 1u, choff_y = (ch >> 1) & 1u, choff_z = ch >> 2;
  for (uint32_t i0 = (blockIdx.x * wpb + (tid >> 5)) * 32u; i0 < prev_n; i0 += clear_ctas * wpb * 32u) {
    uint32_t base = 0u, dim = 0u;
    if (i0 + lane < prev_n) {
      const WorkItem w = plist_prev[i0 + lane];
      const uint32_t lp = w.cell == 0u ? 0u : level_of_d(w.cell);
      uint32_t px, py, pz;
      cell_coords_lv(w.cell - level_offset_d(lp), lp, px, py, pz);
      dim = 2u << lp;
      base = scenes[w.scene].cell_off + level_offset_d(lp + 1u) + lin3(2u * px, 2u * py, 2u * pz, dim);
    }
    const uint32_t nb = min(32u, prev_n - i0);
    for (uint32_t j = 0; j < nb; j++) {
      const uint32_t b = __shfl_sync(0xFFFFFFFFu, base, j), d = __shfl_sync(0xFFFFFFFFu, dim, j);
      if (lane < 24u) {
        const uint32_t c = b + choff_x + d * (choff_y + d * choff_z);
        reinterpret_cast<float4 *>(fields)[(size_t)c * 3u + part] = make_float4(0.f, 0.f, 0.f, 0.f);
      }
    }
  }
  stamp_end(stamp);
  grid_dependents_may_launch();
}

// ----------------------------------------------------------- upward, warps
//
// One warp per 8x8x8-leaf subtree.  Lane L owns the subtree's level D-1
// cells 2L and 2L+1 in Morton order, so lanes 4p .. 4p+3 hold the eight
// children of level D-2 cell p: each lane sums its cells' leaves itself and
// two rounds of shuffles give the level D-2 cells, three more the root.  No
// CTA barrier is taken and a CTA works on eight subtrees at once.  Lane 0
// writes the root and takes the completion tickets; the scene's last warp
// reduces levels r-1 .. 0 the same way from the level-r cells.  All sums are
// integers modulo 2^32, so the order of addition does not matter.

// Block coordinates of Morton index m over s levels (x in the lowest bit).
__device__ __forceinline__ void morton_xyz(uint32_t m, uint32_t s, uint32_t &x, uint32_t &y, uint32_t &z) {
  x = y = z = 0u;
#pragma unroll
  for (uint32_t b = 0; b < 3u; b++) {
    if (b < s) {
      x |= ((m >> (3u * b)) & 1u) << b;
      y |= ((m >> (3u * b + 1u)) & 1u) << b;
      z |= ((m >> (3u * b + 2u)) & 1u) << b;
    }
  }
}

__device__ __forceinline__ uint4 shfl_xor_add(uint4 v, uint32_t mask) {
  return add_moment(v, make_uint4(__shfl_xor_sync(0xFFFFFFFFu, v.x, mask),
                                  __shfl_xor_sync(0xFFFFFFFFu, v.y, mask),
                                  __shfl_xor_sync(0xFFFFFFFFu, v.z, mask),
                                  __shfl_xor_sync(0xFFFFFFFFu, v.w, mask)));
}

// Lists up to four candidate cells per lane (count > 16, wgsl:472-476) with
// one atomic for the warp.
__device__ __forceinline__ void warp_list_parents(uint32_t scene, const uint32_t cell[4],
                                                  const bool want[4], WorkItem *__restrict__ plist,
                                                  uint32_t plist_cap, Counters *__restrict__ ctr,
                                                  uint32_t list_par) {
  const uint32_t lane = threadIdx.x & 31u, below = (1u << lane) - 1u;
  uint32_t ball[4], total = 0u;
#pragma unroll
  for (int i = 0; i < 4; i++) {
    ball[i] = __ballot_sync(0xFFFFFFFFu, want[i]);
    total += __popc(ball[i]);
  }
  if (total == 0u) return;
  uint32_t base = 0u;
  if (lane == 0u) {
    base = atomicAdd(&ctr->parents[list_par], total);
    if (base + total > plist_cap) atomicCAS(&ctr->error, 0u, (uint32_t)kDevErrListOverflow);
  }
  base = __shfl_sync(0xFFFFFFFFu, base, 0);
  uint32_t before = 0u;
#pragma unroll
  for (int i = 0; i < 4; i++) {
    const uint32_t at = base + before + __popc(ball[i] & below);
    if (want[i] && at < plist_cap) plist[at] = WorkItem{scene, cell[i]};
    before += __popc(ball[i]);
  }
}

__device__ __forceinline__ bool above_capacity(uint32_t count) {
  return (int32_t)count > (int32_t)kAdaptive;
}

__device__ __forceinline__ void upward_warp_task(
    const SceneDesc &S, uint32_t scene, uint32_t sub, uint4 *__restrict__ mom,
    uint4 *__restrict__ mom_next, float4 *__restrict__ src, float4 *__restrict__ aux,
    uint32_t *__restrict__ choice, WorkItem *__restrict__ plist, uint32_t plist_cap,
    Counters *__restrict__ ctr, uint32_t list_par, uint32_t *__restrict__ tickets) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t D = S.depth, r = S.sub_level;  // r = D - 3
  uint32_t sx, sy, sz;
  cell_coords_lv(sub, r, sx, sy, sz);
  const uint32_t leaf_base = S.cell_off + level_offset_d(D);
  // This lane's two level D-1 cells: block coordinates 0..3 per axis.
  uint32_t ux[2], uy[2], uz[2];
  uint4 c1[2];
  uint32_t seen = 0u;
#pragma unroll
  for (uint32_t j = 0; j < 2u; j++) {
    morton_xyz(2u * lane + j, 2u, ux[j], uy[j], uz[j]);
    uint4 acc = make_uint4(0u, 0u, 0u, 0u);
#pragma unroll
    for (uint32_t k = 0; k < 8u; k++) {
      const uint4 m = mom[leaf_base + lin3_lv(8u * sx + 2u * ux[j] + (k & 1u), 8u * sy + 2u * uy[j] + ((k >> 1) & 1u),
                                              8u * sz + 2u * uz[j] + (k >> 2), D)];
      seen |= m.x;
      acc = add_moment(acc, m);
    }
    c1[j] = acc;
  }
  // The subtree root in both moment buffers (see upward_task for why a
  // subtree empty in all of these has nothing to write).
  const uint32_t rcell = level_offset_d(r) + lin3_lv(sx, sy, sz, r);
  if (lane == 0u) seen |= mom[S.cell_off + rcell].x | mom_next[S.cell_off + rcell].x;
  const bool live = __any_sync(0xFFFFFFFFu, seen != 0u);
  uint4 c2 = make_uint4(0u, 0u, 0u, 0u), root = c2;
  if (live) {
    c2 = shfl_xor_add(shfl_xor_add(add_moment(c1[0], c1[1]), 1u), 2u);  // level D-2 cell lane >> 2
    root = shfl_xor_add(shfl_xor_add(shfl_xor_add(c2, 4u), 8u), 16u);
    if (lane == 0u) mom[S.cell_off + rcell] = root;
  }
  uint32_t last = 0u;
  if (lane == 0u) {
    const uint32_t ntasks = 1u << (3u * r);
    const uint32_t ngroups = (ntasks + kTicketGroup - 1u) / kTicketGroup;
    const uint32_t group = sub / kTicketGroup;
    const uint32_t gsize = min(kTicketGroup, ntasks - group * kTicketGroup);
    uint32_t *t = tickets + scene * kTicketStride;
    const uint32_t g_old = live ? atomic_add_acq_rel(&t[1u + group], 1u) : atomicAdd(&t[1u + group], 1u);
    if (g_old == gsize - 1u) {  // last subtree of its group
      if (!live) __threadfence();
      t[1u + group] = 0u;
      if (atomic_add_acq_rel(&t[0], 1u) == ngroups - 1u) {  // last group of the scene
        t[0] = 0u;
        last = 1u;
      }
    }
  }
  last = __shfl_sync(0xFFFFFFFFu, last, 0);

  if (live) {
    const uint32_t p = lane >> 2;  // this lane's level D-2 cell (Morton)
    uint32_t px, py, pz;
    morton_xyz(p, 1u, px, py, pz);
    uint32_t cell[4];
    bool want[4];
#pragma unroll
    for (uint32_t j = 0; j < 2u; j++) {
      // Leaves: source records and the cleared next-deposit leaf (the leaf
      // moments are read again, from L1).
#pragma unroll 1
      for (uint32_t k = 0; k < 8u; k++) {
        const uint32_t leaf = leaf_base + lin3_lv(8u * sx + 2u * ux[j] + (k & 1u),
                                                  8u * sy + 2u * uy[j] + ((k >> 1) & 1u),
                                                  8u * sz + 2u * uz[j] + (k >> 2), D);
        const uint4 m = mom[leaf];
        src[leaf] = make_source(m, S.scale, S.gravity, S.n_f);
        aux[leaf] = make_aux(m.x, S.gravity, S.n_f);
        mom_next[leaf] = make_uint4(0u, 0u, 0u, 0u);
        // Sample cell of the leaf: inside the subtree when its root holds
        // more than 16 bodies (the first of levels D-2, D-1 with count <= 16,
        // else the leaf), else unresolved.
        uint32_t v = kChoiceUnresolved;
        if (above_capacity(root.x)) {
          if (!above_capacity(c2.x)) {
            v = ((D - 2u) << 28) | (level_offset_d(D - 2u) + lin3_lv(2u * sx + px, 2u * sy + py, 2u * sz + pz, D - 2u));
          } else if (!above_capacity(c1[j].x)) {
            v = ((D - 1u) << 28) |
                (level_offset_d(D - 1u) + lin3_lv(4u * sx + ux[j], 4u * sy + uy[j], 4u * sz + uz[j], D - 1u));
          } else {
            v = (D << 28) | (leaf - S.cell_off);
          }
        }
        choice[leaf] = v;
      }
      // The level D-1 cell.
      cell[j] = level_offset_d(D - 1u) + lin3_lv(4u * sx + ux[j], 4u * sy + uy[j], 4u * sz + uz[j], D - 1u);
      store_cell(S, cell[j], c1[j], mom, src, aux);
      want[j] = above_capacity(c1[j].x);
    }
    cell[2] = level_offset_d(D - 2u) + lin3_lv(2u * sx + px, 2u * sy + py, 2u * sz + pz, D - 2u);
    want[2] = (lane & 3u) == 0u && above_capacity(c2.x);
    if ((lane & 3u) == 0u) store_cell(S, cell[2], c2, mom, src, aux);
    cell[3] = rcell;
    want[3] = lane == 0u && above_capacity(root.x);
    if (lane == 0u) store_cell(S, rcell, root, mom, src, aux);
    warp_list_parents(scene, cell, want, plist, plist_cap, ctr, list_par);
  }

  if (last) {
    // Levels r-1 .. 0 from the level-r cells (written by other warps; their
    // tickets released those writes to lane 0's acquire).
    __syncwarp();
    __threadfence();
    const uint32_t rbase = S.cell_off + level_offset_d(r);
    uint4 a = make_uint4(0u, 0u, 0u, 0u), b = a;  // level-2 cells 2L, 2L+1 (r >= 2) or level 1 (r == 1)
    uint32_t ax[2], ay[2], az[2];
#pragma unroll
    for (uint32_t j = 0; j < 2u; j++) morton_xyz(2u * lane + j, 2u, ax[j], ay[j], az[j]);
    if (r == 3u) {
#pragma unroll
      for (uint32_t j = 0; j < 2u; j++) {
        uint4 acc = make_uint4(0u, 0u, 0u, 0u);
#pragma unroll
        for (uint32_t k = 0; k < 8u; k++)
          acc = add_moment(acc, __ldcg(&mom[rbase + lin3_lv(2u * ax[j] + (k & 1u), 2u * ay[j] + ((k >> 1) & 1u),
                                                            2u * az[j] + (k >> 2), 3u)]));
        if (j == 0u) a = acc; else b = acc;
      }
    } else if (r == 2u) {
      a = __ldcg(&mom[rbase + lin3_lv(ax[0], ay[0], az[0], 2u)]);
      b = __ldcg(&mom[rbase + lin3_lv(ax[1], ay[1], az[1], 2u)]);
    } else if (lane < 8u) {
      uint32_t x, y, z;
      morton_xyz(lane, 1u, x, y, z);
      a = __ldcg(&mom[rbase + lin3_lv(x, y, z, 1u)]);
    }
    const uint4 l1 = shfl_xor_add(shfl_xor_add(add_moment(a, b), 1u), 2u);  // level-1 cell lane >> 2 (r >= 2)
    const uint4 l0 = r >= 2u ? shfl_xor_add(shfl_xor_add(shfl_xor_add(l1, 4u), 8u), 16u)
                             : shfl_xor_add(shfl_xor_add(shfl_xor_add(a, 1u), 2u), 4u);
    uint32_t cell[4] = {0u, 0u, 0u, 0u};
    bool want[4] = {false, false, false, false};
    if (r == 3u) {
#pragma unroll
      for (uint32_t j = 0; j < 2u; j++) {
        cell[j] = level_offset_d(2u) + lin3_lv(ax[j], ay[j], az[j], 2u);
        const uint4 v = j == 0u ? a : b;
        store_cell(S, cell[j], v, mom, src, aux);
        want[j] = above_capacity(v.x);
      }
    }
    if (r >= 2u && (lane & 3u) == 0u) {
      uint32_t x, y, z;
      morton_xyz(lane >> 2, 1u, x, y, z);
      cell[2] = level_offset_d(1u) + lin3_lv(x, y, z, 1u);
      store_cell(S, cell[2], l1, mom, src, aux);
      want[2] = above_capacity(l1.x);
    }
    if (lane == 0u) {
      cell[3] = 0u;
      store_cell(S, 0u, l0, mom, src, aux);
      want[3] = above_capacity(l0.x);
    }
    warp_list_parents(scene, cell, want, plist, plist_cap, ctr, list_par);
  }
}

// Persistent upward pass over the active subtree tasks (task_list, or every
// task when null).  The first `clear_ctas` CTAs only clear the fields of the
// previous step's targets (children of its listed parents; fields are zero
// off the M2L path), so the subtree CTAs start their reductions at once.
template <bool kWide>
__global__ void __launch_bounds__(256, 4) k_upward(const SceneDesc *__restrict__ scenes,
                                                const uint32_t *__restrict__ task_scene,
                                                const uint32_t *__restrict__ task_list,
                                                uint32_t ntasks_all,
                                                uint4 *__restrict__ mom, uint4 *__restrict__ mom_next,
                                                float4 *__restrict__ src, float4 *__restrict__ aux,
                                                uint32_t *__restrict__ choice,
                                                float *__restrict__ fields,
                                                WorkItem *__restrict__ plist, uint32_t plist_cap,
                                                const WorkItem *__restrict__ plist_prev,
                                                Counters *__restrict__ ctr, uint32_t list_par,
                                                uint32_t *__restrict__ tickets, uint32_t clear_ctas,
                                                uint32_t warp_min,
                                                unsigned long long *__restrict__ stamp) {
  __shared__ uint4 s0[512];
  __shared__ uint4 s1[64];
  __shared__ uint4 s2[9];     // level D-2, then the subtree root
  __shared__ uint4 s_top[73];  // levels 0 .. r-1 of the last CTA (r <= 3)
  __shared__ WorkItem s_items[160];  // a subtree's 73 cells + the top levels' 73
  __shared__ uint32_t s_nitems, s_base, s_last;
  __shared__ SceneDesc sS;
  if (blockIdx.x < clear_ctas) {
    clear_previous_fields(scenes, fields, plist_prev, ctr, list_par, plist_cap, clear_ctas, stamp);
    return;
  }

  // Scene descriptors and task lists change only by host copies, never by
  // the kernel this launch may overlap, so the first task's scene is staged
  // before waiting for that kernel.
  const uint32_t cta = blockIdx.x - clear_ctas, ncta = gridDim.x - clear_ctas;
  const uint32_t ntasks = task_list != nullptr ? min(ctr->tasks_active, ntasks_all) : ntasks_all;
  if (kWide && ntasks >= warp_min) {  // grid-uniform: one warp per subtree
    const uint32_t wpb = blockDim.x >> 5, warp = threadIdx.x >> 5;
    grid_dependency_wait();  // the previous integrate deposited into mom_next
    stamp_begin(stamp);
    for (uint32_t it = cta + ncta * warp; it < ntasks; it += ncta * wpb) {
      const uint32_t task = task_list != nullptr ? task_list[it] : it;
      const uint32_t scene = task_scene[task];
      const SceneDesc &S = scenes[scene];
      upward_warp_task(S, scene, task - S.task_off, mom, mom_next, src, aux, choice, plist, plist_cap,
                       ctr, list_par, tickets);
    }
    stamp_end(stamp);
    grid_dependents_may_launch();
    return;
  }
  uint32_t task = 0u, scene = 0u;
  if (cta < ntasks) {
    task = task_list != nullptr ? task_list[cta] : cta;
    scene = task_scene[task];
    load_scene(sS, scenes, scene);
  }
  grid_dependency_wait();  // the previous integrate deposited into mom_next
  stamp_begin(stamp);
  for (uint32_t it = cta; it < ntasks; it += ncta) {
    if (it != cta) {
      task = task_list != nullptr ? task_list[it] : it;
      scene = task_scene[task];
      load_scene(sS, scenes, scene);
    }
    upward_task(sS, scene, task - sS.task_off, mom, mom_next, src, aux, choice, plist, plist_cap,
                ctr, list_par, tickets, s0, s1, s2, s_top, s_items, s_nitems, s_base, s_last,
                it + ncta >= ntasks);
  }
  stamp_end(stamp);
  grid_dependents_may_launch();
}

// -------------------------------------------------------------------- M2L

constexpr uint32_t kTileCells = 216u;   // 6x6x6 children of a 3x3x3 parent block
constexpr uint32_t kChunk = 64u;        // stencil slots evaluated per pass (216 = 3 x 64 + 24)
constexpr uint32_t kSlotStride = 65u;   // padded so the 80 summing threads hit distinct banks
constexpr uint32_t kTmaBytes = kTileCells * 16u;

// Stencil slot k in the reference's loop order (source parent (pz, py, px),
// then child (cz, cy, cx)): bits 0-7 the slot's cell in the 6x6x6 tile, bit
// 8 + c set when the cell is adjacent to (or is) child c of the target parent.
__device__ __forceinline__ uint16_t m2l_slot_info(uint32_t k) {
  const uint32_t pidx = k >> 3, ch = k & 7u;
  const int ux = 2 * (int)(pidx % 3u) + (int)(ch & 1u);
  const int uy = 2 * (int)((pidx / 3u) % 3u) + (int)((ch >> 1) & 1u);
  const int uz = 2 * (int)(pidx / 9u) + (int)(ch >> 2);
  uint32_t near = 0u;
  for (uint32_t c = 0; c < 8u; c++) {
    // Source child coordinate minus target coordinate = u - 2 - child.
    const int sx = ux - 2 - (int)(c & 1u), sy = uy - 2 - (int)((c >> 1) & 1u), sz = uz - 2 - (int)(c >> 2);
    if (sx >= -1 && sx <= 1 && sy >= -1 && sy <= 1 && sz >= -1 && sz <= 1) near |= 1u << c;
  }
  return (uint16_t)((uint32_t)(ux + 6 * (uy + 6 * uz)) | (near << 8));
}

struct M2LShared {
  float4 tile[kTileCells];  // first member: 128-byte aligned by the launch
  unsigned long long mbar;
  uint32_t stop;
  uint32_t live[8];         // target cell of each child, or ~0 if the child is empty
  uint16_t slot_info[kTileCells];
  float vals[8][10][kSlotStride];
};

// The compacting variant: each child's contributing slots are listed first and
// evaluated 64 at a time (fewer evaluation rounds and additions when many
// slots are empty, one more pass over the stencil to build the lists).
constexpr uint32_t kRound = 64u;        // listed slots per round: two per lane
constexpr uint32_t kRoundStride = 65u;
struct M2LCompactShared {
  float4 tile[kTileCells];
  unsigned long long mbar;
  uint32_t stop;
  uint32_t live[8];
  uint32_t nvalid[8];            // contributing stencil slots of each child
  uint16_t slot_info[kTileCells];
  uint8_t slots[8][kTileCells];  // those slots, in the reference's loop order
  float vals[8][10][kRoundStride];
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(unsigned long long *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

// Bounded wait on an mbarrier phase (at most `polls` polls); returns false
// when it gave up.
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, uint32_t parity,
                                          uint32_t polls = 1u << 22) {
  const uint32_t addr = smem_u32(bar);
  for (uint32_t it = 0; it < polls; ++it) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(addr), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int x, int y, int z,
                                            unsigned long long *bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}

// M2L with one lane per target (long parent lists): a CTA's 8 warps take 32
// listed parents at a time, warp c handling child c of each (lane j: parent
// 32g + j).  The lanes of a warp walk the same 189 contributing stencil slots
// of child c (the 216 tile cells less the 27 adjacent to it), in the
// reference's loop order, each adding its terms to its own ten sums (no
// partial sum crosses lanes).  Source cells are read through L1.  `clist`
// holds per child the contributing slots' cell offsets in the 6x6x6 block
// (3 bits per axis), built once per CTA.
constexpr uint32_t kContrib = 189u;

__device__ __forceinline__ void build_child_slots(uint16_t (*clist)[kContrib]) {
  if (threadIdx.x < 8u) {
    const uint32_t c = threadIdx.x;
    uint32_t n = 0u;
    for (uint32_t k = 0; k < kTileCells; k++) {
      const uint32_t info = m2l_slot_info(k);
      if ((info >> (8u + c)) & 1u) continue;  // adjacent to (or is) child c
      const uint32_t t = info & 0xFFu;
      if (n < kContrib) clist[c][n++] = (uint16_t)((t % 6u) | (((t / 6u) % 6u) << 3) | ((t / 36u) << 6));
    }
  }
}

__device__ __forceinline__ void m2l_lanes_pass(const SceneDesc *__restrict__ scenes,
                                               const WorkItem *__restrict__ plist, uint32_t count,
                                               const uint4 *__restrict__ mom,
                                               const float4 *__restrict__ src,
                                               float *__restrict__ lfield,
                                               const uint16_t (*clist)[kContrib]) {
  const uint32_t lane = threadIdx.x & 31u, c = threadIdx.x >> 5;  // 256 threads: c = 0..7
  const uint16_t *cl = clist[c];
  const uint32_t groups = (count + 31u) / 32u;
  for (uint32_t g = blockIdx.x; g < groups; g += gridDim.x) {
    const uint32_t item = 32u * g + lane;
    const bool valid = item < count;
    const WorkItem w = valid ? plist[item] : WorkItem{0u, 0u};
    const SceneDesc &S = scenes[w.scene];
    const uint32_t lp = w.cell == 0u ? 0u : level_of_d(w.cell);
    const uint32_t l = lp + 1u, dim = 2u << lp;
    uint32_t upx, upy, upz;
    cell_coords_lv(w.cell - level_offset_d(lp), lp, upx, upy, upz);
    const int bx = 2 * (int)upx - 2, by = 2 * (int)upy - 2, bz = 2 * (int)upz - 2;
    const uint32_t lvl_base = S.cell_off + level_offset_d(l);
    const uint32_t tx = 2u * upx + (c & 1u), ty = 2u * upy + ((c >> 1) & 1u), tz = 2u * upz + (c >> 2);
    const uint32_t target = lvl_base + lin3(tx, ty, tz, dim);
    const bool live = valid && mom[target].x != 0u;  // empty children are not targets
    const float ctx = cell_center_lv(tx, l), cty = cell_center_lv(ty, l), ctz = cell_center_lv(tz, l);
    const float eps = (0.06f * kHalf) * pow2_neg(l);  // wgsl:507
    float acc[10];
#pragma unroll
    for (int k = 0; k < 10; k++) acc[k] = 0.0f;
    if (__any_sync(0xFFFFFFFFu, live)) {
      // Two consecutive slots per iteration: their pair terms are
      // independent chains (the square root and division of one overlap the
      // other's), and they are added in slot order.  The next two slots'
      // sources are requested meanwhile.
      auto fetch = [&](uint32_t k, float4 &sv) {
        const uint32_t e = cl[k];
        const int x = bx + (int)(e & 7u), y = by + (int)((e >> 3) & 7u), z = bz + (int)(e >> 6);
        sv = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (live && (uint32_t)x < dim && (uint32_t)y < dim && (uint32_t)z < dim)
          sv = __ldg(&src[lvl_base + lin3((uint32_t)x, (uint32_t)y, (uint32_t)z, dim)]);
      };
      static_assert(kContrib % 2u == 1u, "the loop below ends with one single slot");
      float4 n0, n1;
      fetch(0u, n0);
      fetch(1u, n1);
      for (uint32_t k = 0; k + 1u < kContrib; k += 2u) {
        const float4 s0 = n0, s1 = n1;
        fetch(k + 2u, n0);  // k + 2 <= kContrib - 1
        if (k + 3u < kContrib) fetch(k + 3u, n1);
        // Both 1/r chains first, then the terms slot by slot (absent and
        // empty slots read w = 0 and add nothing).
        const PairSetup p0 = pair_setup(s0, ctx, cty, ctz, eps);
        const PairSetup p1 = pair_setup(s1, ctx, cty, ctz, eps);
        if (s0.w != 0.0f) {
          float out[10];
          pair_terms(p0, out);
#pragma unroll
          for (int m = 0; m < 10; m++) acc[m] = acc[m] + out[m];
        }
        if (s1.w != 0.0f) {
          float out[10];
          pair_terms(p1, out);
#pragma unroll
          for (int m = 0; m < 10; m++) acc[m] = acc[m] + out[m];
        }
      }
      if (n0.w != 0.0f) {  // the last slot (kContrib - 1)
        float out[10];
        pair_field_d(n0, ctx, cty, ctz, eps, out);
#pragma unroll
        for (int m = 0; m < 10; m++) acc[m] = acc[m] + out[m];
      }
    }
    if (live) {
      float4 *fp = reinterpret_cast<float4 *>(lfield + (size_t)target * 12u);
      fp[0] = make_float4(acc[0], acc[1], acc[2], acc[3]);
      fp[1] = make_float4(acc[4], acc[5], acc[6], acc[7]);
      fp[2] = make_float4(acc[8], acc[9], 0.0f, 0.0f);
    }
  }
}

// The instance with the lane path gets up to 64 registers (4 CTAs per SM)
// for its two-slot chains; the one-scene instance keeps 40 (6 per SM).
template <bool kCompact, bool kWide>
__global__ void __launch_bounds__(256, kWide ? 4 : 6) k_m2l(const SceneDesc *__restrict__ scenes,
                                             const WorkItem *__restrict__ plist, uint32_t plist_cap,
                                             Counters *__restrict__ ctr, uint32_t list_par,
                                             const uint4 *__restrict__ mom,
                                             const float4 *__restrict__ src,
                                             float *__restrict__ lfield,
                                             const CUtensorMap *__restrict__ tmaps,
                                             uint32_t lane_min,
                                             unsigned long long *__restrict__ stamp) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ uint16_t s_clist[kWide ? 8 : 1][kContrib];  // the lane path's per-child slot lists
  // The TMA destination must be 128-byte aligned: align the carve-out by hand
  // (the launch reserves 128 spare bytes).
  const uint32_t pad = (128u - (smem_u32(smem_raw) & 127u)) & 127u;
  using Shared = typename std::conditional<kCompact, M2LCompactShared, M2LShared>::type;
  Shared &sh = *reinterpret_cast<Shared *>(smem_raw + pad);
  const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31u;
  if (tid == 0) {
    mbar_init(&sh.mbar, 1u);
    sh.stop = 0u;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  for (uint32_t k = tid; k < kTileCells; k += blockDim.x) sh.slot_info[k] = m2l_slot_info(k);
  if (kWide) build_child_slots(s_clist);
  grid_dependency_wait();  // the upward pass built the tree and the parent list
  stamp_begin(stamp);
  const uint32_t count = min(ctr->parents[list_par], plist_cap);
  if (blockIdx.x == 0 && tid == 0) ctr->parents[list_par ^ 1u] = 0u;  // reset for the next step
  __syncthreads();
  if (kWide && count >= lane_min) {  // grid-uniform
    m2l_lanes_pass(scenes, plist, count, mom, src, lfield, s_clist);
    stamp_end(stamp);
    grid_dependents_may_launch();
    return;
  }
  uint32_t phase = 0u;

  for (uint32_t item = blockIdx.x; item < count; item += gridDim.x) {
    const WorkItem w = plist[item];
    const SceneDesc &S = scenes[w.scene];
    const uint32_t lp = w.cell == 0u ? 0u : level_of_d(w.cell);
    const uint32_t l = lp + 1u, pdim = 1u << lp, dim = pdim << 1;
    const uint32_t pl = w.cell - level_offset_d(lp);
    uint32_t upx, upy, upz;
    cell_coords_lv(pl, lp, upx, upy, upz);
    const int pcx = (int)upx, pcy = (int)upy, pcz = (int)upz;
    const int bx = 2 * pcx - 2, by = 2 * pcy - 2, bz = 2 * pcz - 2;
    const uint32_t lvl_base = S.cell_off + level_offset_d(l);

    // Stage the 6x6x6 source tile (out-of-range cells read as zero).
    if (l >= 3u) {
      if (tid == 0) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_expect_tx(&sh.mbar, kTmaBytes);
        tma_load_3d(sh.tile, &tmaps[w.scene * 8u + l], 4 * bx, by, bz, &sh.mbar);
      }
    } else {
      for (uint32_t t = tid; t < kTileCells; t += blockDim.x) {
        const int x = bx + (int)(t % 6u), y = by + (int)((t / 6u) % 6u), z = bz + (int)(t / 36u);
        float4 v = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (x >= 0 && y >= 0 && z >= 0 && x < (int)dim && y < (int)dim && z < (int)dim)
          v = src[lvl_base + lin3((uint32_t)x, (uint32_t)y, (uint32_t)z, dim)];
        sh.tile[t] = v;
      }
    }
    // Warp w handles child w of the parent: its target cell, occupancy and
    // centre are read while the tile is in flight; then warp 0 alone waits
    // for the copy (the other warps wait at the barrier without issuing).
    const int cx = (int)(warp & 1u), cy = (int)((warp >> 1) & 1u), cz = (int)(warp >> 2);
    const uint32_t tx = (uint32_t)(2 * pcx + cx), ty = (uint32_t)(2 * pcy + cy), tz = (uint32_t)(2 * pcz + cz);
    const uint32_t target = lvl_base + lin3(tx, ty, tz, dim);
    const bool live = mom[target].x != 0u;  // empty children are not targets
    const float ctx = cell_center_lv(tx, l), cty = cell_center_lv(ty, l), ctz = cell_center_lv(tz, l);
    const float eps = (0.06f * kHalf) * pow2_neg(l);  // wgsl:507, / 2^l as an exact scaling
    if (l >= 3u) {
      if (warp == 0u && !mbar_wait(&sh.mbar, phase)) {
        // Give the copy in flight a second bounded wait before the CTA
        // leaves (its destination is this CTA's shared memory).
        (void)mbar_wait(&sh.mbar, phase);
        if (lane == 0u) {
          if (atomicCAS(&ctr->error, 0u, (uint32_t)kDevErrTmaTimeout) == 0u) ctr->error_info = item;
          sh.stop = 1u;
        }
      }
      phase ^= 1u;
    }
    __syncthreads();
    if (sh.stop) return;

    float acc = 0.0f;  // running sum of (child tid/10, component tid%10)
    if constexpr (kCompact) {
    // Warp w handles child w of the parent.  It first lists the stencil
    // slots that contribute (not adjacent to the child, non-empty source), in
    // the reference's loop order; then rounds of 64 listed slots are
    // evaluated, two per lane, and 80 threads (8 children x 10 components)
    // add each round to their running sums in list order.  Skipped slots
    // would add +0, which cannot change a sum that starts at +0.
    uint32_t nv = 0u;
    if (live) {
      for (uint32_t k0 = 0; k0 < kTileCells; k0 += 32u) {
        const uint32_t k = k0 + lane;
        bool use = false;
        uint32_t cell = 0u;
        if (k < kTileCells) {
          const uint32_t info = sh.slot_info[k];
          cell = info & 0xFFu;
          use = !((info >> (8u + warp)) & 1u) && sh.tile[cell].w != 0.0f;
        }
        const uint32_t mask = __ballot_sync(0xFFFFFFFFu, use);
        if (use) sh.slots[warp][nv + __popc(mask & ((1u << lane) - 1u))] = (uint8_t)cell;
        nv += __popc(mask);
      }
    }
    if (lane == 0) {
      sh.live[warp] = live ? target : 0xFFFFFFFFu;
      sh.nvalid[warp] = nv;
    }
    __syncthreads();
    uint32_t rounds = 0u;
#pragma unroll
    for (uint32_t w = 0; w < 8u; w++) rounds = max(rounds, (sh.nvalid[w] + kRound - 1u) / kRound);
    const uint32_t my_n = tid < 80u ? sh.nvalid[tid / 10u] : 0u;
    for (uint32_t r = 0; r < rounds; r++) {
      for (uint32_t h = 0; h < 2u; h++) {
        const uint32_t j = r * kRound + 32u * h + lane;
        if (j < nv) {
          const uint32_t cell = sh.slots[warp][j];
          float out[10];
          pair_field_d(sh.tile[cell], ctx, cty, ctz, eps, out);
#pragma unroll
          for (int c = 0; c < 10; c++) sh.vals[warp][c][32u * h + lane] = out[c];
        }
      }
      __syncthreads();
      if (tid < 80u && r * kRound < my_n) {
        const float *row = sh.vals[tid / 10u][tid % 10u];
        const uint32_t m = min(kRound, my_n - r * kRound);
        if (m == kRound) {
#pragma unroll
          for (uint32_t kk = 0; kk < kRound; kk++) acc = acc + row[kk];
        } else {
          for (uint32_t kk = 0; kk < m; kk++) acc = acc + row[kk];
        }
      }
      __syncthreads();
    }
    } else {
    // Warp w evaluates the stencil of child w of the parent, a chunk of slots
    // at a time; 80 threads (8 children x 10 components) then add the chunk to
    // their running sums, strictly in slot order.
    if (lane == 0) sh.live[warp] = live ? target : 0xFFFFFFFFu;
    for (uint32_t c0 = 0; c0 < kTileCells; c0 += kChunk) {
      const uint32_t m = min(kChunk, kTileCells - c0);
      if (live) {
        for (uint32_t kk = lane; kk < m; kk += 32u) {
          const uint32_t info = sh.slot_info[c0 + kk];
          const bool near = (info >> (8u + warp)) & 1u;
          const float4 src4 = sh.tile[info & 0xFFu];
          float out[10];
          if (!near && src4.w != 0.0f) {
            pair_field_d(src4, ctx, cty, ctz, eps, out);
          } else {
#pragma unroll
            for (int c = 0; c < 10; c++) out[c] = 0.0f;
          }
#pragma unroll
          for (int c = 0; c < 10; c++) sh.vals[warp][c][kk] = out[c];
        }
      }
      __syncthreads();
      if (tid < 80u && sh.live[tid / 10u] != 0xFFFFFFFFu) {
        const float *row = sh.vals[tid / 10u][tid % 10u];
#pragma unroll 8
        for (uint32_t kk = 0; kk < m; kk++) acc = acc + row[kk];
      }
      __syncthreads();
    }
    }
    if (tid < 96u) {
      const uint32_t t = tid < 80u ? tid / 10u : (tid - 80u) >> 1;
      const uint32_t tgt = sh.live[t];
      if (tgt != 0xFFFFFFFFu) {
        if (tid < 80u) {
          lfield[(size_t)tgt * 12u + tid % 10u] = acc;
        } else {
          lfield[(size_t)tgt * 12u + 10u + (tid & 1u)] = 0.0f;
        }
      }
    }
    __syncthreads();
  }
  stamp_end(stamp);
  grid_dependents_may_launch();
}

// --------------------------------------------------- L2L + near, lanes
//
// One lane per target (long parent lists): lane t of the pass takes child
// t & 7 of listed parent t >> 3 and carries all twelve field components
// itself, so the top-down chain needs no shuffles and the 26 near terms are
// added by the lane that forms them, in the same order as the warp path (an
// absent or empty neighbour adds nothing: the running field is never -0, so
// adding +0 would not change it).  Global warp w is warp w / gridDim.x of CTA
// w % gridDim.x, so the list spreads over every multiprocessor.
__device__ __forceinline__ void l2l_lanes_pass(const SceneDesc *__restrict__ scenes,
                                               const WorkItem *__restrict__ plist, uint32_t count,
                                               const uint4 *__restrict__ mom,
                                               const float4 *__restrict__ src,
                                               const float *__restrict__ lfield,
                                               float *__restrict__ fields) {
  const uint32_t lanes = 8u * count;
  const uint32_t stride = gridDim.x * (blockDim.x >> 5);
  for (uint32_t gw = blockIdx.x + gridDim.x * (threadIdx.x >> 5u); 32u * gw < lanes; gw += stride) {
    const uint32_t t = 32u * gw + (threadIdx.x & 31u);
    if (t >= lanes) continue;
    const WorkItem w = plist[t >> 3];
    const SceneDesc &S = scenes[w.scene];
    const uint32_t lp = w.cell == 0u ? 0u : level_of_d(w.cell);
    const uint32_t l = lp + 1u, dim = 2u << lp;
    uint32_t upx, upy, upz;
    cell_coords_lv(w.cell - level_offset_d(lp), lp, upx, upy, upz);
    const uint32_t ch = t & 7u;
    const uint32_t tx = 2u * upx + (ch & 1u), ty = 2u * upy + ((ch >> 1) & 1u), tz = 2u * upz + (ch >> 2);
    const uint32_t lvl_base = S.cell_off + level_offset_d(l);
    const uint32_t target = lvl_base + lin3(tx, ty, tz, dim);
    const uint32_t tcount = mom[target].x;
    if (tcount == 0u) continue;

    // f_a = m2l(a) + inherited(f_{a-1}) from the root field 0 (wgsl:574-611).
    float f[10];
#pragma unroll
    for (int k = 0; k < 10; k++) f[k] = 0.0f;
#pragma unroll
    for (uint32_t a = 1u; a <= 6u; a++) {
      if (a <= l) {
        const uint32_t sh_ = l - a;
        const uint32_t ax = tx >> sh_, ay = ty >> sh_, az = tz >> sh_;
        const float4 *gp = reinterpret_cast<const float4 *>(
            lfield + (size_t)(S.cell_off + level_offset_d(a) + lin3_lv(ax, ay, az, a)) * 12u);
        const float4 g0 = __ldg(gp), g1 = __ldg(gp + 1), g2 = __ldg(gp + 2);
        const float dx = cell_center_lv(ax, a) - cell_center_lv(ax >> 1, a - 1u);
        const float dy = cell_center_lv(ay, a) - cell_center_lv(ay >> 1, a - 1u);
        const float dz = cell_center_lv(az, a) - cell_center_lv(az >> 1, a - 1u);
        // a += J . delta, phi -= a . delta, J unchanged (wgsl:603-609).
        const float tax = (f[4] * dx + f[5] * dy) + f[6] * dz;
        const float tay = (f[5] * dx + f[7] * dy) + f[8] * dz;
        const float taz = (f[6] * dx + f[8] * dy) + f[9] * dz;
        const float tph = (f[0] * dx + f[1] * dy) + f[2] * dz;
        f[0] = g0.x + (f[0] + tax);
        f[1] = g0.y + (f[1] + tay);
        f[2] = g0.z + (f[2] + taz);
        f[3] = g0.w + (f[3] + (-tph));
        f[4] = g1.x + f[4];
        f[5] = g1.y + f[5];
        f[6] = g1.z + f[6];
        f[7] = g1.w + f[7];
        f[8] = g2.x + f[8];
        f[9] = g2.y + f[9];
      }
    }

    const bool leaf = tcount <= kAdaptive || l == S.depth;  // wgsl:537-541
    if (leaf && S.near_mode == kNearReference) {
      const float ctx = cell_center_lv(tx, l), cty = cell_center_lv(ty, l), ctz = cell_center_lv(tz, l);
      const float near_eps = fmaxf(S.softening, (0.72f * kHalf) * pow2_neg(l));
      for (uint32_t j = 0; j < 27u; j++) {
        if (j == 13u) continue;  // the target itself
        const int sx = (int)tx + (int)(j % 3u) - 1, sy = (int)ty + (int)((j / 3u) % 3u) - 1,
                  sz = (int)tz + (int)(j / 9u) - 1;
        if (sx < 0 || sy < 0 || sz < 0 || sx >= (int)dim || sy >= (int)dim || sz >= (int)dim) continue;
        const float4 s = __ldg(&src[lvl_base + lin3((uint32_t)sx, (uint32_t)sy, (uint32_t)sz, dim)]);
        if (s.w == 0.0f) continue;
        float out[10];
        pair_field_d(s, ctx, cty, ctz, near_eps, out);
#pragma unroll
        for (int k = 0; k < 10; k++) f[k] = f[k] + out[k];
      }
    }
    float4 *fp = reinterpret_cast<float4 *>(fields + (size_t)target * 12u);
    fp[0] = make_float4(f[0], f[1], f[2], f[3]);
    fp[1] = make_float4(f[4], f[5], f[6], f[7]);
    fp[2] = make_float4(f[8], f[9], 0.0f, 0.0f);
  }
}

// ------------------------------------------------------------ L2L + near

struct L2LShared {
  float vals[8][10][27];
  float centre[127];  // cell_center_lv(c, l) at [2^l - 1 + c], levels 0..6
};

template <bool kWide>
__global__ void __launch_bounds__(256) k_l2l_near(const SceneDesc *__restrict__ scenes,
                                                  const WorkItem *__restrict__ plist,
                                                  uint32_t plist_cap,
                                                  const Counters *__restrict__ ctr,
                                                  uint32_t list_par, const uint4 *__restrict__ mom,
                                                  const float4 *__restrict__ src,
                                                  const float *__restrict__ lfield,
                                                  float *__restrict__ fields,
                                                  uint32_t lane_min,
                                                  unsigned long long *__restrict__ stamp) {
  __shared__ L2LShared sh;
  const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31u;
  if (tid < 127u) {
    const uint32_t l = 31u - (uint32_t)__clz((int)(tid + 1u));
    sh.centre[tid] = cell_center_lv(tid + 1u - (1u << l), l);
  }
  grid_dependency_wait();  // M2L results of every target are complete
  stamp_begin(stamp);
  const uint32_t count = min(ctr->parents[list_par], plist_cap);
  // Lane c < 12 owns field component c (ax ay az phi Jxx Jxy Jxz Jyy Jyz Jzz 0 0).
  const uint32_t c = lane < 12u ? lane : 11u;
  // The translation of component c < 4 is f_c +/- ((f_b dx + f_c' dy) + f_d dz):
  // the source lanes of its three terms and its sign.
  constexpr uint32_t kSrcB = 0x0654u, kSrcC = 0x1875u, kSrcD = 0x2986u;  // 4 bits per lane 0..3
  const uint32_t sb = lane < 4u ? (kSrcB >> (4u * lane)) & 15u : lane;
  const uint32_t sc = lane < 4u ? (kSrcC >> (4u * lane)) & 15u : lane;
  const uint32_t sd = lane < 4u ? (kSrcD >> (4u * lane)) & 15u : lane;
  __syncthreads();
  if (kWide && count >= lane_min) {  // grid-uniform
    l2l_lanes_pass(scenes, plist, count, mom, src, lfield, fields);
    stamp_end(stamp);
    grid_dependents_may_launch();
    return;
  }
  for (uint32_t item = blockIdx.x; item < count; item += gridDim.x) {
    const WorkItem w = plist[item];
    const SceneDesc &S = scenes[w.scene];
    const uint32_t lp = w.cell == 0u ? 0u : level_of_d(w.cell);
    const uint32_t l = lp + 1u, pdim = 1u << lp, dim = pdim << 1;
    const uint32_t pl = w.cell - level_offset_d(lp);
    uint32_t upx, upy, upz;
    cell_coords_lv(pl, lp, upx, upy, upz);
    const uint32_t tx = 2u * upx + (warp & 1u);
    const uint32_t ty = 2u * upy + ((warp >> 1) & 1u);
    const uint32_t tz = 2u * upz + (warp >> 2);
    const uint32_t lvl_base = S.cell_off + level_offset_d(l);
    const uint32_t target = lvl_base + lin3(tx, ty, tz, dim);
    // The target's count, its ancestors' M2L components (lane c reads
    // component c) and its 26 neighbours' sources (lane j < 26) do not depend
    // on one another: all are requested before the count is tested.
    const uint32_t tcount = mom[target].x;
    float g[6];
#pragma unroll
    for (uint32_t a = 1u; a <= 6u; a++) {
      g[a - 1] = 0.0f;
      if (a <= l) {
        const uint32_t sh_ = l - a;
        const uint32_t anc = S.cell_off + level_offset_d(a) + lin3_lv(tx >> sh_, ty >> sh_, tz >> sh_, a);
        g[a - 1] = __ldg(lfield + (size_t)anc * 12u + c);
      }
    }
    float4 nsrc = make_float4(0.0f, 0.0f, 0.0f, 0.0f);  // w = 0: no term
    if (lane < 26u && S.near_mode == kNearReference) {
      const uint32_t j = lane < 13u ? lane : lane + 1u;  // skip the centre (13)
      const int dx = (int)(j % 3u) - 1, dy = (int)((j / 3u) % 3u) - 1, dz = (int)(j / 9u) - 1;
      const int sx = (int)tx + dx, sy = (int)ty + dy, sz = (int)tz + dz;
      if (sx >= 0 && sy >= 0 && sz >= 0 && sx < (int)dim && sy < (int)dim && sz < (int)dim)
        nsrc = __ldg(&src[lvl_base + lin3((uint32_t)sx, (uint32_t)sy, (uint32_t)sz, dim)]);
    }
    if (tcount == 0u) continue;  // warp-uniform

    // Top-down chain f_a = m2l(a) + translate(f_{a-1}) from the root field 0
    // (the reference never writes cell 0's field, wgsl:459).
    float f = 0.0f;
#pragma unroll
    for (uint32_t a = 1u; a <= 6u; a++) {
      if (a <= l) {
        const uint32_t sh_ = l - a;
        const uint32_t ax = tx >> sh_, ay = ty >> sh_, az = tz >> sh_;
        const float *cen = sh.centre + (1u << a) - 1u, *pcen = sh.centre + (1u << (a - 1u)) - 1u;
        const float dx = cen[ax] - pcen[ax >> 1];
        const float dy = cen[ay] - pcen[ay >> 1];
        const float dz = cen[az] - pcen[az >> 1];
        // inherited (wgsl:603-609): a += J . delta, phi -= a . delta, J unchanged:
        //   ax + ((Jxx dx + Jxy dy) + Jxz dz), ay + ((Jxy dx + Jyy dy) + Jyz dz),
        //   az + ((Jxz dx + Jyz dy) + Jzz dz), phi - ((ax dx + ay dy) + az dz)
        // (x - t == x + (-t) exactly).
        const float vb = __shfl_sync(0xFFFFFFFFu, f, sb);
        const float vc = __shfl_sync(0xFFFFFFFFu, f, sc);
        const float vd = __shfl_sync(0xFFFFFFFFu, f, sd);
        const float t = (vb * dx + vc * dy) + vd * dz;
        const float inh = lane < 4u ? f + (lane == 3u ? -t : t) : f;
        f = g[a - 1] + inh;
      }
    }

    const bool leaf = tcount <= kAdaptive || l == S.depth;  // wgsl:537-541
    if (leaf && S.near_mode == kNearReference) {
      const float ctx = cell_center_lv(tx, l), cty = cell_center_lv(ty, l),
                  ctz = cell_center_lv(tz, l);
      const float near_eps = fmaxf(S.softening, (0.72f * kHalf) * pow2_neg(l));
      if (lane < 26u) {
        float out[10];
#pragma unroll
        for (int k = 0; k < 10; k++) out[k] = 0.0f;
        if (nsrc.w != 0.0f) pair_field_d(nsrc, ctx, cty, ctz, near_eps, out);
#pragma unroll
        for (int k = 0; k < 10; k++) sh.vals[warp][k][lane] = out[k];
      }
      __syncwarp();
      if (lane < 10u) {
        const float *row = sh.vals[warp][lane];
        for (uint32_t k = 0; k < 26u; k++) f = f + row[k];
      }
      __syncwarp();
    }
    if (lane < 12u) fields[(size_t)target * 12u + lane] = f;
  }
  stamp_end(stamp);
  grid_dependents_may_launch();
}

// ------------------------------------------------------- wait self-check

// One CTA waits, with the kernels' bounded wait, on an mbarrier phase that
// nothing completes (no thread arrives, no copy is issued), then writes
// kDevErrTmaTimeout to *status when the wait gave up as it must.  Nothing is
// in flight, so the CTA leaves cleanly and the context stays usable.
__global__ void __launch_bounds__(32) k_wait_check(uint32_t polls, uint32_t *__restrict__ status) {
  __shared__ unsigned long long bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1u);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncwarp();
  const bool done = mbar_wait(&bar, 0u, polls);
  if (threadIdx.x == 0) *status = done ? (uint32_t)kDevErrNone : (uint32_t)kDevErrTmaTimeout;
}

void launch_wait_check(cudaStream_t stream, uint32_t polls, uint32_t *status) {
  k_wait_check<<<1, 32, 0, stream>>>(polls, status);
}

// --------------------------------------------------------------- launches

// Work-list lengths from which the warp-per-subtree and lane-per-target
// paths run, per tuning value (0: never, 1: always, 2: from the measured
// crossovers: subtree tasks for the upward pass, listed parents for M2L and
// L2L + near).
constexpr uint32_t kNever = 0xFFFFFFFFu;
constexpr uint32_t kUpwardWarpAuto = 4096u;
constexpr uint32_t kM2LLaneAuto = 16384u;
constexpr uint32_t kL2LLaneAuto = 2048u;
static uint32_t lane_min(uint32_t mode, uint32_t automatic) {
  return mode == 0u ? kNever : (mode == 1u ? 0u : automatic);
}
// The kernels carrying the second path are launched only where it can run:
// forced on, or automatic in an engine of several scenes (one scene's lists
// stay below the crossovers; the second path's code costs the per-item path
// registers and time).
static bool wide(uint32_t mode, const LaunchCtx &L) { return mode == 1u || (mode == 2u && L.many_scenes); }

void launch_upward(const LaunchCtx &L, uint32_t list_par, uint32_t tasks) {
  const uint32_t grid = tasks < L.tree_ctas ? tasks : L.tree_ctas;
  // Clearing CTAs: one pass of 32 parents per warp covers 8 * 32 * clear_ctas
  // listed parents.
  uint32_t clear = (L.plist_cap + 2047u) / 2048u;
  clear = clear < 8u ? 8u : (clear > 64u ? 64u : clear);
  launch_step_kernel(L, wide(L.upward_warps, L) ? k_upward<true> : k_upward<false>, dim3(grid + clear),
                     dim3(256), 0, L.scenes, L.task_scene,
                     L.task_list, tasks, L.mom, L.mom_next, L.src, L.aux, L.choice, L.fields,
                     L.plist, L.plist_cap, L.plist_prev, L.ctr, list_par, L.tickets, clear,
                     lane_min(L.upward_warps, kUpwardWarpAuto), stamp_rec(L, 0u));
}

size_t m2l_smem_bytes(bool compact) {
  return (compact ? sizeof(M2LCompactShared) : sizeof(M2LShared)) + 128;
}

void launch_m2l(const LaunchCtx &L, uint32_t list_par) {
  const bool w = wide(L.m2l_lanes, L);
  auto kernel = L.m2l_compact ? (w ? k_m2l<true, true> : k_m2l<true, false>)
                              : (w ? k_m2l<false, true> : k_m2l<false, false>);
  launch_step_kernel(L, kernel, dim3(L.m2l_ctas), dim3(256),
                     m2l_smem_bytes(L.m2l_compact), L.scenes,
                     (const WorkItem *)L.plist, L.plist_cap, L.ctr, list_par, (const uint4 *)L.mom,
                     (const float4 *)L.src, L.lfield, L.tmaps, lane_min(L.m2l_lanes, kM2LLaneAuto),
                     stamp_rec(L, 1u));
}

void launch_l2l_near(const LaunchCtx &L, uint32_t list_par) {
  launch_step_kernel(L, wide(L.l2l_lanes, L) ? k_l2l_near<true> : k_l2l_near<false>, dim3(L.l2l_ctas),
                     dim3(256), 0, L.scenes, (const WorkItem *)L.plist,
                     L.plist_cap, (const Counters *)L.ctr, list_par, (const uint4 *)L.mom,
                     (const float4 *)L.src, (const float *)L.lfield, L.fields,
                     lane_min(L.l2l_lanes, kL2LLaneAuto), stamp_rec(L, 2u));
}

cudaError_t configure_tree_kernels() {
  cudaError_t e = cudaSuccess;
  const std::pair<void (*)(const SceneDesc *, const WorkItem *, uint32_t, Counters *, uint32_t,
                            const uint4 *, const float4 *, float *, const CUtensorMap *, uint32_t,
                            unsigned long long *),
                  bool>
      m2l[4] = {{k_m2l<false, false>, false}, {k_m2l<false, true>, false}, {k_m2l<true, false>, true},
                {k_m2l<true, true>, true}};
  for (const auto &k : m2l)
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k.first, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)m2l_smem_bytes(k.second));
  return e;
}

RFMM_KERNEL_NS_END
