// Resident-order sorts: a stable LSD radix sort of (key, value) pairs with
// 8-bit digits (uploads and the P2P mode's per-step sort), and the leaf
// counting sort that refreshes the order of resident bodies.
//
// The radix sort orders bodies by (scene, Morton leaf key) so each leaf's bodies are
// contiguous: leaf membership and occupancy then come from runs of equal
// keys, and the deposit is a segmented reduction over those runs.  The sort
// is stable, so the resident order is a deterministic function of the input.
//
// Per 8-bit pass:
//   k_sort_hist     per 2048-key tile, digit histogram in shared memory
//   k_sort_scan     one CTA per digit: exclusive scan of that digit's tile
//                   counts (digit-major layout), plus the digit total
//   k_sort_scatter  per tile: digit base + tile offset + stable rank inside
//                   the tile (warp __match_any_sync ranks, warp prefix in
//                   shared memory), then scatter
#include <cuda_runtime.h>

#include "rfmm_device.cuh"
#include "rfmm_kernels.h"

namespace rfmm {

constexpr uint32_t kSortThreads = 256u;
constexpr uint32_t kSortItems = 8u;
constexpr uint32_t kSortTile = kSortThreads * kSortItems;  // 2048 keys

uint32_t sort_tiles(uint32_t n) { return (n + kSortTile - 1u) / kSortTile; }

__global__ void __launch_bounds__(kSortThreads) k_sort_hist(const uint32_t *__restrict__ keys,
                                                            uint32_t n, uint32_t shift,
                                                            uint32_t *__restrict__ hist,
                                                            uint32_t ntiles) {
  __shared__ uint32_t h[256];
  const uint32_t tid = threadIdx.x, tile = blockIdx.x;
  h[tid] = 0u;
  __syncthreads();
  for (uint32_t r = 0; r < kSortItems; r++) {
    const uint32_t i = tile * kSortTile + r * kSortThreads + tid;
    if (i < n) atomicAdd(&h[(keys[i] >> shift) & 255u], 1u);
  }
  __syncthreads();
  hist[tid * ntiles + tile] = h[tid];
}

// Block-wide exclusive scan of one value per thread (256 threads).
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t *warp_sums,
                                                         uint32_t &total) {
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (uint32_t off = 1u; off < 32u; off <<= 1) {
    const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, off);
    if (lane >= off) x += y;
  }
  if (lane == 31u) warp_sums[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t s = lane < (blockDim.x >> 5) ? warp_sums[lane] : 0u;
#pragma unroll
    for (uint32_t off = 1u; off < 32u; off <<= 1) {
      const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, s, off);
      if (lane >= off) s += y;
    }
    if (lane < (blockDim.x >> 5)) warp_sums[lane] = s;
  }
  __syncthreads();
  const uint32_t before = warp == 0 ? 0u : warp_sums[warp - 1];
  total = warp_sums[(blockDim.x >> 5) - 1];
  __syncthreads();
  return before + x - v;
}

__global__ void __launch_bounds__(kSortThreads) k_sort_scan(uint32_t *__restrict__ hist,
                                                            uint32_t ntiles,
                                                            uint32_t *__restrict__ totals) {
  __shared__ uint32_t warp_sums[32];
  uint32_t *row = hist + blockIdx.x * ntiles;
  uint32_t carry = 0u;
  for (uint32_t base = 0; base < ntiles; base += kSortThreads) {
    const uint32_t i = base + threadIdx.x;
    const uint32_t v = i < ntiles ? row[i] : 0u;
    uint32_t chunk_total;
    const uint32_t ex = block_exclusive_scan(v, warp_sums, chunk_total);
    if (i < ntiles) row[i] = carry + ex;
    carry += chunk_total;
  }
  if (threadIdx.x == 0) totals[blockIdx.x] = carry;
}

__global__ void __launch_bounds__(kSortThreads) k_sort_scatter(
    const uint32_t *__restrict__ keys_in, const uint32_t *__restrict__ vals_in,
    uint32_t *__restrict__ keys_out, uint32_t *__restrict__ vals_out, uint32_t n, uint32_t shift,
    const uint32_t *__restrict__ hist, const uint32_t *__restrict__ totals, uint32_t ntiles) {
  __shared__ uint32_t base[256];
  __shared__ uint32_t wcnt[kSortThreads / 32u][256];
  __shared__ uint32_t warp_sums[32];
  const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5, tile = blockIdx.x;
  {
    uint32_t total;
    const uint32_t digit_base = block_exclusive_scan(totals[tid], warp_sums, total);
    base[tid] = digit_base + hist[tid * ntiles + tile];
  }
  const uint32_t lt_mask = (1u << lane) - 1u;
  for (uint32_t r = 0; r < kSortItems; r++) {
#pragma unroll
    for (uint32_t w = 0; w < kSortThreads / 32u; w++) wcnt[w][tid] = 0u;
    __syncthreads();
    const uint32_t i = tile * kSortTile + r * kSortThreads + tid;
    const bool valid = i < n;
    const uint32_t key = valid ? keys_in[i] : 0u;
    const uint32_t digit = valid ? ((key >> shift) & 255u) : 256u + lane;
    const uint32_t peers = __match_any_sync(0xFFFFFFFFu, digit);
    const uint32_t rank = __popc(peers & lt_mask);
    if (valid && rank == 0u) wcnt[warp][digit] = __popc(peers);
    __syncthreads();
    {
      uint32_t run = base[tid];
#pragma unroll
      for (uint32_t w = 0; w < kSortThreads / 32u; w++) {
        const uint32_t c = wcnt[w][tid];
        wcnt[w][tid] = run;
        run += c;
      }
      base[tid] = run;
    }
    __syncthreads();
    if (valid) {
      const uint32_t pos = wcnt[warp][digit] + rank;
      if (pos < n) {  // defensive: offsets from the histograms stay below n
        keys_out[pos] = key;
        vals_out[pos] = vals_in[i];
      }
    }
    __syncthreads();
  }
}

int radix_sort(cudaStream_t stream, SortScratch &s, uint32_t n, uint32_t bits) {
  const uint32_t ntiles = sort_tiles(n);
  int cur = 0;
  for (uint32_t shift = 0; shift < bits; shift += 8u) {
    k_sort_hist<<<ntiles, kSortThreads, 0, stream>>>(s.keys[cur], n, shift, s.hist, ntiles);
    k_sort_scan<<<256, kSortThreads, 0, stream>>>(s.hist, ntiles, s.totals);
    k_sort_scatter<<<ntiles, kSortThreads, 0, stream>>>(s.keys[cur], s.vals[cur], s.keys[cur ^ 1],
                                                        s.vals[cur ^ 1], n, shift, s.hist,
                                                        s.totals, ntiles);
    cur ^= 1;
  }
  return cur;
}

// ------------------------------------------------ leaf counting-sort resort
//
// The periodic refresh of the resident leaf order.  The leaf counts of the
// current positions are already known (integrate deposited them into the next
// step's moments), so bodies are bucketed by leaf with one exclusive scan of
// the counts in Morton order of the leaves and one scatter:
//   k_leaf_block_sums  per 4096-leaf block of a scene, the sum of its counts
//   k_leaf_block_scan  per scene, exclusive scan of its block sums (+ body_off)
//   k_leaf_offsets     per block, exclusive scan of its counts -> first slot of
//                      every leaf (starts, at the scene's cell offset)
//   k_leaf_scatter     every body takes the next slot of its leaf (one atomic
//                      per leaf group of a warp) and moves there with its id
// Bodies of one leaf land in an arbitrary order, which no result depends on:
// each body's update reads only its own state and the tree, and the moment
// sums are exact integers.

namespace {

constexpr uint32_t kLeafBlock = 4096u;
constexpr uint32_t kLeafThreads = 1024u;

__device__ __forceinline__ uint32_t compact3(uint32_t v) {  // inverse of a 3-D bit spread
  v &= 0x09249249u;
  v = (v | (v >> 2)) & 0x030C30C3u;
  v = (v | (v >> 4)) & 0x0300F00Fu;
  v = (v | (v >> 8)) & 0x030000FFu;
  v = (v | (v >> 16)) & 0x000003FFu;
  return v;
}

__device__ __forceinline__ uint32_t spread3s(uint32_t v) {
  v &= 0x3FFu;
  v = (v | (v << 16)) & 0x030000FFu;
  v = (v | (v << 8)) & 0x0300F00Fu;
  v = (v | (v << 4)) & 0x030C30C3u;
  v = (v | (v << 2)) & 0x09249249u;
  return v;
}

// Count of the leaf with Morton index m (x in bit 0) of scene S.
__device__ __forceinline__ uint32_t leaf_count(const SceneDesc &S, const uint4 *mom, uint32_t m) {
  const uint32_t D = S.depth;
  const uint32_t x = compact3(m), y = compact3(m >> 1), z = compact3(m >> 2);
  return mom[S.cell_off + level_offset_d(D) + (x | (y << D) | (z << (2u * D)))].x;
}

// Sum over the 1024-thread block (every thread gets the total).
__device__ __forceinline__ uint32_t block_sum_1024(uint32_t v, uint32_t *warp_buf) {
  for (uint32_t off = 16u; off > 0u; off >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, off);
  __syncthreads();
  if ((threadIdx.x & 31u) == 0u) warp_buf[threadIdx.x >> 5] = v;
  __syncthreads();
  uint32_t t = warp_buf[threadIdx.x & 31u];
  for (uint32_t off = 16u; off > 0u; off >>= 1) t += __shfl_xor_sync(0xFFFFFFFFu, t, off);
  return t;
}

}  // namespace

// The leaf-sort kernels walk scene rows: row y is scene y, or, with an
// active-scene list (serving slots), rows y, y + gridDim, ... take the listed
// scenes in turn.
__device__ __forceinline__ uint32_t scene_rows(const uint32_t *scene_list, const Counters *ctr,
                                               uint32_t scenes) {
  return scene_list != nullptr ? min(ctr->scenes_active, scenes) : scenes;
}

__global__ void __launch_bounds__(kLeafThreads) k_leaf_block_sums(const SceneDesc *__restrict__ scenes,
                                                                  uint32_t nscenes,
                                                                  const uint32_t *__restrict__ scene_list,
                                                                  const Counters *__restrict__ ctr,
                                                                  const uint4 *__restrict__ mom,
                                                                  uint32_t *__restrict__ block_sums,
                                                                  uint32_t max_blocks,
                                                                  unsigned long long *__restrict__ stamp) {
  __shared__ uint32_t warp_buf[32];
  stamp_begin(stamp);  // first of the resort's four kernels
  const uint32_t rows = scene_rows(scene_list, ctr, nscenes);
  for (uint32_t y = blockIdx.y; y < rows; y += gridDim.y) {
    const uint32_t sc = scene_list != nullptr ? scene_list[y] : y;
    const SceneDesc &S = scenes[sc];
    const uint32_t leaves = 1u << (3u * S.depth);
    const uint32_t base = blockIdx.x * kLeafBlock;
    if (S.n == 0u || base >= leaves) continue;  // block-uniform
    uint32_t v = 0u;
    for (uint32_t k = 0; k < kLeafBlock / kLeafThreads; k++) {
      const uint32_t m = base + k * kLeafThreads + threadIdx.x;
      if (m < leaves) v += leaf_count(S, mom, m);
    }
    v = block_sum_1024(v, warp_buf);
    if (threadIdx.x == 0) block_sums[sc * max_blocks + blockIdx.x] = v;
  }
}

// One warp per scene: exclusive scan of the scene's block sums (at most 64
// blocks: depth <= 6), offset by the scene's first slot.
__global__ void __launch_bounds__(32) k_leaf_block_scan(const SceneDesc *__restrict__ scenes,
                                                        uint32_t nscenes,
                                                        const uint32_t *__restrict__ scene_list,
                                                        const Counters *__restrict__ ctr,
                                                        uint32_t *__restrict__ block_sums,
                                                        uint32_t max_blocks) {
  const uint32_t rows = scene_rows(scene_list, ctr, nscenes);
  for (uint32_t y = blockIdx.x; y < rows; y += gridDim.x) {
    const uint32_t sc = scene_list != nullptr ? scene_list[y] : y;
    const SceneDesc &S = scenes[sc];
    if (S.n == 0u) continue;
    const uint32_t lane = threadIdx.x;
    const uint32_t nb = ((1u << (3u * S.depth)) + kLeafBlock - 1u) / kLeafBlock;
    uint32_t *row = block_sums + sc * max_blocks;
    // Lane l holds blocks 2l and 2l + 1.
    const uint32_t a = 2u * lane < nb ? row[2u * lane] : 0u;
    const uint32_t b = 2u * lane + 1u < nb ? row[2u * lane + 1u] : 0u;
    uint32_t x = a + b;
    for (uint32_t off = 1u; off < 32u; off <<= 1) {
      const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, x, off);
      if (lane >= off) x += t;
    }
    const uint32_t before = S.body_off + x - (a + b);
    if (2u * lane < nb) row[2u * lane] = before;
    if (2u * lane + 1u < nb) row[2u * lane + 1u] = before + a;
  }
}

__global__ void __launch_bounds__(kLeafThreads) k_leaf_offsets(const SceneDesc *__restrict__ scenes,
                                                               uint32_t nscenes,
                                                               const uint32_t *__restrict__ scene_list,
                                                               const Counters *__restrict__ ctr,
                                                               const uint4 *__restrict__ mom,
                                                               const uint32_t *__restrict__ block_offs,
                                                               uint32_t max_blocks,
                                                               uint32_t *__restrict__ starts) {
  __shared__ uint32_t warp_sums[32];
  const uint32_t rows = scene_rows(scene_list, ctr, nscenes);
  for (uint32_t y = blockIdx.y; y < rows; y += gridDim.y) {
    const uint32_t sc = scene_list != nullptr ? scene_list[y] : y;
    const SceneDesc &S = scenes[sc];
    const uint32_t leaves = 1u << (3u * S.depth);
    const uint32_t base = blockIdx.x * kLeafBlock;
    if (S.n == 0u || base >= leaves) continue;  // block-uniform
    // Thread t owns leaves base + 4t .. 4t+3 (a contiguous run of the Morton order).
    constexpr uint32_t kPer = kLeafBlock / kLeafThreads;
    uint32_t c[kPer], total = 0u;
    for (uint32_t k = 0; k < kPer; k++) {
      const uint32_t m = base + threadIdx.x * kPer + k;
      c[k] = m < leaves ? leaf_count(S, mom, m) : 0u;
      total += c[k];
    }
    // Exclusive scan of the thread totals across the block.
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t x = total;
    for (uint32_t off = 1u; off < 32u; off <<= 1) {
      const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, x, off);
      if (lane >= off) x += t;
    }
    if (lane == 31u) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
      uint32_t v = warp_sums[lane];
      for (uint32_t off = 1u; off < 32u; off <<= 1) {
        const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, v, off);
        if (lane >= off) v += t;
      }
      warp_sums[lane] = v;
    }
    __syncthreads();
    uint32_t run = block_offs[sc * max_blocks + blockIdx.x] + (warp ? warp_sums[warp - 1] : 0u) + x - total;
    for (uint32_t k = 0; k < kPer; k++) {
      const uint32_t m = base + threadIdx.x * kPer + k;
      if (m < leaves) starts[S.cell_off + m] = run;
      run += c[k];
    }
    __syncthreads();  // warp_sums is rewritten by the next row
  }
}

// Each CTA moves the bodies of kScatterTiles tiles at a time (every tile
// once, or the active tiles of a tile list in turn).  Slots are reserved in
// two levels so a dense leaf (tens of thousands of bodies) sees one global
// atomic per CTA instead of one per warp: warp groups of a leaf reserve their
// offsets in a shared-memory table of the CTA's leaves, then one thread per
// leaf reserves the CTA's whole block of that leaf from `starts`.
constexpr uint32_t kScatterTiles = 2u;
constexpr uint32_t kScatterSlots = 2048u;  // > bodies per CTA, so probing always ends

template <bool kList>
__global__ void __launch_bounds__(256) k_leaf_scatter(const SceneDesc *__restrict__ scenes,
                                                      const uint32_t *__restrict__ tile_scene,
                                                      const uint32_t *__restrict__ tile_list,
                                                      const Counters *__restrict__ ctr,
                                                      const float4 *__restrict__ part_in,
                                                      const uint32_t *__restrict__ ids_in,
                                                      float4 *__restrict__ part_out,
                                                      uint32_t *__restrict__ ids_out,
                                                      uint32_t *__restrict__ starts, uint32_t tiles,
                                                      unsigned long long *__restrict__ stamp) {
  __shared__ uint32_t hkey[kScatterSlots], hcnt[kScatterSlots];
  constexpr uint32_t kEmptyKey = 0xFFFFFFFFu;
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t ntiles = kList ? min(ctr->tiles_active, tiles) : tiles;
  // Without a list the grid has one unit per CTA: the loop runs once.
  for (uint32_t unit = blockIdx.x; unit * kScatterTiles < ntiles; unit += kList ? gridDim.x : ntiles) {
    for (uint32_t i = threadIdx.x; i < kScatterSlots; i += blockDim.x) {
      hkey[i] = kEmptyKey;
      hcnt[i] = 0u;
    }
    __syncthreads();
    float4 p0[kScatterTiles], p1[kScatterTiles];
    uint32_t off[kScatterTiles], hs[kScatterTiles], src[kScatterTiles];
#pragma unroll
    for (uint32_t r = 0; r < kScatterTiles; r++) {
      const uint32_t li = unit * kScatterTiles + r;
      uint32_t key = kEmptyKey;
      src[r] = kEmptyKey;
      if (li < ntiles) {
        const uint32_t tile = kList ? tile_list[li] : li;
        const SceneDesc &S = scenes[tile_scene[tile]];
        const uint32_t slot = tile * 256u + threadIdx.x;
        if (slot - S.body_off < S.n) {
          p0[r] = part_in[2u * slot];
          p1[r] = part_in[2u * slot + 1u];
          src[r] = slot;
          const uint32_t dim = 1u << S.depth;
          key = S.cell_off + (spread3s(cell_of_unit(unit_coord(p0[r].x), dim)) |
                              (spread3s(cell_of_unit(unit_coord(p0[r].y), dim)) << 1) |
                              (spread3s(cell_of_unit(unit_coord(p0[r].z), dim)) << 2));
        }
      }
      const uint32_t peers = __match_any_sync(0xFFFFFFFFu, key);
      const uint32_t leader = __ffs(peers) - 1u;
      uint32_t h = 0u, base = 0u;
      if (key != kEmptyKey && lane == leader) {
        h = (key * 2654435761u) >> 21;  // 11-bit multiplicative hash
        for (uint32_t probe = 0; probe < kScatterSlots; probe++) {
          const uint32_t prev = atomicCAS(&hkey[h], kEmptyKey, key);
          if (prev == kEmptyKey || prev == key) break;
          h = (h + 1u) & (kScatterSlots - 1u);
        }
        base = atomicAdd(&hcnt[h], __popc(peers));
      }
      hs[r] = __shfl_sync(0xFFFFFFFFu, h, leader);
      off[r] = __shfl_sync(0xFFFFFFFFu, base, leader) + __popc(peers & ((1u << lane) - 1u));
    }
    __syncthreads();
    // One global reservation per (CTA, leaf); hcnt becomes the CTA's first slot.
    for (uint32_t i = threadIdx.x; i < kScatterSlots; i += blockDim.x)
      if (hkey[i] != kEmptyKey) hcnt[i] = atomicAdd(&starts[hkey[i]], hcnt[i]);
    __syncthreads();
#pragma unroll
    for (uint32_t r = 0; r < kScatterTiles; r++) {
      if (src[r] == kEmptyKey) continue;
      const uint32_t dst = hcnt[hs[r]] + off[r];
      if (dst >= tiles * 256u) continue;  // defensive: counts and positions always agree
      part_out[2u * dst] = p0[r];
      part_out[2u * dst + 1u] = p1[r];
      ids_out[dst] = ids_in[src[r]];
    }
    if (kList) __syncthreads();  // the table is cleared for the next unit
  }
  stamp_end(stamp);  // last of the resort's four kernels
}

uint32_t leaf_sort_blocks(uint32_t max_depth) {
  return ((1u << (3u * max_depth)) + kLeafBlock - 1u) / kLeafBlock;
}

void leaf_counting_sort(const LaunchCtx &L, uint32_t scenes, uint32_t max_depth, const uint4 *counts,
                        uint32_t *block_scratch, uint32_t *starts, const float4 *part_in,
                        const uint32_t *ids_in, float4 *part_out, uint32_t *ids_out,
                        uint32_t tiles) {
  const uint32_t nb = leaf_sort_blocks(max_depth);
  // With lists (serving slots), a few rows of CTAs walk the active scenes and
  // a persistent grid the active tiles.
  const uint32_t rows = L.scene_list != nullptr ? (scenes < 32u ? scenes : 32u) : scenes;
  const uint32_t units = (tiles + kScatterTiles - 1u) / kScatterTiles;
  const uint32_t scatter = L.tile_list != nullptr ? (units < 8u * L.sms ? units : 8u * L.sms) : units;
  k_leaf_block_sums<<<dim3(nb, rows), kLeafThreads, 0, L.stream>>>(L.scenes, scenes, L.scene_list, L.ctr,
                                                                    counts, block_scratch, nb,
                                                                    stamp_rec(L, 4u));
  k_leaf_block_scan<<<rows, 32, 0, L.stream>>>(L.scenes, scenes, L.scene_list, L.ctr, block_scratch, nb);
  k_leaf_offsets<<<dim3(nb, rows), kLeafThreads, 0, L.stream>>>(L.scenes, scenes, L.scene_list, L.ctr,
                                                                 counts, block_scratch, nb, starts);
  if (L.tile_list != nullptr)
    k_leaf_scatter<true><<<scatter, 256, 0, L.stream>>>(L.scenes, L.tile_scene, L.tile_list, L.ctr, part_in,
                                                        ids_in, part_out, ids_out, starts, tiles,
                                                        stamp_rec(L, 4u));
  else
    k_leaf_scatter<false><<<scatter, 256, 0, L.stream>>>(L.scenes, L.tile_scene, nullptr, L.ctr, part_in,
                                                         ids_in, part_out, ids_out, starts, tiles,
                                                         stamp_rec(L, 4u));
}

}  // namespace rfmm
