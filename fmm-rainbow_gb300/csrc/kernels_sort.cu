// Stable LSD radix sort of (key, value) pairs with 8-bit digits.
//
// It orders bodies by (scene, Morton leaf key) so each leaf's bodies are
// contiguous: leaf membership and occupancy then come from runs of equal
// keys, and the deposit is a segmented reduction over those runs.  The sort
// is stable, so the resident order is a deterministic function of the input.
//
// Per 8-bit pass:
//   k_sort_hist     per 4096-key tile, digit histogram in shared memory
//   k_sort_scan     one CTA per digit: exclusive scan of that digit's tile
//                   counts (digit-major layout), plus the digit total
//   k_sort_scatter  per tile: digit base + tile offset + stable rank inside
//                   the tile (warp __match_any_sync ranks, warp prefix in
//                   shared memory), then scatter
#include <cuda_runtime.h>

#include "rfmm_kernels.h"

namespace rfmm {

constexpr uint32_t kSortThreads = 256u;
constexpr uint32_t kSortItems = 16u;
constexpr uint32_t kSortTile = kSortThreads * kSortItems;  // 4096 keys

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

}  // namespace rfmm
