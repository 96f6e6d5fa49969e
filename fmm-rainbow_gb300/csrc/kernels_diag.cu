// FP64 diagnostics: the direct-sum force reference on sampled targets and
// compensated energy / momentum reductions.  FP64 is used only here; the
// solver itself is binary32 throughout.  Both reductions run in a fixed order
// (per-thread sums, then blocks in index order), so they are deterministic.
#include <cuda_runtime.h>

#include "rfmm_kernels.h"

namespace rfmm {

constexpr uint32_t kDsThreads = 256u;

// Softened direct sum, FP64, sources split over blockIdx.y: partial[s][t][3].
// `part` holds the scene in the caller's order (2 float4 per body).
__global__ void __launch_bounds__(kDsThreads) k_direct_f64(const float4 *__restrict__ part, uint32_t n,
                                                           const uint32_t *__restrict__ targets,
                                                           uint32_t nt, double eps2,
                                                           uint32_t split_len,
                                                           double *__restrict__ partial) {
  __shared__ double sx[kDsThreads], sy[kDsThreads], sz[kDsThreads];
  const uint32_t t = blockIdx.x * kDsThreads + threadIdx.x;
  const uint32_t split = blockIdx.y;
  const uint32_t j0 = split * split_len;
  const uint32_t j1 = min(n, j0 + split_len);
  uint32_t ti = 0xFFFFFFFFu;
  double px = 0.0, py = 0.0, pz = 0.0;
  if (t < nt) {
    ti = targets[t];
    const float4 p = part[2u * ti];
    px = p.x;
    py = p.y;
    pz = p.z;
  }
  double ax = 0.0, ay = 0.0, az = 0.0;
  for (uint32_t base = j0; base < j1; base += kDsThreads) {
    const uint32_t j = base + threadIdx.x;
    if (j < j1) {
      const float4 q = part[2u * j];
      sx[threadIdx.x] = q.x;
      sy[threadIdx.x] = q.y;
      sz[threadIdx.x] = q.z;
    }
    __syncthreads();
    const uint32_t m = min(kDsThreads, j1 - base);
    if (t < nt) {
      for (uint32_t k = 0; k < m; k++) {
        if (base + k == ti) continue;
        const double dx = sx[k] - px, dy = sy[k] - py, dz = sz[k] - pz;
        const double r2 = dx * dx + dy * dy + dz * dz + eps2;
        const double inv = 1.0 / sqrt(r2);
        const double w = inv * inv * inv;
        ax += dx * w;
        ay += dy * w;
        az += dz * w;
      }
    }
    __syncthreads();
  }
  if (t < nt) {
    double *o = partial + ((size_t)split * nt + t) * 3u;
    o[0] = ax;
    o[1] = ay;
    o[2] = az;
  }
}

__global__ void k_direct_reduce(const double *__restrict__ partial, uint32_t splits, uint32_t nt,
                                double gm, double *__restrict__ out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 3u * nt) return;
  double acc = 0.0;
  for (uint32_t s = 0; s < splits; s++) acc += partial[(size_t)s * nt * 3u + i];
  out[i] = gm * acc;
}

void launch_direct_sum_f64(cudaStream_t stream, const float4 *part_caller, uint32_t n,
                           const uint32_t *targets, uint32_t nt, double gravity, double eps,
                           double *partial, uint32_t splits, double *out) {
  const uint32_t split_len = (n + splits - 1u) / splits;
  dim3 grid((nt + kDsThreads - 1u) / kDsThreads, splits);
  k_direct_f64<<<grid, kDsThreads, 0, stream>>>(part_caller, n, targets, nt, eps * eps, split_len,
                                                partial);
  k_direct_reduce<<<(3u * nt + 255u) / 256u, 256, 0, stream>>>(partial, splits, nt,
                                                               gravity / (double)n, out);
}

// Neumaier-compensated running sum.
struct Comp {
  double s = 0.0, c = 0.0;
  __device__ void add(double x) {
    const double t = s + x;
    if (fabs(s) >= fabs(x)) {
      c += (s - t) + x;
    } else {
      c += (x - t) + s;
    }
    s = t;
  }
  __device__ double value() const { return s + c; }
};

// Per body (caller order): mass 1/n, kinetic 1/2 m v^2, potential 1/2 m phi,
// momentum m v, angular momentum m x cross v.  partial[block][9].
__global__ void __launch_bounds__(256) k_diag_partials(const float4 *__restrict__ part,
                                                       const float4 *__restrict__ accphi, uint32_t n,
                                                       double *__restrict__ partial) {
  __shared__ double red[256][9];
  Comp acc[9];
  const double m = 1.0 / (double)n;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float4 p = part[2u * i], v = part[2u * i + 1u];
    const float4 a = accphi[i];
    const double vx = v.x, vy = v.y, vz = v.z, x = p.x, y = p.y, z = p.z;
    acc[0].add(0.5 * m * (vx * vx + vy * vy + vz * vz));
    acc[1].add(0.5 * m * (double)a.w);
    acc[2].add(m * vx);
    acc[3].add(m * vy);
    acc[4].add(m * vz);
    acc[5].add(m * (y * vz - z * vy));
    acc[6].add(m * (z * vx - x * vz));
    acc[7].add(m * (x * vy - y * vx));
    acc[8].add(1.0);
  }
  for (int k = 0; k < 9; k++) red[threadIdx.x][k] = acc[k].value();
  __syncthreads();
  if (threadIdx.x < 9u) {
    Comp c;
    for (uint32_t t = 0; t < blockDim.x; t++) c.add(red[t][threadIdx.x]);
    partial[blockIdx.x * 9u + threadIdx.x] = c.value();
  }
}

__global__ void k_diag_final(const double *__restrict__ partial, uint32_t blocks,
                             double *__restrict__ out) {
  if (threadIdx.x >= 9u) return;
  Comp c;
  for (uint32_t b = 0; b < blocks; b++) c.add(partial[b * 9u + threadIdx.x]);
  out[threadIdx.x] = c.value();
}

void launch_diagnostics(cudaStream_t stream, const float4 *part_caller, const float4 *accphi,
                        uint32_t n, double *partial, uint32_t blocks, double *out) {
  k_diag_partials<<<blocks, 256, 0, stream>>>(part_caller, accphi, n, partial);
  k_diag_final<<<1, 32, 0, stream>>>(partial, blocks, out);
}

}  // namespace rfmm
