// Headless point-splat renderer: the reference's display passes restated as
// CUDA kernels writing an RGBA8 image into device memory (no window, no
// swapchain, no graphics API).
//
// Reference (iskamag/fmm-rainbow):
//   render_vertex / render_fragment   src/rainbow_fmm.wgsl:780-900
//   reconstruct_field + blur passes   src/rainbow_fmm.wgsl:914-970
//   resolve_fragment                  src/rainbow_fmm.wgsl:972-1009
//   pass sequence, texture sizes      app.js:650-710, 216-251 (accumulation at
//                                     half the canvas size, linear clamp sampler)
//
// Differences by design: the additive rgba16float blend becomes a per-pixel
// fixed-point sum (64-bit integer atomics at 2^24 per unit), which is exact
// and independent of the order points arrive in; the blur and resolve
// intermediates are binary32 instead of binary16; bilinear taps use the exact
// fractional position.
#include <cuda_runtime.h>

#include "rfmm_device.cuh"
#include "rfmm_kernels.h"
#include "rfmm_math.h"

namespace rfmm {

namespace {

constexpr float kTau = 6.28318530718f;
constexpr float kFix = 16777216.0f;        // 2^24 fixed-point units per 1.0
constexpr float kFixInv = 1.0f / 16777216.0f;

__device__ __forceinline__ float mixf(float a, float b, float t) { return a * (1.0f - t) + b * t; }

__device__ __forceinline__ float smoothstepf_d(float lo, float hi, float x) {
  const float t = clampf_d((x - lo) / (hi - lo), 0.0f, 1.0f);
  return t * t * (3.0f - 2.0f * t);
}

__device__ __forceinline__ float len3(float x, float y, float z) { return sqrtf((x * x + y * y) + z * z); }

// Fixed-point accumulation texture -> float4 (r, g, b, a).
__device__ __forceinline__ float4 fetch_accum(const unsigned long long *acc, uint32_t w, uint32_t h,
                                              int x, int y) {
  x = min(max(x, 0), (int)w - 1);
  y = min(max(y, 0), (int)h - 1);
  const unsigned long long *p = acc + 4ull * ((size_t)y * w + (size_t)x);
  return make_float4((float)p[0] * kFixInv, (float)p[1] * kFixInv, (float)p[2] * kFixInv,
                     (float)p[3] * kFixInv);
}

__device__ __forceinline__ float4 fetch_tex(const float4 *tex, uint32_t w, uint32_t h, int x, int y) {
  x = min(max(x, 0), (int)w - 1);
  y = min(max(y, 0), (int)h - 1);
  return tex[(size_t)y * w + (size_t)x];
}

__device__ __forceinline__ float4 lerp4(float4 a, float4 b, float f) {
  return make_float4(a.x * (1.0f - f) + b.x * f, a.y * (1.0f - f) + b.y * f,
                     a.z * (1.0f - f) + b.z * f, a.w * (1.0f - f) + b.w * f);
}

__device__ __forceinline__ float4 add4(float4 a, float4 b) {
  return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w);
}

__device__ __forceinline__ float4 scale4(float4 a, float s) {
  return make_float4(a.x * s, a.y * s, a.z * s, a.w * s);
}

}  // namespace

// render_vertex + render_fragment for every drawn instance: the instance's
// body (a fixed hash of the instance index, wgsl:806-808), its camera-space
// position and colour, and the additive splat into the pixel its point
// covers.  `slot_of` maps the caller's body index to its resident slot.
__global__ void __launch_bounds__(256) k_splat(const SceneDesc *__restrict__ scenes, uint32_t scene,
                                               const float4 *__restrict__ part,
                                               const uint32_t *__restrict__ slot_of,
                                               RenderCamera cam, unsigned long long *__restrict__ acc) {
  const SceneDesc &S = scenes[scene];
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= cam.instances || S.n == 0u) return;
  const uint32_t body = (i * 747796405u + 2891336453u) % S.n;
  const uint32_t slot = slot_of[S.body_off + body];
  const float4 pl = part[2u * slot], vh = part[2u * slot + 1u];

  // rotate_camera (wgsl:785-798); the four trigonometric values come in.
  const float yx = cam.cos_yaw * pl.x + cam.sin_yaw * pl.z;
  const float yy = pl.y;
  const float yz = -cam.sin_yaw * pl.x + cam.cos_yaw * pl.z;
  const float rx = yx, ry = cam.cos_pitch * yy - cam.sin_pitch * yz,
              rz = cam.sin_pitch * yy + cam.cos_pitch * yz;
  const float view_z = cam.zoom * kHalf - rz;
  const float perspective = (1.92f * kHalf) / view_z;
  const float cx = rx * perspective / cam.aspect, cy = ry * perspective;
  const float depth = 0.46f + rz * 0.08f;

  const float velocity = len3(vh.x, vh.y, vh.z);
  const float speed = fmaxf(velocity, 0.0001f);
  const float excitation = clampf_d(vh.w, 0.0f, 1.0f);
  const float signed_radial =
      clampf_d(((pl.x * vh.x + pl.y * vh.y) + pl.z * vh.z) / (fmaxf(len3(pl.x, pl.y, pl.z), 0.0001f) * speed),
               -1.0f, 1.0f);
  const float infall = clampf_d(-signed_radial, 0.0f, 1.0f);
  const float outflow = clampf_d(signed_radial, 0.0f, 1.0f);
  float sp[3] = {mixf(0.50f, 0.24f, infall), mixf(0.42f, 0.56f, infall), mixf(0.58f, 1.00f, infall)};
  sp[0] = mixf(sp[0], 1.00f, outflow);
  sp[1] = mixf(sp[1], 0.50f, outflow);
  sp[2] = mixf(sp[2], 0.20f, outflow);
  const float heat = smoothstepf_d(0.18f, 0.85f, excitation);
  const float phase[3] = {0.00f, 0.67f, 0.33f};
  float col[3];
  const float luminosity = 0.30f + excitation * 0.90f;
  const float speed_gain = 0.62f + fminf(velocity * 1.4f, 1.0f) * 0.30f;
  for (int k = 0; k < 3; k++) {
    const float rainbow = 0.5f + 0.5f * rf_cosf(kTau * (pl.w + phase[k]));
    const float tint = rf_powf(rainbow, 0.85f);
    const float s = mixf(sp[k] * tint, sp[k], heat);
    col[k] = s * (speed_gain + excitation * 0.90f) + heat * heat * 0.55f;
  }
  float influence = 0.0f;
  float cc[3] = {0.82f, 1.0f, 0.28f};
  if (S.control_point[3] > 0.5f) {
    const float dx = S.control_point[0] - pl.x, dy = S.control_point[1] - pl.y,
                dz = S.control_point[2] - pl.z;
    const float radius = fmaxf(S.control_radius, 0.02f);
    influence = rf_expf(-2.0f * ((dx * dx + dy * dy) + dz * dz) / (radius * radius));
    const float mode = S.control_axis_mode[3];
    if (mode > 1.5f && mode < 2.5f) {
      cc[0] = 1.0f; cc[1] = 0.38f; cc[2] = 0.18f;
    } else if (mode >= 2.5f) {
      cc[0] = 0.82f; cc[1] = 0.34f; cc[2] = 1.0f;
    }
  }
  for (int k = 0; k < 3; k++) col[k] = mixf(col[k], cc[k], influence * 0.68f);
  const float depth_fade = clampf_d(0.62f + rz * 0.25f, 0.28f, 1.0f) * (0.76f + excitation * 0.48f) *
                           luminosity * (1.0f + influence * 0.72f);

  // Clip volume (x, y in [-1, 1], z in [0, 1]) and the 1-pixel point's pixel.
  if (!(cx >= -1.0f && cx <= 1.0f && cy >= -1.0f && cy <= 1.0f && depth >= 0.0f && depth <= 1.0f))
    return;
  const float fx = (cx + 1.0f) * 0.5f * (float)cam.acc_w;
  const float fy = (1.0f - cy) * 0.5f * (float)cam.acc_h;
  const int px = min((int)floorf(fx), (int)cam.acc_w - 1), py = min((int)floorf(fy), (int)cam.acc_h - 1);
  const float weight = cam.exposure * depth_fade * cam.population_scale;
  unsigned long long *dst = acc + 4ull * ((size_t)py * cam.acc_w + (size_t)px);
  atomicAdd(dst + 0, __float2ull_rn(col[0] * weight * kFix));
  atomicAdd(dst + 1, __float2ull_rn(col[1] * weight * kFix));
  atomicAdd(dst + 2, __float2ull_rn(col[2] * weight * kFix));
  atomicAdd(dst + 3, __float2ull_rn(weight * kFix));
}

// One separable pass of reconstruct_field (wgsl:914-945): five bilinear taps
// along `axis` at +-1.384615 and +-3.230769 steps, step = point_size /
// (canvas size * 3.230769) in texture coordinates.  The first pass reads the
// fixed-point accumulation, the second the first pass's output.
template <bool kFromAccum>
__global__ void __launch_bounds__(256) k_blur(const unsigned long long *__restrict__ acc,
                                              const float4 *__restrict__ src, RenderCamera cam,
                                              int axis, float4 *__restrict__ dst) {
  const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  if (x >= cam.acc_w || y >= cam.acc_h) return;
  const uint32_t w = cam.acc_w, h = cam.acc_h;
  const float dim = axis == 0 ? (float)w : (float)h;
  const float out_dim = axis == 0 ? cam.canvas_w : cam.canvas_h;
  const float step = fmaxf(cam.point_size, 1.0f) / (out_dim * 3.230769f);
  const float uv = ((axis == 0 ? (float)x : (float)y) + 0.5f) / dim;
  auto tap = [&](float u) -> float4 {
    const float t = u * dim - 0.5f;
    const float f0 = floorf(t);
    const float f = t - f0;
    const int i0 = (int)f0;
    float4 a, b;
    if (axis == 0) {
      a = kFromAccum ? fetch_accum(acc, w, h, i0, (int)y) : fetch_tex(src, w, h, i0, (int)y);
      b = kFromAccum ? fetch_accum(acc, w, h, i0 + 1, (int)y) : fetch_tex(src, w, h, i0 + 1, (int)y);
    } else {
      a = kFromAccum ? fetch_accum(acc, w, h, (int)x, i0) : fetch_tex(src, w, h, (int)x, i0);
      b = kFromAccum ? fetch_accum(acc, w, h, (int)x, i0 + 1) : fetch_tex(src, w, h, (int)x, i0 + 1);
    }
    return lerp4(a, b, f);
  };
  float4 field = scale4(tap(uv), 0.227027f);
  field = add4(field, scale4(tap(uv + step * 1.384615f), 0.316216f));
  field = add4(field, scale4(tap(uv - step * 1.384615f), 0.316216f));
  field = add4(field, scale4(tap(uv + step * 3.230769f), 0.070270f));
  field = add4(field, scale4(tap(uv - step * 3.230769f), 0.070270f));
  dst[(size_t)y * w + x] = field;
}

// resolve_fragment (wgsl:972-1009) for every canvas pixel: bilinear sample of
// the blurred field, density-normalised colour, filmic curve, gamma 0.82,
// written as RGBA8 (row 0 = top of the canvas).
__global__ void __launch_bounds__(256) k_resolve(const float4 *__restrict__ tex, RenderCamera cam,
                                                 uchar4 *__restrict__ out) {
  const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  const uint32_t W = (uint32_t)cam.canvas_w, H = (uint32_t)cam.canvas_h;
  if (x >= W || y >= H) return;
  const uint32_t w = cam.acc_w, h = cam.acc_h;
  const float u = ((float)x + 0.5f) / cam.canvas_w, v = ((float)y + 0.5f) / cam.canvas_h;
  const float tx = u * (float)w - 0.5f, ty = v * (float)h - 0.5f;
  const float fx0 = floorf(tx), fy0 = floorf(ty);
  const float fx = tx - fx0, fy = ty - fy0;
  const int ix = (int)fx0, iy = (int)fy0;
  const float4 top = lerp4(fetch_tex(tex, w, h, ix, iy), fetch_tex(tex, w, h, ix + 1, iy), fx);
  const float4 bot = lerp4(fetch_tex(tex, w, h, ix, iy + 1), fetch_tex(tex, w, h, ix + 1, iy + 1), fx);
  const float4 a = lerp4(top, bot, fy);
  const float bg[3] = {0.006f, 0.008f, 0.015f};
  float rgb[3] = {bg[0], bg[1], bg[2]};
  if (!(a.w < 0.00001f)) {
    const float avg[3] = {a.x / a.w, a.y / a.w, a.z / a.w};
    const float luma = (avg[0] * 0.2126f + avg[1] * 0.7152f) + avg[2] * 0.0722f;
    const float density = sqrtf(a.w / (a.w + 1.0f));
    for (int k = 0; k < 3; k++) {
      const float vivid = fmaxf(0.0f, mixf(luma, avg[k], 1.16f));
      const float mapped = 1.0f - rf_expf(-vivid * density * 1.58f);
      rgb[k] = rf_powf(clampf_d(mapped + bg[k], 0.0f, 1.0f), 0.82f);
    }
  }
  out[(size_t)y * W + x] = make_uchar4((unsigned char)__float2int_rn(rgb[0] * 255.0f),
                                       (unsigned char)__float2int_rn(rgb[1] * 255.0f),
                                       (unsigned char)__float2int_rn(rgb[2] * 255.0f), 255);
}

void launch_render(const LaunchCtx &L, uint32_t scene, const uint32_t *slot_of, const RenderCamera &cam,
                   unsigned long long *acc, float4 *tex_a, float4 *tex_b, uchar4 *out) {
  cudaMemsetAsync(acc, 0, 32ull * cam.acc_w * cam.acc_h, L.stream);
  k_splat<<<(cam.instances + 255u) / 256u, 256, 0, L.stream>>>(L.scenes, scene, L.part, slot_of, cam, acc);
  const dim3 grid_a((cam.acc_w + 255u) / 256u, cam.acc_h);
  k_blur<true><<<grid_a, 256, 0, L.stream>>>(acc, nullptr, cam, 0, tex_a);
  k_blur<false><<<grid_a, 256, 0, L.stream>>>(nullptr, tex_a, cam, 1, tex_b);
  const dim3 grid_c(((uint32_t)cam.canvas_w + 255u) / 256u, (uint32_t)cam.canvas_h);
  k_resolve<<<grid_c, 256, 0, L.stream>>>(tex_b, cam, out);
}

}  // namespace rfmm
