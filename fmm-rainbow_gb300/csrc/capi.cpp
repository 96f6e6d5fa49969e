// C ABI of the plain single-scene solver (include/rfmm.h).
//
// Each entry point replaces a piece of the reference host's dispatch
// sequence: rfmm_create ~ rebuildSimulation buffer setup (app.js:525-607,
// native/main.rs:290-316), rfmm_seed_galaxy ~ the `initialize` pass
// (native/main.rs:423-434), rfmm_solve_fields ~ the digest solve
// (native/main.rs:436-449), rfmm_step ~ encode_frame (native/main.rs:411-421),
// rfmm_digest ~ digest() (native/main.rs:152-163), rfmm_phase_times ~ the
// timestamp-query frame (native/main.rs:466-520), rfmm_check_finite ~ the
// finiteness scan (native/main.rs:536-549).
#include <cmath>
#include <new>
#include <vector>

#include "engine.h"
#include "rfmm.h"

struct rfmm_handle {
  rfmm::Engine *engine;
  rfmm_params params;
};

namespace {

int guard(const rfmm_handle *h) { return (h == nullptr || h->engine == nullptr) ? RFMM_ERR_INVALID : RFMM_OK; }

}  // namespace

extern "C" {

void rfmm_default_params(rfmm_params *p) {
  if (p == nullptr) return;
  *p = rfmm_params{};
  p->dt = 0.0009f;
  p->gravity = 0.34f;
  p->softening = 0.012f;
  p->speed = 1.0f;
  p->control_strength = 0.7f;
  p->control_radius = 0.22f;
}

const char *rfmm_status_string(int status) { return rfmm::status_string(status); }

int rfmm_create(uint32_t n, const rfmm_params *params, rfmm_handle **out) {
  if (out == nullptr) return RFMM_ERR_INVALID;
  *out = nullptr;
  rfmm::SceneSpec spec;
  spec.n = n;
  if (params != nullptr) {
    spec.params = *params;
  } else {
    rfmm_default_params(&spec.params);
  }
  rfmm::Engine *e = nullptr;
  const int st = rfmm::Engine::create({spec}, &e);
  if (st != RFMM_OK) return st;
  rfmm_handle *h = new (std::nothrow) rfmm_handle{e, spec.params};
  if (h == nullptr) {
    delete e;
    return RFMM_ERR_OOM;
  }
  *out = h;
  return RFMM_OK;
}

int rfmm_destroy(rfmm_handle *h) {
  if (h == nullptr) return RFMM_ERR_INVALID;
  delete h->engine;
  delete h;
  return RFMM_OK;
}

int rfmm_set_stream(rfmm_handle *h, void *stream) {
  if (guard(h)) return RFMM_ERR_INVALID;
  return h->engine->set_stream(static_cast<cudaStream_t>(stream));
}

int rfmm_get_plan(const rfmm_handle *h, rfmm_plan *out) {
  if (guard(h) || out == nullptr) return RFMM_ERR_INVALID;
  const rfmm::SceneDesc &d = h->engine->scene(0);
  out->particles = d.n;
  out->depth = d.depth;
  out->cells = d.cells;
  out->fixed_point_scale = d.scale;
  return RFMM_OK;
}

int rfmm_set_params(rfmm_handle *h, const rfmm_params *params) {
  if (guard(h) || params == nullptr) return RFMM_ERR_INVALID;
  const int st = h->engine->set_params(0, *params);
  if (st == RFMM_OK) h->params = *params;
  return st;
}

int rfmm_upload_particles(rfmm_handle *h, const void *host_aos, size_t bytes) {
  if (guard(h)) return RFMM_ERR_INVALID;
  int st = h->engine->upload(0, host_aos, bytes, cudaMemcpyHostToDevice);
  if (st == RFMM_OK) st = h->engine->commit();
  return st;
}

int rfmm_upload_particles_device(rfmm_handle *h, const void *device_aos, size_t bytes) {
  if (guard(h)) return RFMM_ERR_INVALID;
  int st = h->engine->upload(0, device_aos, bytes, cudaMemcpyDeviceToDevice);
  if (st == RFMM_OK) st = h->engine->commit();
  return st;
}

int rfmm_seed_galaxy(rfmm_handle *h) {
  if (guard(h)) return RFMM_ERR_INVALID;
  int st = h->engine->seed_galaxy(0);
  if (st == RFMM_OK) st = h->engine->commit();
  return st;
}

int rfmm_solve_fields(rfmm_handle *h) {
  if (guard(h)) return RFMM_ERR_INVALID;
  return h->engine->solve_fields();
}

int rfmm_step(rfmm_handle *h, uint32_t steps) {
  if (guard(h)) return RFMM_ERR_INVALID;
  return h->engine->step(steps);
}

int rfmm_sync(rfmm_handle *h) {
  if (guard(h)) return RFMM_ERR_INVALID;
  return h->engine->sync();
}

int rfmm_download(rfmm_handle *h, int which, void *host_dst, size_t bytes) {
  if (guard(h)) return RFMM_ERR_INVALID;
  return h->engine->download(0, which, host_dst, bytes, cudaMemcpyDeviceToHost);
}

int rfmm_download_device(rfmm_handle *h, int which, void *device_dst, size_t bytes) {
  if (guard(h)) return RFMM_ERR_INVALID;
  return h->engine->download(0, which, device_dst, bytes, cudaMemcpyDeviceToDevice);
}

int rfmm_digest(rfmm_handle *h, int which, uint32_t *out) {
  if (guard(h)) return RFMM_ERR_INVALID;
  return h->engine->digest(0, which, out);
}

int rfmm_phase_times(rfmm_handle *h, float ms[7]) {
  if (guard(h)) return RFMM_ERR_INVALID;
  return h->engine->phase_times(ms);
}

int rfmm_check_finite(rfmm_handle *h, uint32_t probe, uint32_t *non_finite, float *max_abs) {
  if (guard(h) || non_finite == nullptr || max_abs == nullptr) return RFMM_ERR_INVALID;
  const rfmm::SceneDesc &d = h->engine->scene(0);
  std::vector<float> all((size_t)d.n * 8u);
  const int st = h->engine->download(0, RFMM_BUF_PARTICLES, all.data(), all.size() * 4u,
                                     cudaMemcpyDeviceToHost);
  if (st != RFMM_OK) return st;
  const size_t count = (size_t)(probe < d.n ? probe : d.n) * 8u;
  uint32_t bad = 0;
  float mx = 0.0f;
  for (size_t i = 0; i < count; i++) {
    const float f = all[i];
    if (std::isfinite(f)) {
      mx = std::fmax(mx, std::fabs(f));
    } else {
      bad++;
    }
  }
  *non_finite = bad;
  *max_abs = mx;
  return RFMM_OK;
}

int rfmm_set_resort_interval(rfmm_handle *h, uint32_t steps) {
  if (guard(h)) return RFMM_ERR_INVALID;
  return h->engine->set_resort_interval(steps);
}

int rfmm_set_near_mode(rfmm_handle *h, uint32_t mode) {
  if (guard(h)) return RFMM_ERR_INVALID;
  return h->engine->set_near_mode(mode);
}

int rfmm_set_float_mode(rfmm_handle *h, uint32_t mode) {
  if (guard(h)) return RFMM_ERR_INVALID;
  return h->engine->set_float_mode(mode);
}

int rfmm_check_wait_timeout(rfmm_handle *h, uint32_t polls) {
  if (guard(h)) return RFMM_ERR_INVALID;
  return h->engine->check_wait_timeout(polls);
}

int rfmm_device_error(rfmm_handle *h, uint32_t *code, uint32_t *info) {
  if (guard(h)) return RFMM_ERR_INVALID;
  return h->engine->device_error(code, info);
}

int rfmm_profile_steps(rfmm_handle *h, uint32_t steps, float *kernel_ms, uint32_t *launches) {
  if (guard(h) || kernel_ms == nullptr || launches == nullptr) return RFMM_ERR_INVALID;
  return h->engine->profile_steps(steps, kernel_ms, launches);
}

int rfmm_launch_count(rfmm_handle *h, uint64_t *out) {
  if (guard(h) || out == nullptr) return RFMM_ERR_INVALID;
  *out = h->engine->launch_count();
  return RFMM_OK;
}

int rfmm_set_timeline(rfmm_handle *h, uint32_t enable) {
  if (guard(h) || enable > 1u) return RFMM_ERR_INVALID;
  return h->engine->set_timeline(enable != 0u);
}

int rfmm_get_timeline(rfmm_handle *h, rfmm_timeline *out) {
  if (guard(h) || out == nullptr) return RFMM_ERR_INVALID;
  return h->engine->get_timeline(out);
}

int rfmm_accelerations(rfmm_handle *h, float *host_out, size_t bytes) {
  if (guard(h) || bytes != 16ull * h->engine->scene(0).n) return RFMM_ERR_INVALID;
  return h->engine->accelerations(0, host_out);
}

int rfmm_force_error(rfmm_handle *h, uint32_t targets, uint64_t seed, double *rms_rel,
                     double *max_rel) {
  if (guard(h)) return RFMM_ERR_INVALID;
  return h->engine->force_error(0, targets, seed, rms_rel, max_rel);
}

int rfmm_get_diagnostics(rfmm_handle *h, rfmm_diagnostics *out) {
  if (guard(h) || out == nullptr) return RFMM_ERR_INVALID;
  double v[9];
  const int st = h->engine->diagnostics(0, v);
  if (st != RFMM_OK) return st;
  out->kinetic = v[0];
  out->potential = v[1];
  out->total = v[0] + v[1];
  for (int k = 0; k < 3; k++) {
    out->momentum[k] = v[2 + k];
    out->angular_momentum[k] = v[5 + k];
  }
  return RFMM_OK;
}

void rfmm_default_render_params(rfmm_render_params *out) {
  if (out == nullptr) return;
  out->width = 1280u;
  out->height = 720u;
  out->instances = 0u;
  out->yaw = -0.18f;  // app.js:75-77
  out->pitch = -0.14f;
  out->zoom = 1.78f;
  out->point_size = 5.0f;  // index.html "gradient radius" default
  out->exposure = 1.0f;
}

int rfmm_render(rfmm_handle *h, const rfmm_render_params *params, void *host_rgba, size_t bytes) {
  if (guard(h) || params == nullptr) return RFMM_ERR_INVALID;
  return h->engine->render(0, *params, host_rgba, bytes, cudaMemcpyDeviceToHost);
}

int rfmm_render_device(rfmm_handle *h, const rfmm_render_params *params, void *device_rgba,
                       size_t bytes) {
  if (guard(h) || params == nullptr) return RFMM_ERR_INVALID;
  return h->engine->render(0, *params, device_rgba, bytes, cudaMemcpyDeviceToDevice);
}

int rfmm_get_tuning(rfmm_handle *h, rfmm_tuning *out) {
  if (guard(h)) return RFMM_ERR_INVALID;
  return h->engine->get_tuning(out);
}

int rfmm_set_tuning(rfmm_handle *h, const rfmm_tuning *tuning) {
  if (guard(h) || tuning == nullptr) return RFMM_ERR_INVALID;
  return h->engine->set_tuning(*tuning);
}

int rfmm_autotune(rfmm_handle *h, uint32_t steps_per_trial, rfmm_tuning *best) {
  if (guard(h)) return RFMM_ERR_INVALID;
  return h->engine->autotune(steps_per_trial, best);
}

}  // extern "C"
