// C ABI of the batched form (include/rfmm.h, rfmm_batch_*): one engine over
// many scenes, so each step's kernels cover every scene in one launch.
#include <new>
#include <vector>

#include "engine.h"
#include "rfmm.h"

struct rfmm_batch {
  rfmm::Engine *engine;
};

namespace {

bool bad(const rfmm_batch *b) { return b == nullptr || b->engine == nullptr; }

bool bad_scene(const rfmm_batch *b, uint32_t scene) {
  return bad(b) || scene >= b->engine->num_scenes();
}

}  // namespace

extern "C" {

int rfmm_batch_create(uint32_t scenes, const uint32_t *bodies_per_scene, const rfmm_params *params,
                      rfmm_batch **out) {
  if (out == nullptr || scenes == 0u || bodies_per_scene == nullptr) return RFMM_ERR_INVALID;
  *out = nullptr;
  std::vector<rfmm::SceneSpec> specs(scenes);
  for (uint32_t i = 0; i < scenes; i++) {
    specs[i].n = bodies_per_scene[i];
    if (params != nullptr) {
      specs[i].params = params[i];
    } else {
      rfmm_default_params(&specs[i].params);
    }
  }
  rfmm::Engine *e = nullptr;
  const int st = rfmm::Engine::create(specs, &e);
  if (st != RFMM_OK) return st;
  rfmm_batch *b = new (std::nothrow) rfmm_batch{e};
  if (b == nullptr) {
    delete e;
    return RFMM_ERR_OOM;
  }
  *out = b;
  return RFMM_OK;
}

int rfmm_batch_destroy(rfmm_batch *b) {
  if (b == nullptr) return RFMM_ERR_INVALID;
  delete b->engine;
  delete b;
  return RFMM_OK;
}

int rfmm_batch_set_stream(rfmm_batch *b, void *stream) {
  if (bad(b)) return RFMM_ERR_INVALID;
  return b->engine->set_stream(static_cast<cudaStream_t>(stream));
}

int rfmm_batch_get_plan(const rfmm_batch *b, uint32_t scene, rfmm_plan *out) {
  if (bad_scene(b, scene) || out == nullptr) return RFMM_ERR_INVALID;
  const rfmm::SceneDesc &d = b->engine->scene(scene);
  out->particles = d.n;
  out->depth = d.depth;
  out->cells = d.cells;
  out->fixed_point_scale = d.scale;
  return RFMM_OK;
}

int rfmm_batch_set_params(rfmm_batch *b, uint32_t scene, const rfmm_params *params) {
  if (bad_scene(b, scene) || params == nullptr) return RFMM_ERR_INVALID;
  return b->engine->set_params(scene, *params);
}

int rfmm_batch_upload(rfmm_batch *b, uint32_t scene, const void *host_aos, size_t bytes) {
  if (bad_scene(b, scene)) return RFMM_ERR_INVALID;
  return b->engine->upload(scene, host_aos, bytes, cudaMemcpyHostToDevice);
}

int rfmm_batch_upload_device(rfmm_batch *b, uint32_t scene, const void *device_aos, size_t bytes) {
  if (bad_scene(b, scene)) return RFMM_ERR_INVALID;
  return b->engine->upload(scene, device_aos, bytes, cudaMemcpyDeviceToDevice);
}

int rfmm_batch_upload_device_all(rfmm_batch *b, const void *const *device_aos) {
  if (bad(b)) return RFMM_ERR_INVALID;
  return b->engine->upload_all_device(device_aos);
}

int rfmm_batch_seed_galaxy(rfmm_batch *b, uint32_t scene) {
  if (bad_scene(b, scene)) return RFMM_ERR_INVALID;
  return b->engine->seed_galaxy(scene);
}

int rfmm_batch_commit(rfmm_batch *b) {
  if (bad(b)) return RFMM_ERR_INVALID;
  return b->engine->commit();
}

int rfmm_batch_solve_fields(rfmm_batch *b) {
  if (bad(b)) return RFMM_ERR_INVALID;
  return b->engine->solve_fields();
}

int rfmm_batch_step(rfmm_batch *b, uint32_t steps) {
  if (bad(b)) return RFMM_ERR_INVALID;
  return b->engine->step(steps);
}

int rfmm_batch_sync(rfmm_batch *b) {
  if (bad(b)) return RFMM_ERR_INVALID;
  return b->engine->sync();
}

int rfmm_batch_download(rfmm_batch *b, uint32_t scene, int which, void *host_dst, size_t bytes) {
  if (bad_scene(b, scene)) return RFMM_ERR_INVALID;
  return b->engine->download(scene, which, host_dst, bytes, cudaMemcpyDeviceToHost);
}

int rfmm_batch_download_all(rfmm_batch *b, int which, void *const *host_dst) {
  if (bad(b)) return RFMM_ERR_INVALID;
  return b->engine->download_all(which, host_dst, cudaMemcpyDeviceToHost);
}

int rfmm_batch_download_device(rfmm_batch *b, uint32_t scene, int which, void *device_dst,
                               size_t bytes) {
  if (bad_scene(b, scene)) return RFMM_ERR_INVALID;
  return b->engine->download(scene, which, device_dst, bytes, cudaMemcpyDeviceToDevice);
}

int rfmm_batch_digest(rfmm_batch *b, uint32_t scene, int which, uint32_t *out) {
  if (bad_scene(b, scene)) return RFMM_ERR_INVALID;
  return b->engine->digest(scene, which, out);
}

int rfmm_batch_launch_count(rfmm_batch *b, uint64_t *out) {
  if (bad(b) || out == nullptr) return RFMM_ERR_INVALID;
  *out = b->engine->launch_count();
  return RFMM_OK;
}

int rfmm_batch_profile_steps(rfmm_batch *b, uint32_t steps, float *kernel_ms, uint32_t *launches) {
  if (bad(b) || kernel_ms == nullptr || launches == nullptr) return RFMM_ERR_INVALID;
  return b->engine->profile_steps(steps, kernel_ms, launches);
}

int rfmm_batch_set_timeline(rfmm_batch *b, uint32_t enable) {
  if (bad(b) || enable > 1u) return RFMM_ERR_INVALID;
  return b->engine->set_timeline(enable != 0u);
}

int rfmm_batch_get_timeline(rfmm_batch *b, rfmm_timeline *out) {
  if (bad(b) || out == nullptr) return RFMM_ERR_INVALID;
  return b->engine->get_timeline(out);
}

int rfmm_batch_set_float_mode(rfmm_batch *b, uint32_t mode) {
  if (bad(b)) return RFMM_ERR_INVALID;
  return b->engine->set_float_mode(mode);
}

int rfmm_batch_set_resort_interval(rfmm_batch *b, uint32_t steps) {
  if (bad(b)) return RFMM_ERR_INVALID;
  return b->engine->set_resort_interval(steps);
}

int rfmm_batch_set_near_mode(rfmm_batch *b, uint32_t mode) {
  if (bad(b)) return RFMM_ERR_INVALID;
  return b->engine->set_near_mode(mode);
}

int rfmm_batch_force_error(rfmm_batch *b, uint32_t scene, uint32_t targets, uint64_t seed,
                           double *rms_rel, double *max_rel) {
  if (bad_scene(b, scene)) return RFMM_ERR_INVALID;
  return b->engine->force_error(scene, targets, seed, rms_rel, max_rel);
}

int rfmm_batch_get_tuning(rfmm_batch *b, rfmm_tuning *out) {
  if (bad(b)) return RFMM_ERR_INVALID;
  return b->engine->get_tuning(out);
}

int rfmm_batch_set_tuning(rfmm_batch *b, const rfmm_tuning *tuning) {
  if (bad(b) || tuning == nullptr) return RFMM_ERR_INVALID;
  return b->engine->set_tuning(*tuning);
}

int rfmm_batch_autotune(rfmm_batch *b, uint32_t steps_per_trial, rfmm_tuning *best) {
  if (bad(b)) return RFMM_ERR_INVALID;
  return b->engine->autotune(steps_per_trial, best);
}

}  // extern "C"
