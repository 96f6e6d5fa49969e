// Served form: continuous batching of solve requests on one GPU.
//
// A request is a scene (bodies in the reference Particle layout), physics
// parameters and a step count.  The server owns one engine whose scenes are
// fixed-capacity slots sized to fit a device-memory budget.  Requests queue
// on submit; a free slot admits the oldest waiting request while the others
// keep running, and every step of the engine advances all occupied slots in
// the same launches (the batched step).  Finished scenes leave their slot at
// a step boundary and the slot is refilled.
//
// Three host threads keep copies off the critical path:
//   stage-in  copies a request's bodies into its slot on a copy stream;
//   worker    activates staged slots (sort + deposit), steps the engine, and
//             retires finished slots (bodies back to the caller's order in a
//             scratch range, then an event);
//   drain     waits for that event and copies the result to host memory on
//             its own stream, then frees the slot.
// Results are bit-identical to a plain solve of the same scene (same kernels,
// order-independent arithmetic), whatever else shares the batch.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <new>
#include <thread>
#include <unordered_map>
#include <vector>

#include "engine.h"
#include "rfmm.h"
#include "rfmm_internal.h"

namespace rfmm {
namespace {

double now_s() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

enum ReqState { kQueued = 0, kRunning = 1, kDone = 2, kFailed = 3 };
enum SlotState { kFree, kStaging, kStaged, kActive, kDraining };

struct Request {
  uint64_t id = 0;
  uint32_t n = 0, steps = 0, left = 0;
  rfmm_params params{};
  std::vector<uint8_t> input, output;
  int state = kQueued;
  int status = RFMM_OK;
  int slot = -1;
  double t_submit = 0, t_admit = 0, t_done = 0;
};

struct Slot {
  SlotState state = kFree;
  Request *req = nullptr;
  cudaEvent_t ready = nullptr;  // staged input on the device / result in scratch
};

}  // namespace

class Server {
 public:
  static int create(const rfmm_server_config &cfg, Server **out);
  ~Server();
  int submit(const void *host, uint32_t n, const rfmm_params *p, uint32_t steps, uint64_t *id);
  int status(uint64_t id, int *state);
  int wait(uint64_t id, uint32_t timeout_ms);
  int result(uint64_t id, void *dst, size_t bytes);
  int stats(rfmm_server_stats *out);

 private:
  void stage_loop();
  void worker_loop();
  void drain_loop();
  int pick_free_slot(uint32_t n) const;

  Engine *E_ = nullptr;
  int device_ = 0;
  uint32_t max_chunk_ = 4;
  cudaStream_t copy_in_ = nullptr, copy_out_ = nullptr;
  std::vector<Slot> slots_;
  std::mutex m_;
  std::condition_variable cv_;  // any state change
  std::deque<Request *> queue_;
  std::deque<int> staged_fifo_, drain_fifo_;
  std::unordered_map<uint64_t, Request *> reqs_;
  uint64_t next_id_ = 1;
  bool stop_ = false;
  int failure_ = RFMM_OK;
  std::thread stage_thr_, worker_thr_, drain_thr_;
  // statistics
  std::vector<double> latencies_ms_;
  double first_submit_ = 0, last_done_ = 0, body_steps_ = 0;
  uint64_t submitted_ = 0, completed_ = 0;
};

int Server::create(const rfmm_server_config &cfg, Server **out) {
  if (out == nullptr || cfg.max_bodies == 0u || cfg.max_bodies > (1u << 23)) return RFMM_ERR_INVALID;
  *out = nullptr;
  const uint32_t cap = cfg.max_bodies;
  const uint32_t depth = depth_for_particles(cap);
  // Device bytes per slot: bodies (2 x 32 B + 2 x 4 B ids + 16 B sort scratch),
  // tree (2 x 16 moments + 16 src + 16 aux + 4 choice + 48 lfield + 48 fields
  // + 16 work lists), plus tensor maps.
  const uint64_t per_slot = (uint64_t)((cap + 255u) / 256u) * 256u * 88u +
                            (uint64_t)total_cells(depth) * 184u + 8u * 128u;
  uint64_t nslots = cfg.memory_budget_bytes / per_slot;
  if (cfg.max_slots != 0u) nslots = std::min<uint64_t>(nslots, cfg.max_slots);
  nslots = std::min<uint64_t>(nslots, 4096u);
  if (nslots == 0u) return RFMM_ERR_BUDGET;

  std::vector<SceneSpec> specs(nslots);
  for (auto &sp : specs) {
    sp.n = cap;
    rfmm_default_params(&sp.params);
    sp.params.depth = depth;
    sp.slot = true;
  }
  Server *S = new (std::nothrow) Server();
  if (S == nullptr) return RFMM_ERR_OOM;
  int st = Engine::create(specs, &S->E_);
  if (st != RFMM_OK) {
    delete S;
    return st;
  }
  cudaGetDevice(&S->device_);
  S->max_chunk_ = cfg.max_chunk_steps ? cfg.max_chunk_steps : 4u;
  S->slots_.resize(nslots);
  cudaError_t e = cudaStreamCreateWithFlags(&S->copy_in_, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&S->copy_out_, cudaStreamNonBlocking);
  for (auto &sl : S->slots_)
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl.ready, cudaEventDisableTiming);
  if (e != cudaSuccess) {
    delete S;
    return cuda_status(e);
  }
  S->stage_thr_ = std::thread(&Server::stage_loop, S);
  S->worker_thr_ = std::thread(&Server::worker_loop, S);
  S->drain_thr_ = std::thread(&Server::drain_loop, S);
  *out = S;
  return RFMM_OK;
}

Server::~Server() {
  {
    std::lock_guard<std::mutex> lk(m_);
    stop_ = true;
  }
  cv_.notify_all();
  if (stage_thr_.joinable()) stage_thr_.join();
  if (worker_thr_.joinable()) worker_thr_.join();
  if (drain_thr_.joinable()) drain_thr_.join();
  for (auto &kv : reqs_) delete kv.second;
  for (auto &sl : slots_)
    if (sl.ready != nullptr) cudaEventDestroy(sl.ready);
  if (copy_in_ != nullptr) cudaStreamDestroy(copy_in_);
  if (copy_out_ != nullptr) cudaStreamDestroy(copy_out_);
  delete E_;
}

int Server::pick_free_slot(uint32_t n) const {
  for (size_t i = 0; i < slots_.size(); i++)
    if (slots_[i].state == kFree && E_->capacity((uint32_t)i) >= n) return (int)i;
  return -1;
}

int Server::submit(const void *host, uint32_t n, const rfmm_params *p, uint32_t steps,
                   uint64_t *id) {
  if (host == nullptr || n == 0u || steps == 0u || id == nullptr) return RFMM_ERR_INVALID;
  if (n > E_->capacity(0)) return RFMM_ERR_BUDGET;
  Request *r = new (std::nothrow) Request();
  if (r == nullptr) return RFMM_ERR_OOM;
  r->n = n;
  r->steps = r->left = steps;
  if (p != nullptr) {
    r->params = *p;
  } else {
    rfmm_default_params(&r->params);
  }
  const uint32_t depth = r->params.depth ? r->params.depth : depth_for_particles(n);
  if (depth < 4u || depth > depth_for_particles(E_->capacity(0))) {
    delete r;
    return RFMM_ERR_BUDGET;
  }
  r->input.resize(32ull * n);
  std::memcpy(r->input.data(), host, r->input.size());
  std::lock_guard<std::mutex> lk(m_);
  if (failure_ != RFMM_OK) {
    delete r;
    return failure_;
  }
  r->id = next_id_++;
  r->t_submit = now_s();
  if (submitted_ == 0) first_submit_ = r->t_submit;
  submitted_++;
  reqs_[r->id] = r;
  queue_.push_back(r);
  *id = r->id;
  cv_.notify_all();
  return RFMM_OK;
}

// Copies the oldest queued request into a free slot on the input copy stream.
void Server::stage_loop() {
  cudaSetDevice(device_);
  for (;;) {
    Request *r = nullptr;
    int s = -1;
    {
      std::unique_lock<std::mutex> lk(m_);
      cv_.wait(lk, [&] {
        return stop_ || (!queue_.empty() && pick_free_slot(queue_.front()->n) >= 0);
      });
      if (stop_) return;
      r = queue_.front();
      queue_.pop_front();
      s = pick_free_slot(r->n);
      slots_[s].state = kStaging;
      slots_[s].req = r;
      r->slot = s;
    }
    float4 *dst = E_->slot_bodies((uint32_t)s);
    cudaError_t e = cudaMemcpyAsync(dst, r->input.data(), r->input.size(), cudaMemcpyHostToDevice,
                                    copy_in_);
    if (e == cudaSuccess) e = cudaEventRecord(slots_[s].ready, copy_in_);
    if (e == cudaSuccess) e = cudaEventSynchronize(slots_[s].ready);
    std::lock_guard<std::mutex> lk(m_);
    if (e != cudaSuccess) {
      r->state = kFailed;
      r->status = cuda_status(e);
      slots_[s].state = kFree;
      slots_[s].req = nullptr;
    } else {
      slots_[s].state = kStaged;
      staged_fifo_.push_back(s);
    }
    cv_.notify_all();
  }
}

void Server::worker_loop() {
  cudaSetDevice(device_);
  std::vector<int> active;
  for (;;) {
    std::vector<int> to_activate;
    {
      std::unique_lock<std::mutex> lk(m_);
      cv_.wait(lk, [&] { return stop_ || !staged_fifo_.empty() || !active.empty(); });
      if (stop_) return;
      to_activate.assign(staged_fifo_.begin(), staged_fifo_.end());
      staged_fifo_.clear();
    }
    int st = RFMM_OK;
    for (int s : to_activate) {
      Request *r = slots_[s].req;
      st = E_->activate((uint32_t)s, r->n, r->params, nullptr, cudaMemcpyDeviceToDevice);
      std::lock_guard<std::mutex> lk(m_);
      if (st != RFMM_OK) {
        r->state = kFailed;
        r->status = st;
        slots_[s].state = kFree;
        slots_[s].req = nullptr;
        failure_ = st;
      } else {
        slots_[s].state = kActive;
        r->state = kRunning;
        r->t_admit = now_s();
        active.push_back(s);
      }
    }
    if (active.empty()) continue;
    uint32_t chunk = max_chunk_;
    for (int s : active) chunk = std::min(chunk, slots_[s].req->left);
    st = E_->step(chunk);
    std::vector<int> finished;
    for (int s : active) {
      slots_[s].req->left -= chunk;
      if (slots_[s].req->left == 0u) finished.push_back(s);
    }
    for (int s : finished) {
      if (st == RFMM_OK) st = E_->retire((uint32_t)s);  // unpermute into scratch, slot emptied
      if (st == RFMM_OK) st = cuda_status(cudaEventRecord(slots_[s].ready, E_->stream()));
      active.erase(std::find(active.begin(), active.end(), s));
      std::lock_guard<std::mutex> lk(m_);
      slots_[s].state = kDraining;
      drain_fifo_.push_back(s);
    }
    if (st != RFMM_OK) {
      std::lock_guard<std::mutex> lk(m_);
      failure_ = st;
    }
    if (!finished.empty()) cv_.notify_all();
  }
}

void Server::drain_loop() {
  cudaSetDevice(device_);
  for (;;) {
    int s = -1;
    {
      std::unique_lock<std::mutex> lk(m_);
      cv_.wait(lk, [&] { return stop_ || !drain_fifo_.empty(); });
      if (stop_ && drain_fifo_.empty()) return;
      s = drain_fifo_.front();
      drain_fifo_.pop_front();
    }
    Request *r = slots_[s].req;
    r->output.resize(32ull * r->n);
    cudaError_t e = cudaStreamWaitEvent(copy_out_, slots_[s].ready, 0);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(r->output.data(), E_->slot_scratch((uint32_t)s), r->output.size(),
                          cudaMemcpyDeviceToHost, copy_out_);
    if (e == cudaSuccess) e = cudaStreamSynchronize(copy_out_);
    std::lock_guard<std::mutex> lk(m_);
    r->t_done = now_s();
    if (e != cudaSuccess) {
      r->state = kFailed;
      r->status = cuda_status(e);
    } else {
      r->state = kDone;
      latencies_ms_.push_back(1e3 * (r->t_done - r->t_submit));
      body_steps_ += (double)r->n * r->steps;
      last_done_ = r->t_done;
      completed_++;
    }
    slots_[s].state = kFree;
    slots_[s].req = nullptr;
    cv_.notify_all();
  }
}

int Server::status(uint64_t id, int *state) {
  std::lock_guard<std::mutex> lk(m_);
  auto it = reqs_.find(id);
  if (it == reqs_.end() || state == nullptr) return RFMM_ERR_INVALID;
  *state = it->second->state;
  return it->second->state == kFailed ? it->second->status : RFMM_OK;
}

int Server::wait(uint64_t id, uint32_t timeout_ms) {
  std::unique_lock<std::mutex> lk(m_);
  auto it = reqs_.find(id);
  if (it == reqs_.end()) return RFMM_ERR_INVALID;
  Request *r = it->second;
  const bool ok = cv_.wait_for(lk, std::chrono::milliseconds(timeout_ms),
                               [&] { return r->state == kDone || r->state == kFailed; });
  if (!ok) return RFMM_ERR_TIMEOUT;
  return r->state == kFailed ? r->status : RFMM_OK;
}

int Server::result(uint64_t id, void *dst, size_t bytes) {
  std::unique_lock<std::mutex> lk(m_);
  auto it = reqs_.find(id);
  if (it == reqs_.end() || dst == nullptr) return RFMM_ERR_INVALID;
  Request *r = it->second;
  if (r->state == kFailed) {
    const int st = r->status;
    reqs_.erase(it);
    delete r;
    return st;
  }
  if (r->state != kDone) return RFMM_ERR_STATE;
  if (bytes != r->output.size()) return RFMM_ERR_INVALID;
  std::memcpy(dst, r->output.data(), bytes);
  reqs_.erase(it);
  delete r;
  return RFMM_OK;
}

int Server::stats(rfmm_server_stats *out) {
  if (out == nullptr) return RFMM_ERR_INVALID;
  std::lock_guard<std::mutex> lk(m_);
  std::memset(out, 0, sizeof(*out));
  out->submitted = submitted_;
  out->completed = completed_;
  out->queued = queue_.size();
  uint64_t act = 0;
  for (const Slot &sl : slots_) act += sl.state != kFree ? 1u : 0u;
  out->in_flight = act;
  out->slots = (uint32_t)slots_.size();
  out->slot_capacity = E_->capacity(0);
  out->device_bytes = E_->device_bytes();
  if (!latencies_ms_.empty()) {
    std::vector<double> v = latencies_ms_;
    std::sort(v.begin(), v.end());
    auto q = [&](double f) { return v[std::min(v.size() - 1, (size_t)(f * (v.size() - 1) + 0.5))]; };
    out->p50_ms = q(0.50);
    out->p99_ms = q(0.99);
    double sum = 0;
    for (double x : v) sum += x;
    out->mean_ms = sum / v.size();
    out->max_ms = v.back();
  }
  if (last_done_ > first_submit_) out->body_steps_per_s = body_steps_ / (last_done_ - first_submit_);
  out->body_steps = body_steps_;
  return failure_;
}

}  // namespace rfmm

struct rfmm_server {
  rfmm::Server *impl;
};

extern "C" {

int rfmm_server_create(const rfmm_server_config *cfg, rfmm_server **out) {
  if (cfg == nullptr || out == nullptr) return RFMM_ERR_INVALID;
  *out = nullptr;
  rfmm::Server *s = nullptr;
  const int st = rfmm::Server::create(*cfg, &s);
  if (st != RFMM_OK) return st;
  *out = new (std::nothrow) rfmm_server{s};
  if (*out == nullptr) {
    delete s;
    return RFMM_ERR_OOM;
  }
  return RFMM_OK;
}

int rfmm_server_destroy(rfmm_server *srv) {
  if (srv == nullptr) return RFMM_ERR_INVALID;
  delete srv->impl;
  delete srv;
  return RFMM_OK;
}

int rfmm_server_submit(rfmm_server *srv, const void *host_aos, uint32_t n, const rfmm_params *params,
                       uint32_t steps, uint64_t *request_id) {
  if (srv == nullptr) return RFMM_ERR_INVALID;
  return srv->impl->submit(host_aos, n, params, steps, request_id);
}

int rfmm_server_status(rfmm_server *srv, uint64_t request_id, int *state) {
  if (srv == nullptr) return RFMM_ERR_INVALID;
  return srv->impl->status(request_id, state);
}

int rfmm_server_wait(rfmm_server *srv, uint64_t request_id, uint32_t timeout_ms) {
  if (srv == nullptr) return RFMM_ERR_INVALID;
  return srv->impl->wait(request_id, timeout_ms);
}

int rfmm_server_result(rfmm_server *srv, uint64_t request_id, void *host_dst, size_t bytes) {
  if (srv == nullptr) return RFMM_ERR_INVALID;
  return srv->impl->result(request_id, host_dst, bytes);
}

int rfmm_server_get_stats(rfmm_server *srv, rfmm_server_stats *out) {
  if (srv == nullptr) return RFMM_ERR_INVALID;
  return srv->impl->stats(out);
}

}  // extern "C"
