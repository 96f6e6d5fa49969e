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
// Host staging: submit copies the caller's bodies into a pinned input ring
// (a pageable copy when the ring is full), so the device copy runs at the
// host-link rate; the ring space returns as soon as the request is on the
// device.  Results land in a pinned output ring until the caller takes them.
// Host threads keep the copies off the critical path:
//   stage-in (kStageThreads)  copy queued requests into free slots, each on
//                             its own copy stream;
//   worker                    activates staged slots (sort + deposit), steps
//                             the engine, and retires finished slots (bodies
//                             back to the caller's order in a scratch range,
//                             then an event);
//   drain                     waits for that event, copies the result into
//                             the output ring on its own stream, frees the
//                             slot.
// Latency runs from the request's arrival (the entry into submit, or the
// arrival time the caller gives rfmm_server_submit_at) to the moment its
// result is in host memory.
// Results are bit-identical to a plain solve of the same scene (same kernels,
// order-independent arithmetic), whatever else shares the batch.
#include <algorithm>
#include <chrono>
#include <cmath>
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

constexpr int kStageThreads = 4;
constexpr uint64_t kDefaultStagingBytes = 4ull << 30;

// A ring of pinned host memory handing out contiguous blocks in allocation
// order; blocks may be released in any order, and the space of the oldest
// block returns once every older block is released too.
class PinnedRing {
 public:
  ~PinnedRing() {
    if (base_ != nullptr) cudaFreeHost(base_);
  }
  bool init(size_t bytes) {
    if (bytes == 0) return true;
    void *p = nullptr;
    if (cudaHostAlloc(&p, bytes, cudaHostAllocPortable) != cudaSuccess) {
      (void)cudaGetLastError();
      return false;
    }
    base_ = static_cast<uint8_t *>(p);
    cap_ = bytes;
    return true;
  }
  // A block of `bytes`, or null when the ring cannot hold it now.
  uint8_t *alloc(size_t bytes) {
    bytes = (bytes + 255u) & ~size_t(255);
    std::lock_guard<std::mutex> lk(m_);
    if (base_ == nullptr || bytes > cap_) return nullptr;
    size_t off;
    if (blocks_.empty()) {
      off = 0;
    } else {
      const size_t tail = blocks_.front().off;
      if (head_ > tail) {  // live region [tail, head): free [head, cap) and [0, tail)
        if (bytes <= cap_ - head_) {
          off = head_;
        } else if (bytes < tail) {
          off = 0;
        } else {
          return nullptr;
        }
      } else if (head_ < tail) {  // wrapped: free [head, tail)
        if (bytes < tail - head_) {
          off = head_;
        } else {
          return nullptr;
        }
      } else {
        return nullptr;  // head == tail with live blocks: full
      }
    }
    blocks_.push_back({off, true});
    head_ = off + bytes;
    return base_ + off;
  }
  // Blocks may come back in any order; null and foreign pointers are ignored.
  void release(uint8_t *p) {
    if (p == nullptr || base_ == nullptr || p < base_ || p >= base_ + cap_) return;
    std::lock_guard<std::mutex> lk(m_);
    const size_t off = (size_t)(p - base_);
    for (Block &b : blocks_)
      if (b.off == off && b.live) {
        b.live = false;
        break;
      }
    while (!blocks_.empty() && !blocks_.front().live) blocks_.pop_front();
    if (blocks_.empty()) head_ = 0;
  }

 private:
  struct Block {
    size_t off;
    bool live;
  };
  uint8_t *base_ = nullptr;
  size_t cap_ = 0, head_ = 0;
  std::deque<Block> blocks_;
  std::mutex m_;
};

struct Request {
  uint64_t id = 0;
  uint32_t n = 0, steps = 0, left = 0;
  rfmm_params params{};
  uint8_t *in_ring = nullptr;   // input in the pinned input ring, or null: `input`
  uint8_t *out_ring = nullptr;  // result in the pinned output ring, or null: `output`
  std::vector<uint8_t> input, output;
  int state = kQueued;
  int status = RFMM_OK;
  int slot = -1;
  double t_arrival = 0, t_admit = 0, t_done = 0;
  const uint8_t *in() const { return in_ring != nullptr ? in_ring : input.data(); }
  uint8_t *out() { return out_ring != nullptr ? out_ring : output.data(); }
};

struct Slot {
  SlotState state = kFree;
  Request *req = nullptr;
  cudaEvent_t ready = nullptr;  // staged input on the device / result in scratch
  uint32_t buffer = 0;          // engine particle buffer holding the staged input / the result
};

}  // namespace

class Server {
 public:
  static int create(const rfmm_server_config &cfg, Server **out);
  ~Server();
  // arrival_s: the request's arrival on now_s()'s clock; NaN = now.
  int submit(const void *host, uint32_t n, const rfmm_params *p, uint32_t steps, double arrival_s,
             uint64_t *id);
  int status(uint64_t id, int *state);
  int wait(uint64_t id, uint32_t timeout_ms);
  int result(uint64_t id, void *dst, size_t bytes);
  int stats(rfmm_server_stats *out);
  int timeline(rfmm_timeline *out);

 private:
  void stage_loop(int k);
  void worker_loop();
  void drain_loop();
  int pick_free_slot(uint32_t n) const;

  Engine *E_ = nullptr;
  int device_ = 0;
  uint32_t max_chunk_ = 4;
  cudaStream_t copy_in_[kStageThreads] = {}, copy_out_ = nullptr;
  PinnedRing in_ring_, out_ring_;
  // Pinned bounce buffers (one largest request each) for inputs and results
  // that missed the rings: the copies stay asynchronous device transfers
  // from pinned memory instead of taking the driver's pageable path.
  uint8_t *bounce_in_[kStageThreads] = {}, *bounce_out_ = nullptr;
  std::vector<Slot> slots_;
  std::mutex m_;
  std::mutex eng_m_;  // the engine: held by the worker for an iteration, and by timeline()
  std::condition_variable cv_;  // any state change
  std::deque<Request *> queue_;
  std::deque<int> staged_fifo_, drain_fifo_;
  std::unordered_map<uint64_t, Request *> reqs_;
  uint64_t next_id_ = 1;
  bool stop_ = false;
  int failure_ = RFMM_OK;
  std::vector<std::thread> stage_thr_;
  std::thread worker_thr_, drain_thr_;
  // statistics
  std::vector<double> latencies_ms_;
  double first_submit_ = 0, last_done_ = 0, body_steps_ = 0;
  uint64_t submitted_ = 0, completed_ = 0;
  // worker counters (written by the worker thread under m_)
  uint64_t chunks_ = 0, pageable_inputs_ = 0;
  double active_sum_ = 0, wait_s_ = 0, admit_s_ = 0, lists_s_ = 0, step_s_ = 0, retire_s_ = 0;
  double gpu_step_ms_ = 0, gpu_between_ms_ = 0;
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
  // The engine indexes body slots with 32-bit arithmetic (at most 2^30 slots).
  nslots = std::min<uint64_t>(nslots, (1ull << 30) / ((uint64_t)((cap + 255u) / 256u) * 256u));
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
  if (cfg.float_mode > 1u) {
    delete S;
    return RFMM_ERR_INVALID;
  }
  st = S->E_->set_float_mode(cfg.float_mode);
  if (st == RFMM_OK && cfg.timeline != 0u) st = S->E_->set_timeline(true);
  // Every step graph a chunk can need, captured now rather than while the
  // first requests wait.
  S->max_chunk_ = cfg.max_chunk_steps ? cfg.max_chunk_steps : 4u;
  if (st == RFMM_OK) st = S->E_->prepare_graphs(std::min(S->max_chunk_, 16u));
  if (st != RFMM_OK) {
    delete S;
    return st;
  }
  // Staging: three quarters for inputs (they wait in the queue), one quarter
  // for results; at least one largest request each.
  const uint64_t staging = cfg.staging_bytes ? cfg.staging_bytes : kDefaultStagingBytes;
  const uint64_t one = 32ull * cap;
  if (!S->in_ring_.init(std::max<uint64_t>(staging / 4 * 3, one)) ||
      !S->out_ring_.init(std::max<uint64_t>(staging / 4, one))) {
    delete S;
    return RFMM_ERR_OOM;
  }
  S->slots_.resize(nslots);
  cudaError_t e = cudaSuccess;
  for (auto &b : S->bounce_in_)
    if (e == cudaSuccess) e = cudaHostAlloc((void **)&b, one, cudaHostAllocDefault);
  if (e == cudaSuccess) e = cudaHostAlloc((void **)&S->bounce_out_, one, cudaHostAllocDefault);
  for (auto &cs : S->copy_in_)
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&S->copy_out_, cudaStreamNonBlocking);
  for (auto &sl : S->slots_)
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl.ready, cudaEventDisableTiming);
  if (e != cudaSuccess) {
    delete S;
    return cuda_status(e);
  }
  for (int k = 0; k < kStageThreads; k++) S->stage_thr_.emplace_back(&Server::stage_loop, S, k);
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
  for (auto &t : stage_thr_)
    if (t.joinable()) t.join();
  if (worker_thr_.joinable()) worker_thr_.join();
  if (drain_thr_.joinable()) drain_thr_.join();
  if (E_ != nullptr) E_->sync();
  for (auto &kv : reqs_) delete kv.second;
  for (auto &sl : slots_)
    if (sl.ready != nullptr) cudaEventDestroy(sl.ready);
  for (auto &cs : copy_in_) {
    if (cs == nullptr) continue;
    cudaStreamSynchronize(cs);
    cudaStreamDestroy(cs);
  }
  if (copy_out_ != nullptr) {
    cudaStreamSynchronize(copy_out_);
    cudaStreamDestroy(copy_out_);
  }
  for (auto &b : bounce_in_)
    if (b != nullptr) cudaFreeHost(b);
  if (bounce_out_ != nullptr) cudaFreeHost(bounce_out_);
  delete E_;
}

int Server::pick_free_slot(uint32_t n) const {
  for (size_t i = 0; i < slots_.size(); i++)
    if (slots_[i].state == kFree && E_->capacity((uint32_t)i) >= n) return (int)i;
  return -1;
}

int Server::submit(const void *host, uint32_t n, const rfmm_params *p, uint32_t steps,
                   double arrival_s, uint64_t *id) {
  const double t_entry = now_s();  // before any copy: the copy is part of the latency
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
  r->in_ring = in_ring_.alloc(32ull * n);
  const bool pageable = r->in_ring == nullptr;
  if (pageable) r->input.resize(32ull * n);
  std::memcpy(r->in_ring != nullptr ? r->in_ring : r->input.data(), host, 32ull * n);
  std::lock_guard<std::mutex> lk(m_);
  if (failure_ != RFMM_OK) {
    in_ring_.release(r->in_ring);
    delete r;
    return failure_;
  }
  r->id = next_id_++;
  if (pageable) pageable_inputs_++;
  r->t_arrival = std::isnan(arrival_s) ? t_entry : arrival_s;
  if (submitted_ == 0 || r->t_arrival < first_submit_) first_submit_ = r->t_arrival;
  submitted_++;
  reqs_[r->id] = r;
  queue_.push_back(r);
  *id = r->id;
  cv_.notify_all();
  return RFMM_OK;
}

// Copies the oldest queued request into a free slot on this thread's copy
// stream, then returns the request's input ring space.
void Server::stage_loop(int k) {
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
    // The engine's scratch particle buffer as of now (admission gathers from
    // it into the current one; a resort that flips the buffers before
    // admission makes the admission copy the slot across).
    const uint32_t buf = E_->scratch_buffer();
    slots_[s].buffer = buf;
    float4 *dst = E_->slot_bodies((uint32_t)s, buf);
    const void *from = r->in();
    if (r->in_ring == nullptr) {  // missed the ring: through this thread's bounce buffer
      std::memcpy(bounce_in_[k], r->input.data(), 32ull * r->n);
      from = bounce_in_[k];
    }
    cudaError_t e = cudaMemcpyAsync(dst, from, 32ull * r->n, cudaMemcpyHostToDevice, copy_in_[k]);
    if (e == cudaSuccess) e = cudaEventRecord(slots_[s].ready, copy_in_[k]);
    if (e == cudaSuccess) e = cudaEventSynchronize(slots_[s].ready);
    in_ring_.release(r->in_ring);  // the input is on the device (or the copy failed)
    r->in_ring = nullptr;
    std::vector<uint8_t>().swap(r->input);
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

// Slot changes (admissions, retirements) update the engine's active lists
// once per iteration.  The worker stays at most kRunAhead chunks ahead of the
// GPU, so a request staged meanwhile is admitted behind little queued work.
constexpr int kRunAhead = 2;

void Server::worker_loop() {
  cudaSetDevice(device_);
  std::vector<int> active;
  cudaEvent_t ahead[kRunAhead] = {};
  for (auto &ev : ahead) cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
  // Timing events around each chunk's step graph: chunk c uses entry
  // c % kTimed; chunk c - kTimed + 1 is read back (long complete: the worker
  // stays kRunAhead chunks ahead) just before entry c % kTimed, which holds
  // its predecessor's end, is reused.
  constexpr uint64_t kTimed = 8;
  cudaEvent_t t_begin[kTimed] = {}, t_end[kTimed] = {};
  for (uint64_t i = 0; i < kTimed; i++) {
    cudaEventCreate(&t_begin[i]);
    cudaEventCreate(&t_end[i]);
  }
  auto harvest = [&](uint64_t c) {  // c = the chunk about to be enqueued
    if (c + 1 < kTimed) return;
    const uint64_t j = (c + 1) % kTimed, pred = c % kTimed;
    float step_ms = 0.0f, between_ms = 0.0f;
    if (cudaEventSynchronize(t_end[j]) != cudaSuccess ||
        cudaEventElapsedTime(&step_ms, t_begin[j], t_end[j]) != cudaSuccess)
      return;
    const bool has_pred = c >= kTimed;  // chunk c - kTimed exists
    if (has_pred && cudaEventElapsedTime(&between_ms, t_end[pred], t_begin[j]) != cudaSuccess) between_ms = 0.0f;
    std::lock_guard<std::mutex> lk(m_);
    gpu_step_ms_ += step_ms;
    gpu_between_ms_ += between_ms;
  };
  auto destroy_events = [&] {
    for (auto &ev : ahead) cudaEventDestroy(ev);
    for (uint64_t i = 0; i < kTimed; i++) {
      cudaEventDestroy(t_begin[i]);
      cudaEventDestroy(t_end[i]);
    }
  };
  uint64_t chunks = 0;
  bool lists_stale = false;  // slots retired since the last list refresh
  for (;;) {
    std::vector<int> to_activate;
    {
      std::unique_lock<std::mutex> lk(m_);
      cv_.wait(lk, [&] { return stop_ || !staged_fifo_.empty() || !active.empty(); });
      if (stop_) {
        destroy_events();
        return;
      }
      to_activate.assign(staged_fifo_.begin(), staged_fifo_.end());
      staged_fifo_.clear();
    }
    std::lock_guard<std::mutex> engine_lock(eng_m_);  // until the end of this iteration
    // Admissions; then one refresh of the active lists covers them and the
    // retirements of the previous iteration.
    double t0 = now_s();
    int st = RFMM_OK;
    if (!to_activate.empty()) {
      // Every staged slot admitted with one sort.
      std::vector<Engine::Admission> adm;
      for (int s : to_activate)
        adm.push_back({(uint32_t)s, slots_[s].req->n, slots_[s].req->params, slots_[s].buffer});
      st = E_->activate_many(adm);
      std::lock_guard<std::mutex> lk(m_);
      for (int s : to_activate) {
        Request *r = slots_[s].req;
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
    }
    double t1 = now_s();
    const double list_wait0 = E_->list_wait_seconds();
    if ((lists_stale || !to_activate.empty()) && st == RFMM_OK) {
      st = E_->refresh_lists();
      lists_stale = false;
    }
    double t2 = now_s();
    const double list_wait = E_->list_wait_seconds() - list_wait0;
    if (active.empty()) {
      std::lock_guard<std::mutex> lk(m_);
      admit_s_ += t1 - t0;
      lists_s_ += t2 - t1 - list_wait;
      wait_s_ += list_wait;
      continue;
    }
    // Bounded run-ahead: wait for the chunk enqueued kRunAhead chunks ago.
    cudaEvent_t &slot_ev = ahead[chunks % kRunAhead];
    if (chunks >= (uint64_t)kRunAhead) cudaEventSynchronize(slot_ev);
    const double t3 = now_s();
    const size_t n_active = active.size();
    uint32_t chunk = max_chunk_;
    for (int s : active) chunk = std::min(chunk, slots_[s].req->left);
    harvest(chunks);
    if (st == RFMM_OK) st = cuda_status(cudaEventRecord(t_begin[chunks % kTimed], E_->stream()));
    if (st == RFMM_OK) st = E_->step(chunk);
    if (st == RFMM_OK) st = cuda_status(cudaEventRecord(t_end[chunks % kTimed], E_->stream()));
    if (st == RFMM_OK) st = cuda_status(cudaEventRecord(slot_ev, E_->stream()));
    chunks++;
    const double t4 = now_s();
    std::vector<int> finished;
    for (int s : active) {
      slots_[s].req->left -= chunk;
      if (slots_[s].req->left == 0u) finished.push_back(s);
    }
    if (!finished.empty()) {
      // One unpermute into the scratch buffer for every finished slot; the
      // emptied slots reach the device with the next admission or list
      // refresh, before the next step.
      std::vector<uint32_t> done(finished.begin(), finished.end());
      if (st == RFMM_OK) st = E_->retire_many(done);
      const uint32_t out_buf = E_->scratch_buffer();
      for (int s : finished) {
        slots_[s].buffer = out_buf;
        if (st == RFMM_OK) st = cuda_status(cudaEventRecord(slots_[s].ready, E_->stream()));
        active.erase(std::find(active.begin(), active.end(), s));
      }
      std::lock_guard<std::mutex> lk(m_);
      for (int s : finished) {
        slots_[s].state = kDraining;
        drain_fifo_.push_back(s);
      }
    }
    if (!finished.empty()) lists_stale = true;
    const double t5 = now_s();
    {
      std::lock_guard<std::mutex> lk(m_);
      if (st != RFMM_OK) failure_ = st;
      chunks_++;
      active_sum_ += (double)n_active;
      admit_s_ += t1 - t0;
      lists_s_ += t2 - t1 - list_wait;
      wait_s_ += list_wait + (t3 - t2);
      step_s_ += t4 - t3;
      retire_s_ += t5 - t4;
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
    r->out_ring = out_ring_.alloc(32ull * r->n);
    if (r->out_ring == nullptr) r->output.resize(32ull * r->n);
    cudaError_t e = cudaStreamWaitEvent(copy_out_, slots_[s].ready, 0);
    // A result that missed the output ring goes through the bounce buffer.
    uint8_t *to = r->out_ring != nullptr ? r->out_ring : bounce_out_;
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(to, E_->slot_bodies((uint32_t)s, slots_[s].buffer), 32ull * r->n,
                          cudaMemcpyDeviceToHost, copy_out_);
    if (e == cudaSuccess) e = cudaStreamSynchronize(copy_out_);
    if (e == cudaSuccess && r->out_ring == nullptr) std::memcpy(r->output.data(), bounce_out_, 32ull * r->n);
    std::lock_guard<std::mutex> lk(m_);
    r->t_done = now_s();
    if (e != cudaSuccess) {
      r->state = kFailed;
      r->status = cuda_status(e);
    } else {
      r->state = kDone;
      latencies_ms_.push_back(1e3 * (r->t_done - r->t_arrival));
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
  Request *r = nullptr;
  {
    std::unique_lock<std::mutex> lk(m_);
    auto it = reqs_.find(id);
    if (it == reqs_.end() || dst == nullptr) return RFMM_ERR_INVALID;
    r = it->second;
    if (r->state == kFailed) {
      const int st = r->status;
      reqs_.erase(it);
      out_ring_.release(r->out_ring);
      delete r;
      return st;
    }
    if (r->state != kDone) return RFMM_ERR_STATE;
    if (bytes != 32ull * r->n) return RFMM_ERR_INVALID;
    reqs_.erase(it);  // this caller owns the request from here
  }
  std::memcpy(dst, r->out(), bytes);  // outside the lock: other threads keep going
  out_ring_.release(r->out_ring);
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
  out->chunks = chunks_;
  out->mean_active_slots = chunks_ ? active_sum_ / (double)chunks_ : 0.0;
  out->pageable_inputs = pageable_inputs_;
  out->worker_gpu_wait_ms = 1e3 * wait_s_;
  out->worker_admit_ms = 1e3 * admit_s_;
  out->worker_lists_ms = 1e3 * lists_s_;
  out->worker_step_ms = 1e3 * step_s_;
  out->worker_retire_ms = 1e3 * retire_s_;
  out->gpu_step_ms = gpu_step_ms_;
  out->gpu_between_ms = gpu_between_ms_;
  return failure_;
}

int Server::timeline(rfmm_timeline *out) {
  if (out == nullptr) return RFMM_ERR_INVALID;
  std::lock_guard<std::mutex> lk(eng_m_);
  return E_->get_timeline(out);
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
  return srv->impl->submit(host_aos, n, params, steps, std::nan(""), request_id);
}

int rfmm_server_submit_at(rfmm_server *srv, const void *host_aos, uint32_t n,
                          const rfmm_params *params, uint32_t steps, double arrival_s,
                          uint64_t *request_id) {
  if (srv == nullptr || !std::isfinite(arrival_s)) return RFMM_ERR_INVALID;
  return srv->impl->submit(host_aos, n, params, steps, arrival_s, request_id);
}

int rfmm_server_clock(double *now) {
  if (now == nullptr) return RFMM_ERR_INVALID;
  *now = rfmm::now_s();
  return RFMM_OK;
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

int rfmm_server_get_timeline(rfmm_server *srv, rfmm_timeline *out) {
  if (srv == nullptr) return RFMM_ERR_INVALID;
  return srv->impl->timeline(out);
}

}  // extern "C"
