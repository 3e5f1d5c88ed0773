// Serving: a request loop over packed multi-job batches (hasty_server_* in
// hasty_gpu.h). Three kinds of threads share one mutex:
//   * callers submit requests, poll finished ones and read their images;
//   * loader threads parse scenes and build BVHs on the host, then upload
//     them once the device-memory budget has room (scene cache keyed by the
//     scene file; scenes without users are evicted least recently used);
//   * the batch thread admits requests (a job slot and FP64 sums within the
//     budget), packs the passes of the resident requests into a batch
//     whenever a render lane frees up, and retires requests whose last batch
//     has been accumulated (their sums are copied to the host).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <climits>
#include <cmath>
#include <condition_variable>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "packed.h"

namespace hasty {
namespace {

using Clock = std::chrono::steady_clock;

struct SceneEntry {
  enum State { kLoading, kReady, kFailed };
  std::string key;
  State state = kLoading;
  bool claimed = false;               // a loader is working on it
  std::unique_ptr<hasty_job> job;     // scene only (no single-job buffers)
  int error_code = HASTY_ERR_LOAD;
  std::string error;
  int refs = 0;                       // pending + resident requests using it
  int64_t bytes = 0;                  // device bytes (the estimate while uploading)
  uint64_t last_use = 0;
};

struct Request {
  enum State { kPending, kActive, kDone, kFailed };
  int64_t id = 0;
  std::string job_path, scene_key;
  RenderSettingsH st;
  uint64_t seed = 0;
  int32_t passes = 0;
  State state = kPending;
  int status = HASTY_OK;
  std::string error;
  double t_submit = 0, t_admit = 0, t_done = 0;
  int slot = -1;
  SceneEntry* scene = nullptr;
  double* d_acc = nullptr;            // FP64 sums on the device: colour, normal, albedo (npix x 3 each)
  int64_t acc_bytes = 0;
  uint32_t npix = 0;
  int32_t passes_issued = 0;          // passes packed into launched batches
  float exposure = 0.f;
  std::vector<double> acc;            // the sums after completion (3 x npix x 3)
  bool reported = false;
};

// A launched batch: its timing events and the requests whose last passes it
// holds.
struct InFlight {
  cudaEvent_t start = nullptr, end = nullptr;
  std::vector<Request*> finishing;
};

constexpr int64_t kDefaultBudget = int64_t(120) << 30;

std::string canonical_path(const std::string& p) {
  char buf[PATH_MAX];
  if (realpath(p.c_str(), buf)) return std::string(buf);
  return p;
}

}  // namespace
}  // namespace hasty

using namespace hasty;

struct hasty_server {
  hasty_ctx* ctx = nullptr;
  hasty_server_config cfg{};
  PackedLanes lanes;
  std::mutex mu;
  std::condition_variable cv_work, cv_load, cv_done;
  std::thread batch_thread;
  std::vector<std::thread> loaders;
  bool stopping = false;
  int fatal_code = HASTY_OK;
  std::string fatal;
  Clock::time_point t0;
  int64_t next_id = 1;
  std::map<int64_t, std::unique_ptr<Request>> requests;
  std::deque<Request*> pending;       // submitted, not yet resident (FIFO)
  std::vector<Request*> slots;        // resident requests by job slot
  std::deque<int64_t> finished;       // finished, not yet returned by poll
  std::map<std::string, std::unique_ptr<SceneEntry>> scenes;
  int64_t scene_bytes = 0, acc_bytes = 0, peak_bytes = 0;
  uint64_t use_clock = 0;
  size_t rr = 0;
  uint64_t submitted = 0, admitted = 0, completed = 0, failed = 0, samples = 0, batches = 0, launches = 0;
  double device_ms = 0;
  unsigned long long lane_stats[ST_COUNT] = {};

  double now_ms() const { return std::chrono::duration<double, std::milli>(Clock::now() - t0).count(); }
  int64_t resident_bytes() const { return lanes.bytes + scene_bytes + acc_bytes; }
  void note_peak() { peak_bytes = std::max(peak_bytes, resident_bytes()); }

  // --- all *_locked functions run with `mu` held ---
  void finish_locked(Request* r, Request::State st, int code, const std::string& msg) {
    r->state = st;
    r->status = code;
    r->error = msg;
    r->t_done = now_ms();
    if (r->scene) {
      r->scene->refs--;
      r->scene->last_use = ++use_clock;
      r->scene = nullptr;
    }
    if (st == Request::kDone) ++completed; else ++failed;
    finished.push_back(r->id);
    cv_done.notify_all();
    cv_load.notify_all();
  }

  // Drops failed scene entries nobody uses, then (if `need` > 0 bytes must be
  // freed, or the scene count is at its limit) evicts unused ready scenes,
  // least recently used first.
  void evict_locked(int64_t need, bool for_new_scene) {
    for (auto it = scenes.begin(); it != scenes.end();) {
      if (it->second->state == SceneEntry::kFailed && it->second->refs == 0) it = scenes.erase(it); else ++it;
    }
    auto over = [&] {
      int n_loaded = 0;
      for (auto& kv : scenes) if (kv.second->state != SceneEntry::kFailed) ++n_loaded;
      bool count_over = for_new_scene && n_loaded > cfg.max_resident_scenes;
      return count_over || (need > 0 && resident_bytes() + need > cfg.memory_budget);
    };
    while (over()) {
      SceneEntry* victim = nullptr;
      for (auto& kv : scenes) {
        SceneEntry* e = kv.second.get();
        if (e->state == SceneEntry::kReady && e->refs == 0 && (!victim || e->last_use < victim->last_use)) victim = e;
      }
      if (!victim) return;
      scene_bytes -= victim->bytes;
      scenes.erase(victim->key);   // frees the scene's device buffers
    }
  }

  void unload_others_locked(SceneEntry* keep) {
    for (auto& kv : scenes) {
      SceneEntry* o = kv.second.get();
      if (o == keep || o->state != SceneEntry::kReady) continue;
      scene_bytes -= o->bytes;
      o->bytes = 0;
      o->job.reset();
      o->state = SceneEntry::kLoading;
      o->claimed = false;
    }
    cv_load.notify_all();
  }

  void admit_locked(std::vector<Request*>& newly) {
    for (auto it = pending.begin(); it != pending.end();) {
      Request* r = *it;
      SceneEntry* e = r->scene;
      if (e->state == SceneEntry::kFailed) {
        it = pending.erase(it);
        finish_locked(r, Request::kFailed, e->error_code, e->error);
        continue;
      }
      if (e->state != SceneEntry::kReady) { ++it; continue; }   // later requests with a loaded scene may go first
      int slot = -1;
      for (size_t k = 0; k < slots.size(); ++k) if (!slots[k]) { slot = int(k); break; }
      if (slot < 0) return;
      const int64_t need = int64_t(r->npix) * 9 * int64_t(sizeof(double));
      if (int64_t(r->npix) > lanes.lane_paths) {
        it = pending.erase(it);
        finish_locked(r, Request::kFailed, HASTY_ERR_ARG, "frame is larger than a render lane (paths_in_flight)");
        continue;
      }
      if (lanes.bytes + e->bytes + need > cfg.memory_budget) {
        it = pending.erase(it);
        finish_locked(r, Request::kFailed, HASTY_ERR_MEMORY, "request does not fit the server's memory budget");
        continue;
      }
      if (resident_bytes() + need > cfg.memory_budget) {
        evict_locked(need, false);
        // Nothing renders, so nothing will free memory by itself: drop the
        // other loaded scenes (pending requests reload them later).
        if (resident_bytes() + need > cfg.memory_budget && acc_bytes == 0) unload_others_locked(e);
        if (resident_bytes() + need > cfg.memory_budget) return;   // memory is admitted in order
      }
      try {
        check_job_settings(r->st, e->job->host);
      } catch (const LoadError& err) {
        it = pending.erase(it);
        finish_locked(r, Request::kFailed, HASTY_ERR_LOAD, err.what());
        continue;
      }
      it = pending.erase(it);
      r->state = Request::kActive;
      r->slot = slot;
      r->t_admit = now_ms();
      r->acc_bytes = need;
      r->exposure = e->job->host.cam.exposure;
      acc_bytes += need;
      note_peak();
      slots[size_t(slot)] = r;
      ++admitted;
      newly.push_back(r);
    }
  }

  bool has_unissued_passes() const {
    for (Request* r : slots) if (r && r->state == Request::kActive && r->passes_issued < r->passes) return true;
    return false;
  }

  void fail_all_locked(int code, const std::string& msg) {
    while (!pending.empty()) {
      Request* r = pending.front();
      pending.pop_front();
      finish_locked(r, Request::kFailed, code, msg);
    }
    for (Request*& r : slots) {
      if (r && r->state == Request::kActive) {
        acc_bytes -= r->acc_bytes;
        finish_locked(r, Request::kFailed, code, msg);
      }
      r = nullptr;
    }
  }

  void batch_loop();
  void loader_loop();
};

void hasty_server::batch_loop() {
  std::vector<PackedJob> jobs(slots.size());
  std::vector<uint32_t> pass_base(slots.size(), 0);
  std::vector<int32_t> left(slots.size(), 0);
  std::deque<InFlight> inflight;
  std::vector<cudaEvent_t> spare;     // timing events for reuse
  cudaEvent_t origin = nullptr;       // reference point of the batches' device times
  cudaStream_t copy_stream = nullptr;
  double covered_ms = 0.0;            // device time counted so far ends here (ms after origin)
  int turn = 0;                       // kernel class of the next batch (pack_next)
  auto take_event = [&]() {
    if (!spare.empty()) { cudaEvent_t e = spare.back(); spare.pop_back(); return e; }
    cudaEvent_t e = nullptr;
    ck(cudaEventCreate(&e), "event");
    return e;
  };
  try {
    ck(cudaSetDevice(ctx->device), "cudaSetDevice");
    ck(cudaStreamCreateWithFlags(&copy_stream, cudaStreamNonBlocking), "stream");
    ck(cudaEventCreate(&origin), "event");
    ck(cudaEventRecord(origin, lanes.acc_stream), "event");
    for (;;) {
      std::vector<Request*> newly;
      std::vector<int> order;
      {
        std::unique_lock<std::mutex> lk(mu);
        for (;;) {
          if (stopping) break;
          admit_locked(newly);
          if (!newly.empty() || !inflight.empty() || has_unissued_passes()) break;
          cv_work.wait_for(lk, std::chrono::milliseconds(50));
        }
        if (stopping) break;
        // visiting order of the resident requests with passes left
        const size_t n = slots.size();
        for (size_t k = 0; k < n; ++k) {
          const size_t i = (rr + k) % n;
          Request* r = slots[i];
          if (r && r->state == Request::kActive && r->passes_issued < r->passes) order.push_back(int(i));
        }
        if (cfg.policy == HASTY_SERVE_SHORTEST_FIRST) {
          std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
            const Request* a = slots[size_t(x)];
            const Request* b = slots[size_t(y)];
            return uint64_t(a->passes - a->passes_issued) * a->npix < uint64_t(b->passes - b->passes_issued) * b->npix;
          });
        }
      }
      for (Request* r : newly) {
        ck(cudaMallocAsync(reinterpret_cast<void**>(&r->d_acc), size_t(r->acc_bytes), lanes.acc_stream),
           "cudaMallocAsync (sums)");
        ck(cudaMemsetAsync(r->d_acc, 0, size_t(r->acc_bytes), lanes.acc_stream), "memset sums");
        PackedJob& j = jobs[size_t(r->slot)];
        j.sc = r->scene->job->sd;
        j.sc.width = int32_t(r->st.width);
        j.sc.height = int32_t(r->st.height);
        j.sc.max_depth = r->st.max_depth;
        j.sc.rr_start = r->st.roulette_start;
        j.sc.rr_q = r->st.roulette_q;
        j.sc.two_strategies = (r->scene->job->host.has_light() && r->st.use_mis) ? 1 : 0;
        j.seed = r->seed;
        j.npix = int32_t(r->npix);
        j.path_kernel = use_path_kernel(ctx, j.sc);
        j.simple_trace = simple_trace_bvh(j.sc);
        for (int a = 0; a < 3; ++a) j.acc[a] = r->d_acc + size_t(a) * 3 * r->npix;
        pass_base[size_t(r->slot)] = 0;
        left[size_t(r->slot)] = r->passes;
      }
      if (!newly.empty()) lanes.wait_for(lanes.acc_stream);   // sums cleared before any lane adds to them
      // one batch per free lane
      while (int(inflight.size()) < lanes.n_lanes && !order.empty()) {
        std::vector<PackedChunk> chunks =
            pack_next(jobs, order, pass_base, left, lanes.lane_paths, cfg.quantum_samples, turn);
        if (chunks.empty()) break;
        InFlight f;
        f.start = take_event();
        f.end = take_event();
        lanes.launch(jobs, chunks, true, f.start);
        ck(cudaEventRecord(f.end, lanes.acc_stream), "event");
        {
          std::lock_guard<std::mutex> lk(mu);
          for (const PackedChunk& c : chunks) {
            Request* r = slots[size_t(c.job)];
            r->passes_issued += c.n_passes;
            if (r->passes_issued == r->passes) f.finishing.push_back(r);
          }
          if (!order.empty()) rr = size_t(chunks.back().job + 1) % slots.size();
          ++batches;
          launches = lanes.launches;
        }
        inflight.push_back(std::move(f));
        order.erase(std::remove_if(order.begin(), order.end(), [&](int i) { return left[size_t(i)] <= 0; }),
                    order.end());
      }
      if (inflight.empty()) continue;
      // the oldest batch: wait for its accumulation, then retire its requests
      InFlight f = std::move(inflight.front());
      inflight.pop_front();
      ck(cudaEventSynchronize(f.end), "batch");
      float t_start = 0.f, t_end = 0.f;
      ck(cudaEventElapsedTime(&t_start, origin, f.start), "event time");
      ck(cudaEventElapsedTime(&t_end, origin, f.end), "event time");
      const double busy = std::max(0.0, double(t_end) - std::max(covered_ms, double(t_start)));
      covered_ms = std::max(covered_ms, double(t_end));
      spare.push_back(f.start);
      spare.push_back(f.end);
      for (Request* r : f.finishing) {
        r->acc.resize(size_t(r->npix) * 9);
        ck(cudaMemcpyAsync(r->acc.data(), r->d_acc, size_t(r->acc_bytes), cudaMemcpyDeviceToHost, copy_stream),
           "copy sums");
        ck(cudaFreeAsync(r->d_acc, copy_stream), "cudaFreeAsync (sums)");
        r->d_acc = nullptr;
      }
      if (!f.finishing.empty()) ck(cudaStreamSynchronize(copy_stream), "copy sums");
      unsigned long long st[ST_COUNT];
      lanes.read_stats(st);
      std::lock_guard<std::mutex> lk(mu);
      device_ms += busy;
      std::memcpy(lane_stats, st, sizeof(st));
      for (Request* r : f.finishing) {
        slots[size_t(r->slot)] = nullptr;
        acc_bytes -= r->acc_bytes;
        samples += uint64_t(r->npix) * uint64_t(r->passes);
        finish_locked(r, Request::kDone, HASTY_OK, "");
      }
    }
  } catch (const ApiError& e) {
    std::lock_guard<std::mutex> lk(mu);
    fatal_code = e.code;
    fatal = e.msg;
    fail_all_locked(e.code, "server batch loop failed: " + e.msg);
    stopping = true;
    cv_load.notify_all();
    cv_done.notify_all();
  } catch (const std::exception& e) {
    std::lock_guard<std::mutex> lk(mu);
    fatal_code = HASTY_ERR_CUDA;
    fatal = e.what();
    fail_all_locked(HASTY_ERR_CUDA, std::string("server batch loop failed: ") + e.what());
    stopping = true;
    cv_load.notify_all();
    cv_done.notify_all();
  }
  // batches still in flight finish before their events and sums go away
  for (int k = 0; k < lanes.n_lanes; ++k) if (lanes.lane_stream[k]) cudaStreamSynchronize(lanes.lane_stream[k]);
  if (lanes.acc_stream) cudaStreamSynchronize(lanes.acc_stream);
  for (InFlight& f : inflight) { spare.push_back(f.start); spare.push_back(f.end); }
  for (cudaEvent_t e : spare) cudaEventDestroy(e);
  if (origin) cudaEventDestroy(origin);
  if (copy_stream) { cudaStreamSynchronize(copy_stream); cudaStreamDestroy(copy_stream); }
}

void hasty_server::loader_loop() {
  cudaSetDevice(ctx->device);
  for (;;) {
    SceneEntry* e = nullptr;
    std::string path;
    {
      std::unique_lock<std::mutex> lk(mu);
      for (;;) {
        if (stopping) return;
        for (Request* r : pending) {
          if (r->scene->state == SceneEntry::kLoading && !r->scene->claimed) { e = r->scene; path = r->job_path; break; }
        }
        if (e) { e->claimed = true; break; }
        cv_load.wait_for(lk, std::chrono::milliseconds(100));
      }
    }
    std::unique_ptr<hasty_job> j;
    int code = HASTY_OK;
    std::string msg;
    try {
      j = load_job_host(ctx, path);
      const int64_t est = prepare_job_upload(*j);   // host BVH build; exact device bytes of the upload
      {
        std::unique_lock<std::mutex> lk(mu);
        for (;;) {
          if (stopping) { code = HASTY_ERR_STOPPED; msg = "server stopped"; break; }
          if (lanes.bytes + est > cfg.memory_budget) {
            code = HASTY_ERR_MEMORY;
            msg = "scene needs " + std::to_string(est) + " device bytes; the server's memory budget cannot hold it";
            break;
          }
          evict_locked(est, true);
          bool fits = resident_bytes() + est <= cfg.memory_budget;
          int n_loaded = 0;
          for (auto& kv : scenes) if (kv.second->state == SceneEntry::kReady) ++n_loaded;
          if (fits && n_loaded < cfg.max_resident_scenes) break;
          cv_load.wait_for(lk, std::chrono::milliseconds(50));
        }
        if (code == HASTY_OK) {
          e->bytes = est;
          scene_bytes += est;
          note_peak();
        }
      }
      if (code == HASTY_OK) {
        try {
          finish_job_load(*j, false);
        } catch (...) {
          std::lock_guard<std::mutex> lk(mu);
          scene_bytes -= est;
          e->bytes = 0;
          throw;
        }
      }
    } catch (const ApiError& err) {
      code = err.code; msg = err.msg;
    } catch (const LoadError& err) {
      code = HASTY_ERR_LOAD; msg = err.what();
    } catch (const std::bad_alloc&) {
      code = HASTY_ERR_MEMORY; msg = "host allocation failed";
    } catch (const std::exception& err) {
      code = HASTY_ERR_CUDA; msg = err.what();
    }
    std::lock_guard<std::mutex> lk(mu);
    if (code == HASTY_OK) {
      scene_bytes += j->bytes - e->bytes;
      e->bytes = j->bytes;
      e->job = std::move(j);
      e->state = SceneEntry::kReady;
      e->last_use = ++use_clock;
      note_peak();
    } else {
      e->state = SceneEntry::kFailed;
      e->error_code = code;
      e->error = msg;
    }
    cv_work.notify_all();
  }
}

namespace {

Request* find_request(hasty_server* s, int64_t id) {
  auto it = s->requests.find(id);
  if (it == s->requests.end()) throw ApiError{HASTY_ERR_ARG, "unknown request id " + std::to_string(id)};
  return it->second.get();
}

Request* finished_request(hasty_server* s, int64_t id, int aov, size_t w, size_t h) {
  Request* r = find_request(s, id);
  if (r->state != Request::kDone) throw ApiError{HASTY_ERR_ARG, "request " + std::to_string(id) + " has no result"};
  if (aov < 0 || aov > 2) throw ApiError{HASTY_ERR_ARG, "bad aov"};
  if (w != r->st.width || h != r->st.height) throw ApiError{HASTY_ERR_ARG, "buffer size does not match the frame"};
  return r;
}

void clamp_config(hasty_server_config& c) {
  if (c.lanes <= 0) c.lanes = 2;
  if (c.lanes > kMaxLanes) throw ApiError{HASTY_ERR_ARG, "render lanes must be 1.." + std::to_string(kMaxLanes)};
  c.paths_in_flight = packed_lane_paths(c.paths_in_flight, 1);
  if (c.max_resident_jobs <= 0) c.max_resident_jobs = 32;
  if (c.max_resident_scenes <= 0) c.max_resident_scenes = 32;
  if (c.memory_budget <= 0) c.memory_budget = kDefaultBudget;
  if (c.loader_threads <= 0) c.loader_threads = 2;
  if (c.quantum_samples <= 0) c.quantum_samples = std::max<int64_t>(1, c.paths_in_flight / 4);
  if (c.policy != HASTY_SERVE_ROUND_ROBIN && c.policy != HASTY_SERVE_SHORTEST_FIRST)
    throw ApiError{HASTY_ERR_ARG, "unknown serving policy"};
}

}  // namespace

extern "C" {

int hasty_server_start(hasty_ctx* ctx, const hasty_server_config* cfg, hasty_server** out) {
  return guarded([&] {
    if (!ctx || !out) throw ApiError{HASTY_ERR_ARG, "null argument"};
    std::unique_ptr<hasty_server> s(new hasty_server());
    s->ctx = ctx;
    if (cfg) s->cfg = *cfg;
    clamp_config(s->cfg);
    s->lanes.init(ctx, s->cfg.lanes, s->cfg.paths_in_flight);
    s->lanes.resolve_threads = s->cfg.resolve_threads;
    s->lanes.sample_threads = s->cfg.sample_threads;
    s->lanes.trace_blocks_per_sm = s->cfg.trace_blocks_per_sm;
    s->slots.assign(size_t(s->cfg.max_resident_jobs), nullptr);
    s->t0 = Clock::now();
    s->note_peak();
    hasty_server* raw = s.get();
    s->batch_thread = std::thread([raw] { raw->batch_loop(); });
    for (int k = 0; k < s->cfg.loader_threads; ++k) s->loaders.emplace_back([raw] { raw->loader_loop(); });
    *out = s.release();
    return HASTY_OK;
  });
}

int hasty_server_submit(hasty_server* s, const char* path, int32_t passes, const uint64_t* seed, int64_t* id) {
  return guarded([&] {
    if (!s || !path || !id) throw ApiError{HASTY_ERR_ARG, "null argument"};
    std::unique_ptr<Request> r(new Request());
    std::string scene_path;
    load_job_settings(path, r->st, scene_path);
    if (r->st.max_depth <= 0) throw ApiError{HASTY_ERR_ARG, "max_depth must be positive for serving"};
    uint64_t npix = uint64_t(r->st.width) * uint64_t(r->st.height);
    if (npix >= (uint64_t(1) << 31)) throw ApiError{HASTY_ERR_ARG, "frame too large"};
    r->job_path = path;
    r->scene_key = canonical_path(scene_path);
    r->passes = passes > 0 ? passes : r->st.num_samples;
    if (r->passes <= 0) throw ApiError{HASTY_ERR_ARG, "request has no passes"};
    r->seed = seed ? *seed : r->st.seed;
    r->npix = uint32_t(npix);
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stopping) throw ApiError{HASTY_ERR_STOPPED, s->fatal.empty() ? "server stopped" : "server failed: " + s->fatal};
    r->id = s->next_id++;
    r->t_submit = s->now_ms();
    auto& slot = s->scenes[r->scene_key];
    if (!slot) { slot.reset(new SceneEntry()); slot->key = r->scene_key; }
    slot->refs++;
    r->scene = slot.get();
    *id = r->id;
    s->pending.push_back(r.get());
    s->requests[r->id] = std::move(r);
    ++s->submitted;
    s->cv_load.notify_all();
    s->cv_work.notify_all();
    return HASTY_OK;
  });
}

int hasty_server_poll(hasty_server* s, hasty_server_result* out, size_t max, size_t* n, int32_t wait_ms) {
  return guarded([&] {
    if (!s || !n || (max && !out)) throw ApiError{HASTY_ERR_ARG, "null argument"};
    std::unique_lock<std::mutex> lk(s->mu);
    if (s->finished.empty() && wait_ms > 0)
      s->cv_done.wait_for(lk, std::chrono::milliseconds(wait_ms), [&] { return !s->finished.empty() || s->stopping; });
    size_t k = 0;
    while (k < max && !s->finished.empty()) {
      int64_t id = s->finished.front();
      s->finished.pop_front();
      auto it = s->requests.find(id);
      if (it == s->requests.end()) continue;
      Request* r = it->second.get();
      hasty_server_result& o = out[k++];
      std::memset(&o, 0, sizeof(o));
      o.id = r->id;
      o.status = r->status;
      o.width = int32_t(r->st.width);
      o.height = int32_t(r->st.height);
      o.passes = r->passes;
      o.samples = r->state == Request::kDone ? uint64_t(r->npix) * uint64_t(r->passes) : 0;
      o.submit_ms = r->t_submit;
      o.admit_ms = r->t_admit;
      o.finish_ms = r->t_done;
      o.latency_ms = r->t_done - r->t_submit;
      std::strncpy(o.error, r->error.c_str(), sizeof(o.error) - 1);
      r->reported = true;
    }
    *n = k;
    return HASTY_OK;
  });
}

int hasty_server_read_sums(hasty_server* s, int64_t id, int aov, double* host, size_t w, size_t h) {
  return guarded([&] {
    if (!s || !host) throw ApiError{HASTY_ERR_ARG, "null argument"};
    std::lock_guard<std::mutex> lk(s->mu);
    Request* r = finished_request(s, id, aov, w, h);
    std::memcpy(host, r->acc.data() + size_t(aov) * 3 * r->npix, sizeof(double) * 3 * r->npix);
    return HASTY_OK;
  });
}

int hasty_server_read(hasty_server* s, int64_t id, int aov, float* host, size_t w, size_t h) {
  return guarded([&] {
    if (!s || !host) throw ApiError{HASTY_ERR_ARG, "null argument"};
    std::lock_guard<std::mutex> lk(s->mu);
    Request* r = finished_request(s, id, aov, w, h);
    const float den = 1e-7f + float(r->passes);
    const float scale = aov == HASTY_AOV_COLOR ? std::pow(2.0f, r->exposure) : 1.0f;
    const double* sums = r->acc.data() + size_t(aov) * 3 * r->npix;
    for (size_t i = 0; i < size_t(r->npix) * 3; ++i) host[i] = (float(sums[i]) / den) * scale;
    return HASTY_OK;
  });
}

int hasty_server_release(hasty_server* s, int64_t id) {
  return guarded([&] {
    if (!s) throw ApiError{HASTY_ERR_ARG, "null argument"};
    std::lock_guard<std::mutex> lk(s->mu);
    Request* r = find_request(s, id);
    if (r->state == Request::kPending || r->state == Request::kActive)
      throw ApiError{HASTY_ERR_ARG, "request " + std::to_string(id) + " has not finished"};
    s->requests.erase(id);
    return HASTY_OK;
  });
}

int hasty_server_stats_get(hasty_server* s, hasty_server_stats* out) {
  return guarded([&] {
    if (!s || !out) throw ApiError{HASTY_ERR_ARG, "null argument"};
    std::lock_guard<std::mutex> lk(s->mu);
    std::memset(out, 0, sizeof(*out));
    out->submitted = s->submitted; out->admitted = s->admitted; out->completed = s->completed; out->failed = s->failed;
    out->samples = s->samples;
    out->rays = s->lane_stats[ST_RAYS]; out->shaded = s->lane_stats[ST_SHADED];
    out->batches = s->batches; out->kernel_launches = s->launches;
    out->device_ms = s->device_ms;
    out->uptime_ms = s->now_ms();
    out->resident_bytes = s->resident_bytes();
    out->peak_resident_bytes = s->peak_bytes;
    out->engine_bytes = s->lanes.bytes;
    int rj = 0;
    for (Request* r : s->slots) if (r) ++rj;
    out->resident_jobs = rj;
    int rs = 0;
    for (auto& kv : s->scenes) if (kv.second->state == SceneEntry::kReady) ++rs;
    out->resident_scenes = rs;
    out->pending = int32_t(s->pending.size());
    return HASTY_OK;
  });
}

int hasty_server_wait_idle(hasty_server* s, int32_t timeout_ms) {
  return guarded([&] {
    if (!s) throw ApiError{HASTY_ERR_ARG, "null argument"};
    std::unique_lock<std::mutex> lk(s->mu);
    auto idle = [&] { return s->completed + s->failed == s->submitted; };
    bool ok = timeout_ms < 0 ? (s->cv_done.wait(lk, idle), true)
                             : s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), idle);
    if (!ok) throw ApiError{HASTY_ERR_STOPPED, "requests still running at the timeout"};
    if (s->fatal_code != HASTY_OK) throw ApiError{s->fatal_code, "server batch loop failed: " + s->fatal};
    return HASTY_OK;
  });
}

int hasty_server_stop(hasty_server* s) {
  if (!s) return fail(HASTY_ERR_ARG, "null argument");
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stopping = true;
    s->cv_work.notify_all();
    s->cv_load.notify_all();
    s->cv_done.notify_all();
  }
  if (s->batch_thread.joinable()) s->batch_thread.join();
  for (std::thread& t : s->loaders) if (t.joinable()) t.join();
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->fail_all_locked(HASTY_ERR_STOPPED, "server stopped");
  }
  // request sums still on the device were allocated on the accumulation stream
  for (auto& kv : s->requests) {
    if (kv.second->d_acc) cudaFreeAsync(kv.second->d_acc, s->lanes.acc_stream);
  }
  if (s->lanes.acc_stream) cudaStreamSynchronize(s->lanes.acc_stream);
  delete s;
  return HASTY_OK;
}

}  // extern "C"
