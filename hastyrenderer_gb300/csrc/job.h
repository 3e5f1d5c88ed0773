// Internal state behind the C ABI: context, job and the error helpers
// shared by api.cpp (single-job path) and engine.cpp (multi-job engine).
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstddef>
#include <functional>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "bvh_build.h"
#include "hasty_gpu.h"
#include "scene_load.h"
#include "wavefront.h"

namespace hasty {

extern thread_local std::string g_error;

struct ApiError {
  int code; std::string msg;
};

inline int fail(int code, const std::string& m) { g_error = m; return code; }

inline void ck(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    int code = (e == cudaErrorMemoryAllocation) ? HASTY_ERR_MEMORY : HASTY_ERR_CUDA;
    throw ApiError{code, std::string(what) + ": " + cudaGetErrorString(e)};
  }
}

template <class F>
int guarded(F&& f) {
  try {
    return f();
  } catch (const ApiError& e) {
    return fail(e.code, e.msg);
  } catch (const LoadError& e) {
    return fail(HASTY_ERR_LOAD, e.what());
  } catch (const std::bad_alloc&) {
    return fail(HASTY_ERR_MEMORY, "host allocation failed");
  } catch (const std::exception& e) {
    return fail(HASTY_ERR_CUDA, e.what());
  }
}
}  // namespace hasty

using hasty::ApiError;
using hasty::ck;
using hasty::HostScene;
using hasty::SceneDev;
using hasty::PathsDev;

namespace hasty {
struct PmDev;                    // photon-mapper state (photon_map.cpp)
void destroy_pm(PmDev* pm);
}  // namespace hasty

struct hasty_ctx {
  int device = 0;
  int sm_count = 0;
  uint32_t flags = 0;
};

struct hasty_job {
  hasty_ctx* ctx = nullptr;
  HostScene host;
  int32_t bvh_depth = 0;
  double bvh_ms = 0, bvh_tree_ms = 0, parse_ms = 0, upload_ms = 0;
  SceneDev sd{};
  PathsDev pd{};                      // lane 0's path buffers (and the job's statistics)
  cudaStream_t stream = nullptr;      // uploads, accumulation (in batch order), read-back
  // Two render lanes: consecutive batches alternate between lane 0 (paths
  // `pd`) and lane 1 (paths `pd2`, allocated when first used), each on its
  // own stream, so that one batch's tracing overlaps the other's shading.
  // A batch's accumulation runs on `stream` after the batch (event
  // lane_done), so everything later on `stream` sees the rendering done; a
  // lane starts its next batch after the accumulation that read its
  // buffers (event lane_free). Lanes wait for `stream` (event main_ready)
  // only after it cleared state they use (statistics, counters).
  PathsDev pd2{};
  cudaStream_t lane_stream[2] = {nullptr, nullptr};
  cudaEvent_t lane_done[2] = {nullptr, nullptr}, lane_free[2] = {nullptr, nullptr}, main_ready = nullptr;
  bool lane_free_valid[2] = {false, false};
  bool lanes_wait_main = true;
  int next_lane = 0;
  hasty::PmDev* pm = nullptr;         // photon mapper (device buffers are in `allocs`)
  // host-side scene data between prepare and upload (BVH, guide tables)
  struct Prepared {
    hasty::BvhHost bvh;
    bool binary = false;
    std::vector<uint32_t> light_guide, env_guide;
    uint32_t light_guide_log2 = 0, env_guide_log2 = 0;
  };
  std::unique_ptr<Prepared> prep;
  struct Block { void* p; size_t bytes; };
  std::vector<Block> allocs;
  int64_t bytes = 0;
  double* acc[3] = {nullptr, nullptr, nullptr};
  float* est = nullptr;
  // Progressive read-back: the estimates of the captured AOVs are computed
  // on `stream` behind the passes enqueued so far into `dev`, then copied on
  // `copy_stream` into pinned host memory, so rendering enqueued afterwards
  // does not wait for the copy. Slot 0 serves hasty_job_snapshot, slot 1
  // hasty_job_write_outputs_async. Buffers are allocated on first use.
  struct Snapshot {
    float* dev = nullptr;           // 3 AOVs x npix x 3 floats
    float* host = nullptr;          // pinned
    cudaEvent_t copied = nullptr;   // recorded on copy_stream after the copies
    bool pending = false;           // a snapshot was enqueued (its copy may still run)
    uint32_t mask = 0;              // AOVs captured (1 << HASTY_AOV_*)
    int32_t samples = 0;            // passes it covers
  };
  Snapshot snap[2];
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t snap_est = nullptr;     // estimates written (recorded on `stream`)
  std::thread writer;                 // hasty_job_write_outputs_async
  int writer_rc = HASTY_OK;
  std::string writer_err;
  int64_t capacity = 0;
  int32_t samples_done = 0;
  uint64_t seed = 0;
  std::atomic<bool> stop{false};
  double kernel_ms = 0.0, trace_ms = 0.0, shade_ms = 0.0, path_ms = 0.0;
  uint64_t trace_launches = 0, kernel_launches = 0, path_launches = 0;
  // Path kernel (cache-resident scenes): slot pools of the two render lanes,
  // allocated on first use.
  PathsDev slots[2] = {};
  bool path_kernel = false;
  bool stage_timing = false;
  // (start, end, stage) with stage 0: whole batch, 1: trace, 2: shade, 3: path kernel
  struct Ev { cudaEvent_t a, b; int stage; };
  std::vector<Ev> pending_events;

  template <class T>
  T* alloc(size_t n) {
    void* p = nullptr;
    size_t b = std::max<size_t>(n, 1) * sizeof(T);
    ck(cudaMalloc(&p, b), "cudaMalloc");
    allocs.push_back({p, b});
    bytes += int64_t(b);
    return static_cast<T*>(p);
  }
  // Frees one block obtained from alloc (no-op for null or foreign pointers).
  void release(void* p) {
    if (!p) return;
    for (size_t i = 0; i < allocs.size(); ++i) {
      if (allocs[i].p == p) {
        cudaFree(p);
        bytes -= int64_t(allocs[i].bytes);
        allocs.erase(allocs.begin() + std::ptrdiff_t(i));
        return;
      }
    }
  }
  template <class T>
  T* upload(const std::vector<T>& v) {
    if (v.empty()) return nullptr;
    T* p = alloc<T>(v.size());
    ck(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, stream), "upload");
    return p;
  }
  void collect_events() {
    for (auto& e : pending_events) {
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, e.a, e.b) == cudaSuccess) {
        if (e.stage == 0) kernel_ms += ms; else if (e.stage == 1) trace_ms += ms;
        else if (e.stage == 2) shade_ms += ms; else path_ms += ms;
      }
      cudaEventDestroy(e.a); cudaEventDestroy(e.b);
    }
    pending_events.clear();
  }
  ~hasty_job() {
    if (writer.joinable()) writer.join();
    if (stream) cudaStreamSynchronize(stream);
    for (cudaStream_t s : lane_stream) if (s) cudaStreamSynchronize(s);
    if (copy_stream) cudaStreamSynchronize(copy_stream);
    collect_events();
    for (Snapshot& s : snap) {
      if (s.host) cudaFreeHost(s.host);
      if (s.copied) cudaEventDestroy(s.copied);
    }
    if (snap_est) cudaEventDestroy(snap_est);
    if (copy_stream) cudaStreamDestroy(copy_stream);
    hasty::destroy_pm(pm);
    for (const Block& b : allocs) cudaFree(b.p);
    for (int k = 0; k < 2; ++k) {
      if (lane_done[k]) cudaEventDestroy(lane_done[k]);
      if (lane_free[k]) cudaEventDestroy(lane_free[k]);
      if (lane_stream[k]) cudaStreamDestroy(lane_stream[k]);
    }
    if (main_ready) cudaEventDestroy(main_ready);
    if (stream) cudaStreamDestroy(stream);
  }
};


namespace hasty {
// Carves path-state buffers for `cap` slots out of `alloc` (no device
// work); statistics are carved too unless `stats` is given.
// The medium-stack overflow pool gets media_blocks blocks (0: one per 4
// slots, 64 at least: 80 B per slot; a scene of six nested glass shells took
// more than one per 64).
void carve_paths(PathsDev& p, int64_t cap, int n_stats, const std::function<void*(size_t)>& alloc,
                 unsigned long long* stats = nullptr, int64_t media_blocks = 0);
// carve_paths, then clears the queue counters, and the statistics when they
// were carved (api.cpp).
void alloc_paths_into(PathsDev& p, int64_t cap, int n_stats, const std::function<void*(size_t)>& alloc, cudaStream_t st,
                      unsigned long long* stats = nullptr);
// Bytes that carve_paths for `cap` slots followed by `extra_blocks` blocks of
// `extra_bytes` takes from a carving allocator whose blocks start on
// `align`-byte boundaries.
int64_t carved_bytes(int64_t cap, int n_stats, size_t align, size_t extra_blocks, size_t extra_bytes);
// Single-job path state for at least `need` paths (at most j.capacity),
// allocated on first use and grown when a call needs more.
void ensure_paths(hasty_job& j, int64_t need);
// Loads renderJob.json, builds the BVH and uploads the scene. `plain`: also
// the FP64 accumulators, estimate buffer and statistics of the single-job
// path; without it the job holds only the scene (multi-job engine use).
std::unique_ptr<hasty_job> load_job(hasty_ctx* ctx, const std::string& path, bool plain);
// The halves of load_job: host parse (no device work), then BVH build and
// upload. prepare_job_upload builds the BVH and guide tables on the host and
// returns the exact device bytes the scene upload will take.
std::unique_ptr<hasty_job> load_job_host(hasty_ctx* ctx, const std::string& path);
int64_t prepare_job_upload(hasty_job& j);
void finish_job_load(hasty_job& j, bool plain);
// Resident blocks per SM of the persistent closest-hit kernel while another
// render lane's batch runs beside it (api.cpp).
int lane_trace_blocks();
// Whether a scene is rendered by the path kernel: scenes of at most
// path_kernel_max_triangles() triangles (their BVH and triangles stay in
// L1/L2; HASTY_PATH_KERNEL_TRIS sets the bound, 0: never), unless the
// context says otherwise (HASTY_CTX_WAVEFRONT, HASTY_CTX_PATH_KERNEL).
int64_t path_kernel_max_triangles();
bool use_path_kernel(const hasty_ctx* ctx, const SceneDev& sc);
// Slot pool of the path kernel (path_slots() slots; its statistics are `stats`).
void alloc_path_slots(PathsDev& p, const std::function<void*(size_t)>& alloc, unsigned long long* stats);
}  // namespace hasty
