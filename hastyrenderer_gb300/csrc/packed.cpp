// Packed multi-job batches (packed.h) and the batching entry point's packed
// mode.
#include "packed.h"

#include <algorithm>
#include <chrono>
#include <cstring>

#include "engine.h"

namespace hasty {

void* PackedLanes::alloc(size_t b) {
  void* p = nullptr;
  ck(cudaMalloc(&p, std::max<size_t>(b, 16)), "cudaMalloc (packed lanes)");
  allocs.push_back(p);
  bytes += int64_t(b);
  return p;
}

void PackedLanes::init(hasty_ctx* c, int lanes, int64_t paths) {
  ctx = c;
  ck(cudaSetDevice(ctx->device), "cudaSetDevice");
  if (lanes < 1 || lanes > kMaxLanes) throw ApiError{HASTY_ERR_ARG, "render lanes must be 1.." + std::to_string(kMaxLanes)};
  if (paths < 1 || paths > int64_t(INT32_MAX) / 2) throw ApiError{HASTY_ERR_ARG, "bad paths-per-lane value"};
  n_lanes = lanes;
  lane_paths = paths;
  bvh_kind = (ctx->flags & HASTY_CTX_BINARY_BVH) ? 0 : 1;
  ck(cudaStreamCreateWithFlags(&acc_stream, cudaStreamNonBlocking), "stream");
  ck(cudaEventCreateWithFlags(&acc_ready, cudaEventDisableTiming), "event");
  stats = static_cast<unsigned long long*>(alloc(sizeof(unsigned long long) * ST_COUNT));
  ck(cudaMemsetAsync(stats, 0, sizeof(unsigned long long) * ST_COUNT, acc_stream), "memset stats");
  for (int k = 0; k < n_lanes; ++k) {
    ck(cudaStreamCreateWithFlags(&lane_stream[k], cudaStreamNonBlocking), "stream");
    ck(cudaEventCreateWithFlags(&lane_done[k], cudaEventDisableTiming), "event");
    ck(cudaEventCreateWithFlags(&lane_free[k], cudaEventDisableTiming), "event");
    alloc_paths_into(pd[k], lane_paths, ST_COUNT, [&](size_t b) { return alloc(b); }, acc_stream, stats);
    // the path kernel's slot pool, so the lanes' footprint is fixed from the start
    alloc_path_slots(slots[k], [&](size_t b) { return alloc(b); }, stats);
    ck(cudaMemsetAsync(slots[k].counts, 0, sizeof(uint32_t) * kCountSlots, acc_stream), "memset counts");
  }
  wait_for(acc_stream);
}

void PackedLanes::wait_for(cudaStream_t s) {
  ck(cudaEventRecord(acc_ready, s), "event");
  for (int k = 0; k < n_lanes; ++k) ck(cudaStreamWaitEvent(lane_stream[k], acc_ready, 0), "lane wait");
  if (s != acc_stream) ck(cudaStreamWaitEvent(acc_stream, acc_ready, 0), "wait");
}

void PackedLanes::launch(const std::vector<PackedJob>& jobs, const std::vector<PackedChunk>& chunks, bool overlap,
                         cudaEvent_t start) {
  if (chunks.empty()) return;
  if (chunks.size() > size_t(kMaxChunks)) throw ApiError{HASTY_ERR_ARG, "too many chunks in one batch"};
  // Tables as kernel parameters (the launch copies them).
  static thread_local ChunkTable ct;
  static thread_local TraceTable tt;
  std::memset(&ct, 0, sizeof(ct));
  std::memset(&tt, 0, sizeof(tt));
  int64_t slot = 0;
  int max_depth = 0;
  for (size_t c = 0; c < chunks.size(); ++c) {
    const PackedChunk& ch = chunks[c];
    const PackedJob& j = jobs[size_t(ch.job)];
    ChunkDev& d = ct.c[c];
    d.sc = j.sc;
    d.seed = j.seed;
    d.first_slot = int32_t(slot);
    d.pass_base = ch.pass_base;
    d.npix = j.npix;
    d.n_passes = ch.n_passes;
    tt.c[c].nodes = j.sc.nodes;
    tt.c[c].tris = j.sc.isect_tris;
    tt.c[c].nee_first_hit = j.sc.n_light_tris == 0 ? 1 : 0;
    tt.c[c].n_nodes = j.sc.n_nodes;
    tt.c[c].n_tris = j.sc.n_tris;
    slot += int64_t(ch.n_passes) * j.npix;
    max_depth = std::max(max_depth, j.sc.max_depth);
  }
  if (slot > lane_paths) throw ApiError{HASTY_ERR_ARG, "batch does not fit a render lane"};
  ct.n = int32_t(chunks.size());
  ct.n_paths = int32_t(slot);
  tt.n = ct.n;
  tt.bvh_kind = bvh_kind;
  const int lane = next_lane;
  next_lane = (next_lane + 1) % n_lanes;
  PathsDev& p = pd[lane];
  cudaStream_t ls = lane_stream[lane];
  if (lane_free_valid[lane]) ck(cudaStreamWaitEvent(ls, lane_free[lane], 0), "lane wait");
  if (start) ck(cudaEventRecord(start, ls), "event");
  const int trace_cap =
      overlap && n_lanes > 1 ? (trace_blocks_per_sm > 0 ? trace_blocks_per_sm : lane_trace_blocks()) : 0;
  const int n_paths = ct.n_paths;
  const bool path_kernel = jobs[size_t(chunks[0].job)].path_kernel;
  if (path_kernel) {
    launch_paths_packed(ct, bvh_kind, slots[lane], p, ls);
  } else {
    launch_raygen_packed(ct, p, ls);
    for (int bounce = 0; bounce < max_depth; ++bounce) {
      const int q = bounce & 1;
      launch_trace_packed(tt, p, q, 2 * n_paths, ls, trace_cap);
      launch_shade_packed(ct, p, q, n_paths, ls, resolve_threads, sample_threads);
    }
  }
  ck(cudaEventRecord(lane_done[lane], ls), "lane event");
  ck(cudaStreamWaitEvent(acc_stream, lane_done[lane], 0), "lane wait");
  for (size_t c = 0; c < chunks.size(); ++c) {
    const PackedJob& j = jobs[size_t(chunks[c].job)];
    launch_accumulate_range(p, ct.c[c].first_slot, j.npix, chunks[c].n_passes, j.acc[0], j.acc[1], j.acc[2], acc_stream);
  }
  ck(cudaGetLastError(), "packed batch launch");
  ck(cudaEventRecord(lane_free[lane], acc_stream), "lane event");
  lane_free_valid[lane] = true;
  ++batches;
  launches += (path_kernel ? 1u : uint64_t(1 + 3 * max_depth)) + chunks.size();
}

void PackedLanes::read_stats(unsigned long long* out) {
  ck(cudaMemcpyAsync(out, stats, sizeof(unsigned long long) * ST_COUNT, cudaMemcpyDeviceToHost, acc_stream), "stats");
  ck(cudaStreamSynchronize(acc_stream), "stats");
}

PackedLanes::~PackedLanes() {
  for (int k = 0; k < n_lanes; ++k) if (lane_stream[k]) cudaStreamSynchronize(lane_stream[k]);
  if (acc_stream) cudaStreamSynchronize(acc_stream);
  for (void* p : allocs) cudaFree(p);
  for (int k = 0; k < n_lanes; ++k) {
    if (lane_done[k]) cudaEventDestroy(lane_done[k]);
    if (lane_free[k]) cudaEventDestroy(lane_free[k]);
    if (lane_stream[k]) cudaStreamDestroy(lane_stream[k]);
  }
  if (acc_ready) cudaEventDestroy(acc_ready);
  if (acc_stream) cudaStreamDestroy(acc_stream);
}

std::vector<PackedChunk> pack_batch(const std::vector<PackedJob>& jobs, const std::vector<int>& order,
                                    std::vector<uint32_t>& pass_base, std::vector<int32_t>& left, int64_t slots,
                                    int64_t job_samples) {
  std::vector<PackedChunk> out;
  int64_t used = 0;
  for (int j : order) {
    if (out.size() >= size_t(kMaxChunks)) break;
    if (left[size_t(j)] <= 0) continue;
    const int64_t npix = jobs[size_t(j)].npix;
    const int64_t fit = (slots - used) / npix;
    if (fit <= 0) continue;
    int64_t k = std::min<int64_t>(fit, left[size_t(j)]);
    if (job_samples > 0) k = std::min<int64_t>(k, std::max<int64_t>(1, job_samples / npix));
    out.push_back({j, pass_base[size_t(j)], int32_t(k)});
    pass_base[size_t(j)] += uint32_t(k);
    left[size_t(j)] -= int32_t(k);
    used += k * npix;
  }
  return out;
}

std::vector<int> class_order(const std::vector<PackedJob>& jobs, const std::vector<int>& order, int cls) {
  std::vector<int> out;
  for (int j : order) if (kernel_class(jobs[size_t(j)]) == cls) out.push_back(j);
  return out;
}

std::vector<PackedChunk> pack_next(const std::vector<PackedJob>& jobs, const std::vector<int>& order,
                                   std::vector<uint32_t>& pass_base, std::vector<int32_t>& left, int64_t slots,
                                   int64_t job_samples, int& turn) {
  for (int attempt = 0; attempt < kKernelClasses; ++attempt) {
    const int cls = ((turn % kKernelClasses) + kKernelClasses) % kKernelClasses;
    turn = cls + 1;
    std::vector<PackedChunk> c = pack_batch(jobs, class_order(jobs, order, cls), pass_base, left, slots, job_samples);
    if (!c.empty()) return c;
  }
  return {};
}

int64_t packed_lane_paths(int64_t requested, int64_t largest_frame) {
  int64_t p = requested > 0 ? requested : (int64_t(1) << 24);
  return std::max(p, largest_frame);
}

}  // namespace hasty

using namespace hasty;

namespace {

// Packed mode of hasty_batch_render: every job's passes in job order, packed
// into batches that alternate over the render lanes.
void batch_render_packed(hasty_ctx* ctx, hasty_job** jobs, const int32_t* passes, size_t n_jobs,
                         const hasty_batch_config* cfg, hasty_batch_stats* out) {
  auto t0 = std::chrono::steady_clock::now();
  std::vector<PackedJob> pj(n_jobs);
  std::vector<uint32_t> base(n_jobs);
  std::vector<int32_t> left(n_jobs);
  std::vector<int> order;
  int64_t largest = 1;
  uint64_t samples = 0;
  for (size_t i = 0; i < n_jobs; ++i) {
    hasty_job* j = jobs[i];
    pj[i].sc = j->sd;
    pj[i].seed = j->seed;
    for (int a = 0; a < 3; ++a) pj[i].acc[a] = j->acc[a];
    pj[i].npix = j->sd.width * j->sd.height;
    pj[i].path_kernel = j->path_kernel;
    pj[i].simple_trace = simple_trace_bvh(j->sd);
    base[i] = uint32_t(j->samples_done);
    left[i] = passes[i];
    largest = std::max<int64_t>(largest, pj[i].npix);
    samples += uint64_t(pj[i].npix) * uint64_t(passes[i]);
    if (passes[i] > 0) order.push_back(int(i));
  }
  const int n_lanes = (cfg && cfg->lanes > 0) ? cfg->lanes : 2;
  const int64_t lane_paths = packed_lane_paths(cfg ? cfg->paths_in_flight : 0, largest);
  PackedLanes L;
  L.init(ctx, n_lanes, lane_paths);
  if (cfg) {
    L.resolve_threads = cfg->resolve_threads;
    L.sample_threads = cfg->sample_threads;
    L.trace_blocks_per_sm = cfg->trace_blocks_per_sm;
  }
  cudaEvent_t a = nullptr, b = nullptr;
  ck(cudaEventCreate(&a), "event");
  ck(cudaEventCreate(&b), "event");
  ck(cudaEventRecord(a, L.acc_stream), "event");
  L.wait_for(L.acc_stream);
  int turn = 0;
  for (;;) {
    std::vector<PackedChunk> chunks = pack_next(pj, order, base, left, lane_paths, 0, turn);
    if (chunks.empty()) break;
    bool more = false;
    for (int i : order) more = more || left[size_t(i)] > 0;
    L.launch(pj, chunks, more || L.batches > 0);
  }
  ck(cudaEventRecord(b, L.acc_stream), "event");
  ck(cudaEventSynchronize(b), "batch");
  float ms = 0.f;
  cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  unsigned long long st[ST_COUNT];
  L.read_stats(st);
  for (size_t i = 0; i < n_jobs; ++i) jobs[i]->samples_done += passes[i];
  if (out) {
    std::memset(out, 0, sizeof(*out));
    out->device_ms = ms;
    out->wall_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    out->samples = samples;
    out->rays = st[ST_RAYS];
    out->shaded = st[ST_SHADED];
    out->nan_samples = st[ST_NAN];
    out->iterations = L.batches;
    out->paths_in_flight = lane_paths * n_lanes;
    out->engine_bytes = L.bytes;
    out->kernel_launches = L.launches;
    out->media_overflow = st[ST_MEDIA_OVERFLOW];
  }
}

}  // namespace

extern "C" int hasty_debug_pack(const int32_t* npix, const int32_t* passes, const int32_t* cls, size_t n_jobs,
                                int64_t slots, int64_t job_samples, int32_t* out, size_t max_chunks, size_t* n_out) {
  return guarded([&] {
    if (!n_out || (n_jobs && (!npix || !passes || !cls)) || (max_chunks && !out) || slots <= 0)
      throw ApiError{HASTY_ERR_ARG, "bad argument"};
    std::vector<PackedJob> pj(n_jobs);
    std::vector<uint32_t> base(n_jobs, 0u);
    std::vector<int32_t> left(n_jobs);
    std::vector<int> order;
    for (size_t i = 0; i < n_jobs; ++i) {
      if (npix[i] <= 0 || npix[i] > slots || passes[i] < 0 || cls[i] < 0 || cls[i] >= kKernelClasses)
        throw ApiError{HASTY_ERR_ARG, "bad job"};
      pj[i].npix = npix[i];
      pj[i].path_kernel = cls[i] == 2;
      pj[i].simple_trace = cls[i] == 1;
      left[i] = passes[i];
      if (passes[i] > 0) order.push_back(int(i));
    }
    size_t n = 0;
    int turn = 0;
    for (int32_t batch = 0;; ++batch) {
      const std::vector<PackedChunk> chunks = pack_next(pj, order, base, left, slots, job_samples, turn);
      if (chunks.empty()) break;
      for (const PackedChunk& c : chunks) {
        if (n < max_chunks) {
          out[4 * n] = batch;
          out[4 * n + 1] = c.job;
          out[4 * n + 2] = int32_t(c.pass_base);
          out[4 * n + 3] = c.n_passes;
        }
        ++n;
      }
    }
    *n_out = n;
    return HASTY_OK;
  });
}

extern "C" int hasty_batch_render(hasty_ctx* ctx, hasty_job** jobs, const int32_t* passes, size_t n_jobs,
                                  const hasty_batch_config* cfg, hasty_batch_stats* out) {
  return guarded([&] {
    if (!ctx || (n_jobs && (!jobs || !passes))) throw ApiError{HASTY_ERR_ARG, "null argument"};
    const int mode = cfg ? cfg->mode : HASTY_BATCH_PACKED;
    if (mode != HASTY_BATCH_PACKED && mode != HASTY_BATCH_REGEN) throw ApiError{HASTY_ERR_ARG, "unknown batch mode"};
    for (size_t i = 0; i < n_jobs; ++i) {
      if (!jobs[i] || passes[i] < 0) throw ApiError{HASTY_ERR_ARG, "bad job or pass count"};
      if (jobs[i]->ctx != ctx) throw ApiError{HASTY_ERR_ARG, "job belongs to another context"};
      if (jobs[i]->sd.max_depth <= 0) throw ApiError{HASTY_ERR_ARG, "max_depth must be positive for batching"};
      if (!jobs[i]->acc[0]) throw ApiError{HASTY_ERR_ARG, "job has no accumulators"};
      ck(cudaStreamSynchronize(jobs[i]->stream), "job sync");
      for (cudaStream_t s : jobs[i]->lane_stream) if (s) ck(cudaStreamSynchronize(s), "job sync");
    }
    if (mode == HASTY_BATCH_REGEN) {
      const int rc = batch_render_regen(ctx, jobs, passes, n_jobs, cfg, out);
      if (rc != HASTY_OK) throw ApiError{rc, g_error};
      return HASTY_OK;
    }
    ck(cudaSetDevice(ctx->device), "cudaSetDevice");
    batch_render_packed(ctx, jobs, passes, n_jobs, cfg, out);
    return HASTY_OK;
  });
}
