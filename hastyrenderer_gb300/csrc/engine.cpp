// Multi-job engine (engine.h) and batching: hasty_batch_render renders many
// resident jobs in one persistent wavefront run.
#include "engine.h"

#include <algorithm>
#include <chrono>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <vector>

namespace hasty {

void* Engine::alloc(size_t b) {
  void* p = nullptr;
  ck(cudaMalloc(&p, std::max<size_t>(b, 16)), "cudaMalloc (engine)");
  allocs.push_back(p);
  bytes += int64_t(b);
  return p;
}

void Engine::init(hasty_ctx* c, int64_t capacity, int slots, uint32_t segments, uint32_t regen_below, uint32_t max_iter) {
  ctx = c;
  ck(cudaSetDevice(ctx->device), "cudaSetDevice");
  if (capacity < 1 || capacity > int64_t(INT32_MAX) / 2) throw ApiError{HASTY_ERR_ARG, "bad paths-in-flight value"};
  if (slots < 1) throw ApiError{HASTY_ERR_ARG, "engine needs at least one job slot"};
  ck(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "stream");
  cap = (capacity + kGroup - 1) / kGroup * kGroup;
  job_slots = slots;
  seg_cap = 64;
  while (seg_cap < segments) {
    if (seg_cap >= (1u << 30)) throw ApiError{HASTY_ERR_ARG, "too many segments"};
    seg_cap <<= 1;
  }
  alloc_paths_into(pd, cap, MS_COUNT, [&](size_t b) { return alloc(b); }, stream);
  // Slots are refilled without a batch boundary to return overflow blocks
  // at, so the engine keeps the medium stack to its first kMaxMedia entries.
  pd.med_pool_blocks = 0;
  d_jobs = static_cast<JobDev*>(alloc(sizeof(JobDev) * size_t(job_slots)));
  d_segs = static_cast<SegDev*>(alloc(sizeof(SegDev) * size_t(seg_cap)));
  d_window = static_cast<uint32_t*>(alloc(sizeof(uint32_t) * 2));
  d_done = static_cast<unsigned long long*>(alloc(sizeof(unsigned long long) * size_t(job_slots)));
  md.jobs = d_jobs;
  md.segs = d_segs;
  md.seg_mask = seg_cap - 1u;
  md.seg_window = d_window;
  md.slot_meta = static_cast<uint4*>(alloc(sizeof(uint4) * size_t(cap)));
  md.free_slots = static_cast<int32_t*>(alloc(sizeof(int32_t) * size_t(cap)));
  md.flags = static_cast<uint8_t*>(alloc(size_t(cap)));
  md.block_sums = static_cast<uint32_t*>(alloc(sizeof(uint32_t) * 3 * size_t(compact_blocks(int(cap)))));
  md.free_count = static_cast<uint32_t*>(alloc(sizeof(uint32_t)));
  md.next_sample = static_cast<unsigned long long*>(alloc(sizeof(unsigned long long)));
  md.total_samples = static_cast<unsigned long long*>(alloc(sizeof(unsigned long long)));
  md.regen_base = static_cast<unsigned long long*>(alloc(sizeof(unsigned long long)));
  md.ctl = static_cast<uint32_t*>(alloc(sizeof(uint32_t) * kCtlWords));
  md.regen_below = regen_below;
  md.max_iter = max_iter;
  ck(cudaMemsetAsync(d_window, 0, sizeof(uint32_t) * 2, stream), "memset");
  ck(cudaMemsetAsync(d_done, 0, sizeof(unsigned long long) * size_t(job_slots), stream), "memset");
  ck(cudaMemsetAsync(d_jobs, 0, sizeof(JobDev) * size_t(job_slots), stream), "memset");
  ck(cudaMemsetAsync(md.next_sample, 0, sizeof(unsigned long long), stream), "memset");
  ck(cudaMemsetAsync(md.total_samples, 0, sizeof(unsigned long long), stream), "memset");
  launch_multi_init(pd, md, int(cap), stream);
  ck(cudaGetLastError(), "engine init");
  const char* mode = std::getenv("HASTY_ENGINE_LAUNCH");
  use_graph = !(mode && std::strcmp(mode, "stream") == 0);
  if (use_graph) build_graph();
  ck(cudaStreamSynchronize(stream), "engine init");
}

void Engine::build_graph() {
  ck(cudaGraphCreate(&graph, 0), "cudaGraphCreate");
  cudaGraphConditionalHandle h;
  ck(cudaGraphConditionalHandleCreate(&h, graph, 1, cudaGraphCondAssignDefault), "conditional handle");
  cudaGraphNodeParams np = {};
  np.type = cudaGraphNodeTypeConditional;
  np.conditional.handle = h;
  np.conditional.type = cudaGraphCondTypeWhile;
  np.conditional.size = 1;
  cudaGraphNode_t node;
  ck(cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &np), "add conditional node");
  cudaGraph_t body = np.conditional.phGraph_out[0];
  ck(cudaStreamBeginCaptureToGraph(stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed), "begin capture");
  launch_multi_iteration(pd, md, int(cap), (ctx->flags & HASTY_CTX_BINARY_BVH) ? 0 : 1, (unsigned long long)h, 1, stream,
                         trace_blocks_per_sm);
  cudaGraph_t captured = nullptr;
  ck(cudaStreamEndCapture(stream, &captured), "end capture");
  ck(cudaGraphInstantiate(&exec, graph, 0), "cudaGraphInstantiate");
}

void Engine::set_job(int slot, const JobDev& j) {
  if (slot < 0 || slot >= job_slots) throw ApiError{HASTY_ERR_ARG, "job slot out of range"};
  JobDev e = j;
  e.done = d_done + slot;
  ck(cudaMemcpyAsync(d_jobs + slot, &e, sizeof(JobDev), cudaMemcpyHostToDevice, stream), "job entry");
  ck(cudaMemsetAsync(d_done + slot, 0, sizeof(unsigned long long), stream), "done counter");
}

void Engine::append(int slot, uint32_t pass, uint32_t npix) {
  if (free_segments() == 0) throw ApiError{HASTY_ERR_ARG, "engine segment ring is full"};
  SegDev s;
  s.begin = total;
  s.job = slot;
  s.pass = pass;
  staged.push_back(s);
  spans.emplace_back(total, npix);
  total += npix;
  ++seg_hi;
}

void Engine::publish() {
  // staged segments occupy logical indices [seg_hi - staged.size(), seg_hi)
  uint32_t first = seg_hi - uint32_t(staged.size());
  size_t k = 0;
  while (k < staged.size()) {
    uint32_t phys = (first + uint32_t(k)) & (seg_cap - 1u);
    size_t run = std::min<size_t>(staged.size() - k, size_t(seg_cap - phys));
    ck(cudaMemcpyAsync(d_segs + phys, staged.data() + k, sizeof(SegDev) * run, cudaMemcpyHostToDevice, stream), "segments");
    k += run;
  }
  staged.clear();
  uint32_t window[2] = {seg_lo, seg_hi};
  ck(cudaMemcpyAsync(d_window, window, sizeof(window), cudaMemcpyHostToDevice, stream), "segment window");
  unsigned long long t = total;
  ck(cudaMemcpyAsync(md.total_samples, &t, sizeof(t), cudaMemcpyHostToDevice, stream), "total");
  // the sources are host stack/heap memory: make the copies complete before they go out of scope
  ck(cudaStreamSynchronize(stream), "publish");
}

bool Engine::run_wave(uint32_t n_iter, bool* bound_hit) {
  launch_wave(n_iter);
  return finish_wave(bound_hit);
}

void Engine::launch_wave(uint32_t n_iter) {
  if (!staged.empty()) publish();
  wave_end = iterations + std::max<uint32_t>(n_iter, 1u);
  ck(cudaMemcpyAsync(&md.ctl[7], &wave_end, sizeof(wave_end), cudaMemcpyHostToDevice, stream), "wave end");
  if (use_graph) {
    ck(cudaGraphLaunch(exec, stream), "cudaGraphLaunch");
    return;
  }
  // the loop condition of the graph's while node, evaluated on the host
  for (;;) {
    launch_multi_iteration(pd, md, int(cap), (ctx->flags & HASTY_CTX_BINARY_BVH) ? 0 : 1, 0ull, 0, stream,
                           trace_blocks_per_sm);
    ck(cudaGetLastError(), "engine iteration");
    uint32_t ctl[8];
    unsigned long long ns = 0;
    uint32_t counts[4];
    ck(cudaMemcpyAsync(ctl, md.ctl, sizeof(ctl), cudaMemcpyDeviceToHost, stream), "ctl");
    ck(cudaMemcpyAsync(&ns, md.next_sample, sizeof(ns), cudaMemcpyDeviceToHost, stream), "next");
    ck(cudaMemcpyAsync(counts, pd.counts, sizeof(counts), cudaMemcpyDeviceToHost, stream), "counts");
    ck(cudaStreamSynchronize(stream), "wave");
    bool more = counts[ctl[0] & 1u] > 0 || ns < total;
    if (!more || ctl[6] != 0 || ctl[5] >= wave_end) break;
  }
}

bool Engine::finish_wave(bool* bound_hit) {
  uint32_t ctl[8];
  unsigned long long ns = 0;
  uint32_t counts[4];
  ck(cudaMemcpyAsync(ctl, md.ctl, sizeof(ctl), cudaMemcpyDeviceToHost, stream), "ctl");
  ck(cudaMemcpyAsync(&ns, md.next_sample, sizeof(ns), cudaMemcpyDeviceToHost, stream), "next");
  ck(cudaMemcpyAsync(counts, pd.counts, sizeof(counts), cudaMemcpyDeviceToHost, stream), "counts");
  ck(cudaStreamSynchronize(stream), "wave");
  iterations = ctl[5];
  if (bound_hit) *bound_hit = ctl[6] != 0;
  next = ns;
  live = counts[ctl[0] & 1u];
  // segments wholly issued are no longer looked up
  bool moved = false;
  while (!spans.empty() && spans.front().first + spans.front().second <= next) {
    spans.pop_front();
    ++seg_lo;
    moved = true;
  }
  if (moved) {
    uint32_t lo = seg_lo;
    ck(cudaMemcpyAsync(d_window, &lo, sizeof(lo), cudaMemcpyHostToDevice, stream), "segment window");
    ck(cudaStreamSynchronize(stream), "segment window");
  }
  return busy();
}

void Engine::read_done(std::vector<unsigned long long>& out) {
  out.resize(size_t(job_slots));
  ck(cudaMemcpyAsync(out.data(), d_done, sizeof(unsigned long long) * out.size(), cudaMemcpyDeviceToHost, stream), "done");
  ck(cudaStreamSynchronize(stream), "done");
}

void Engine::stats(unsigned long long* out) {
  ck(cudaMemcpyAsync(out, pd.stats, sizeof(unsigned long long) * MS_COUNT, cudaMemcpyDeviceToHost, stream), "stats");
  ck(cudaStreamSynchronize(stream), "stats");
}

Engine::~Engine() {
  if (stream) cudaStreamSynchronize(stream);
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  for (void* p : allocs) cudaFree(p);
  if (stream) cudaStreamDestroy(stream);
}

int64_t engine_pool_size(int64_t requested) { return requested > 0 ? requested : (int64_t(1) << 22); }

uint32_t engine_lanes(int64_t cap, uint32_t npix) {
  if (const char* v = std::getenv("HASTY_ENGINE_LANES")) {   // fixed lane count (tuning)
    long l = std::strtol(v, nullptr, 10);
    if (l >= 1 && l <= 64) return uint32_t(l);
  }
  int64_t l = cap / (256 * int64_t(std::max<uint32_t>(npix, 1u)));
  return uint32_t(std::max<int64_t>(1, std::min<int64_t>(16, l)));
}

// Resident closest-hit blocks per SM for an engine that shares the GPU with
// another (the plain path's lanes use the same bound).
constexpr int kSharedTraceBlocksPerSM = 5;

uint32_t engine_regen_threshold(float fraction, int64_t cap) {
  float f = fraction > 0.f ? fraction : 0.9f;
  if (f >= 1.0f) return uint32_t(cap) + 1u;
  return uint32_t(double(cap) * double(f));
}

}  // namespace hasty

// Regeneration mode of hasty_batch_render (the arguments are checked and the
// jobs' streams synchronised by the caller).
int hasty::batch_render_regen(hasty_ctx* ctx, hasty_job** jobs, const int32_t* passes, size_t n_jobs,
                              const hasty_batch_config* cfg, hasty_batch_stats* out) {
  return guarded([&] {
    uint64_t n_segments = 0;
    for (size_t i = 0; i < n_jobs; ++i) n_segments += uint64_t(passes[i]);
    if (n_segments >= (uint64_t(1) << 30)) throw ApiError{HASTY_ERR_ARG, "too many passes in one batch"};
    auto t0 = std::chrono::steady_clock::now();
    // Two engines on two streams, each with half the pool, take alternate
    // passes of every job, so that one engine's tracing overlaps the other's
    // shading. Each job's fixed-point sums have 2 x L lanes (L per engine);
    // the integer fold at the end makes the result the one engine's.
    int n_eng = n_segments >= 2 ? 2 : 1;
    if (const char* v = std::getenv("HASTY_BATCH_ENGINES")) n_eng = std::atoi(v) == 1 ? 1 : n_eng;   // tuning
    int64_t cap = engine_pool_size(cfg ? cfg->paths_in_flight : 0);
    const int64_t cap_each = std::max<int64_t>(kGroup, cap / n_eng);
    uint32_t max_iter = (cfg && cfg->max_iterations > 0) ? uint32_t(cfg->max_iterations) : 50000000u;
    Engine engines[2];
    for (int k = 0; k < n_eng; ++k) {
      engines[k].trace_blocks_per_sm = n_eng > 1 ? kSharedTraceBlocksPerSM : 0;
      engines[k].init(ctx, cap_each, int(std::max<size_t>(n_jobs, 1)),
                      uint32_t(std::max<uint64_t>(n_segments / uint64_t(n_eng) + 1, 1)),
                      engine_regen_threshold(cfg ? cfg->regen_fraction : 0.f, cap_each), max_iter);
    }
    Engine& e = engines[0];
    std::vector<unsigned long long*> accs(n_jobs);
    std::vector<uint32_t> lanes(n_jobs, 1u);
    for (size_t i = 0; i < n_jobs; ++i) {
      hasty_job* j = jobs[i];
      uint32_t npix = uint32_t(j->sd.width) * uint32_t(j->sd.height);
      lanes[i] = engine_lanes(cap_each, npix);
      const size_t lane_words = 9 * size_t(npix);
      const size_t acc_bytes = sizeof(unsigned long long) * lane_words * lanes[i] * size_t(n_eng);
      accs[i] = static_cast<unsigned long long*>(e.alloc(acc_bytes));
      ck(cudaMemsetAsync(accs[i], 0, acc_bytes, e.stream), "memset acc");
      for (int k = 0; k < n_eng; ++k) {
        JobDev d;
        std::memset(&d, 0, sizeof(d));
        d.sc = j->sd;
        d.acc = accs[i] + lane_words * lanes[i] * size_t(k);
        d.seed = j->seed;
        d.npix = npix;
        d.lanes = lanes[i];
        engines[k].set_job(int(i), d);
      }
      // jobs in order, each job's passes in order, alternating engines
      for (int32_t p = 0; p < passes[i]; ++p) engines[p % n_eng].append(int(i), uint32_t(j->samples_done + p), npix);
    }
    ck(cudaStreamSynchronize(e.stream), "memset acc");   // the other engine's kernels add into these sums
    for (int k = 0; k < n_eng; ++k) engines[k].publish();
    cudaEvent_t a, b;
    ck(cudaEventCreate(&a), "event"); ck(cudaEventCreate(&b), "event");
    ck(cudaEventRecord(a, e.stream), "event");
    for (int k = 1; k < n_eng; ++k) ck(cudaStreamWaitEvent(engines[k].stream, a, 0), "event wait");
    cudaEvent_t ends[2] = {b, nullptr};
    if (n_eng > 1) ck(cudaEventCreate(&ends[1]), "event");
    for (int k = 0; k < n_eng; ++k) {
      engines[k].launch_wave(max_iter);
      ck(cudaEventRecord(ends[k], engines[k].stream), "event");
    }
    bool bound = false;
    for (int k = 0; k < n_eng; ++k) {
      bool bk = false;
      engines[k].finish_wave(&bk);
      bound = bound || bk;
    }
    float ms = 0.f;   // device time: from the common start to the last engine's end
    for (int k = 0; k < n_eng; ++k) {
      float mk = 0.f;
      ck(cudaEventSynchronize(ends[k]), "event");
      cudaEventElapsedTime(&mk, a, ends[k]);
      ms = std::max(ms, mk);
    }
    cudaEventDestroy(a); cudaEventDestroy(b);
    if (ends[1]) cudaEventDestroy(ends[1]);
    if (bound) throw ApiError{HASTY_ERR_CUDA, "batch stopped at its iteration bound"};
    // fold the fixed-point sums into each job's FP64 accumulators
    for (size_t i = 0; i < n_jobs; ++i) {
      hasty_job* j = jobs[i];
      launch_fold_lanes(accs[i], j->sd.width * j->sd.height, int(lanes[i]) * n_eng, e.stream);
      launch_fixed_to_double(accs[i], j->sd.width * j->sd.height, j->acc[0], j->acc[1], j->acc[2], e.stream);
      j->samples_done += passes[i];
    }
    ck(cudaGetLastError(), "fold");
    unsigned long long st[MS_COUNT] = {};
    for (int k = 0; k < n_eng; ++k) {
      unsigned long long sk[MS_COUNT];
      engines[k].stats(sk);
      for (int c = 0; c < MS_COUNT; ++c) st[c] += sk[c];
    }
    if (out) {
      std::memset(out, 0, sizeof(*out));
      out->device_ms = ms;
      out->wall_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
      for (int k = 0; k < n_eng; ++k) {
        out->samples += engines[k].total;
        out->iterations = std::max<uint64_t>(out->iterations, engines[k].iterations);
        out->paths_in_flight += engines[k].cap;
        out->engine_bytes += engines[k].bytes;
      }
      out->rays = st[MS_RAYS]; out->shaded = st[MS_SHADED]; out->nan_samples = st[MS_NAN];
      out->saturated = st[MS_SATURATED];
      out->media_overflow = st[MS_MEDIA_OVERFLOW];
    }
    return HASTY_OK;
  });
}
