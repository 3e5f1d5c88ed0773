// Multi-job engine host side: batching (hasty_batch_render) and serving
// (hasty_server_*). Jobs stay resident (scene, BVH and accumulators are the
// jobs' own device buffers); the engine owns one pool of path slots and a
// CUDA graph whose conditional while-node repeats one iteration
// (regenerate, trace, shade, condition) on the device until every issued
// sample is finished or the wave's iteration budget is spent.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "job.h"

namespace hasty {

struct Engine {
  hasty_ctx* ctx = nullptr;
  cudaStream_t stream = nullptr;
  std::vector<void*> allocs;
  int64_t bytes = 0;
  PathsDev pd{};
  MultiDev md{};
  int64_t cap = 0;
  int max_jobs = 0;
  JobDev* d_jobs = nullptr;
  int32_t* d_njobs = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  uint32_t iterations = 0;

  void* alloc(size_t b) {
    void* p = nullptr;
    ck(cudaMalloc(&p, std::max<size_t>(b, 16)), "cudaMalloc (engine)");
    allocs.push_back(p);
    bytes += int64_t(b);
    return p;
  }

  void init(hasty_ctx* c, int64_t capacity, int jobs_max, uint32_t regen_below, uint32_t max_iter) {
    ctx = c;
    ck(cudaSetDevice(ctx->device), "cudaSetDevice");
    ck(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "stream");
    cap = capacity;
    max_jobs = jobs_max;
    alloc_paths_into(pd, cap, MS_COUNT, [&](size_t b) { return alloc(b); }, stream);
    d_jobs = static_cast<JobDev*>(alloc(sizeof(JobDev) * size_t(max_jobs)));
    d_njobs = static_cast<int32_t*>(alloc(sizeof(int32_t)));
    md.jobs = d_jobs;
    md.n_jobs = d_njobs;
    md.slot_job = static_cast<int32_t*>(alloc(sizeof(int32_t) * size_t(cap)));
    md.slot_sample = static_cast<uint32_t*>(alloc(sizeof(uint32_t) * size_t(cap)));
    md.free_slots = static_cast<int32_t*>(alloc(sizeof(int32_t) * size_t(cap)));
    md.free_count = static_cast<uint32_t*>(alloc(sizeof(uint32_t)));
    md.next_sample = static_cast<unsigned long long*>(alloc(sizeof(unsigned long long)));
    md.total_samples = static_cast<unsigned long long*>(alloc(sizeof(unsigned long long)));
    md.regen_base = static_cast<unsigned long long*>(alloc(sizeof(unsigned long long)));
    md.ctl = static_cast<uint32_t*>(alloc(sizeof(uint32_t) * 8));
    md.regen_below = regen_below;
    md.max_iter = max_iter;
    ck(cudaMemsetAsync(d_njobs, 0, sizeof(int32_t), stream), "memset");
    ck(cudaMemsetAsync(md.next_sample, 0, sizeof(unsigned long long), stream), "memset");
    ck(cudaMemsetAsync(md.total_samples, 0, sizeof(unsigned long long), stream), "memset");
    launch_multi_init(pd, md, int(cap), stream);
    ck(cudaGetLastError(), "engine init");
    build_graph();
    ck(cudaStreamSynchronize(stream), "engine init");
  }

  void build_graph() {
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
    launch_multi_iteration(pd, md, int(cap), (unsigned long long)h, 1, stream);
    cudaGraph_t captured = nullptr;
    ck(cudaStreamEndCapture(stream, &captured), "end capture");
    ck(cudaGraphInstantiate(&exec, graph, 0), "cudaGraphInstantiate");
  }

  // Replace the device job table (jobs in sample order) and the total.
  void set_jobs(const std::vector<JobDev>& jobs, unsigned long long total) {
    if (int(jobs.size()) > max_jobs) throw ApiError{HASTY_ERR_ARG, "too many jobs for the engine"};
    int32_t n = int32_t(jobs.size());
    if (n) ck(cudaMemcpyAsync(d_jobs, jobs.data(), sizeof(JobDev) * jobs.size(), cudaMemcpyHostToDevice, stream), "jobs");
    ck(cudaMemcpyAsync(d_njobs, &n, sizeof(n), cudaMemcpyHostToDevice, stream), "n_jobs");
    ck(cudaMemcpyAsync(md.total_samples, &total, sizeof(total), cudaMemcpyHostToDevice, stream), "total");
    ck(cudaStreamSynchronize(stream), "set jobs");
  }

  // Runs up to n_iter iterations on the device (one graph launch); returns
  // true while work remains.
  bool run_wave(uint32_t n_iter, bool* bound_hit) {
    uint32_t end = iterations + n_iter;
    ck(cudaMemcpyAsync(&md.ctl[7], &end, sizeof(end), cudaMemcpyHostToDevice, stream), "wave end");
    ck(cudaGraphLaunch(exec, stream), "cudaGraphLaunch");
    uint32_t ctl[8];
    unsigned long long ns[2];
    uint32_t counts[4];
    ck(cudaMemcpyAsync(ctl, md.ctl, sizeof(ctl), cudaMemcpyDeviceToHost, stream), "ctl");
    ck(cudaMemcpyAsync(ns, md.next_sample, sizeof(unsigned long long), cudaMemcpyDeviceToHost, stream), "next");
    ck(cudaMemcpyAsync(ns + 1, md.total_samples, sizeof(unsigned long long), cudaMemcpyDeviceToHost, stream), "total");
    ck(cudaMemcpyAsync(counts, pd.counts, sizeof(counts), cudaMemcpyDeviceToHost, stream), "counts");
    ck(cudaStreamSynchronize(stream), "wave");
    iterations = ctl[5];
    if (bound_hit) *bound_hit = ctl[6] != 0;
    return counts[ctl[0]] > 0 || ns[0] < ns[1];
  }

  void stats(unsigned long long* out) {
    ck(cudaMemcpy(out, pd.stats, sizeof(unsigned long long) * MS_COUNT, cudaMemcpyDeviceToHost), "stats");
  }

  ~Engine() {
    if (stream) cudaStreamSynchronize(stream);
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    for (void* p : allocs) cudaFree(p);
    if (stream) cudaStreamDestroy(stream);
  }
};

namespace {

int64_t pool_size(const hasty_batch_config* cfg) {
  if (cfg && cfg->paths_in_flight > 0) return cfg->paths_in_flight;
  return int64_t(1) << 22;
}

uint32_t regen_threshold(const hasty_batch_config* cfg, int64_t cap) {
  float f = (cfg && cfg->regen_fraction > 0.f) ? cfg->regen_fraction : 0.9f;
  if (f >= 1.0f) return uint32_t(cap) + 1u;
  return uint32_t(double(cap) * double(f));
}

JobDev job_entry(hasty_job* j, unsigned long long* acc, unsigned long long* done, unsigned long long begin, int passes) {
  JobDev d;
  std::memset(&d, 0, sizeof(d));
  d.sc = j->sd;
  d.acc = acc;
  d.done = done;
  d.seed = j->seed;
  d.sample_begin = begin;
  d.pass_base = uint32_t(j->samples_done);
  d.npix = uint32_t(j->sd.width) * uint32_t(j->sd.height);
  d.n_samples = uint64_t(passes) * d.npix;
  return d;
}

}  // namespace
}  // namespace hasty

using namespace hasty;

extern "C" {

int hasty_batch_render(hasty_ctx* ctx, hasty_job** jobs, const int32_t* passes, size_t n_jobs, const hasty_batch_config* cfg,
                       hasty_batch_stats* out) {
  return guarded([&] {
    if (!ctx || (n_jobs && (!jobs || !passes))) throw ApiError{HASTY_ERR_ARG, "null argument"};
    for (size_t i = 0; i < n_jobs; ++i) {
      if (!jobs[i] || passes[i] < 0) throw ApiError{HASTY_ERR_ARG, "bad job or pass count"};
      if (jobs[i]->ctx != ctx) throw ApiError{HASTY_ERR_ARG, "job belongs to another context"};
      if (jobs[i]->sd.max_depth <= 0) throw ApiError{HASTY_ERR_ARG, "max_depth must be positive for batching"};
      ck(cudaStreamSynchronize(jobs[i]->stream), "job sync");
    }
    auto t0 = std::chrono::steady_clock::now();
    Engine e;
    int64_t cap = pool_size(cfg);
    uint32_t max_iter = (cfg && cfg->max_iterations > 0) ? uint32_t(cfg->max_iterations) : 50000000u;
    e.init(ctx, cap, int(std::max<size_t>(n_jobs, 1)), regen_threshold(cfg, cap), max_iter);
    std::vector<JobDev> table;
    std::vector<unsigned long long*> accs(n_jobs);
    unsigned long long* done = static_cast<unsigned long long*>(e.alloc(sizeof(unsigned long long) * std::max<size_t>(n_jobs, 1)));
    ck(cudaMemsetAsync(done, 0, sizeof(unsigned long long) * std::max<size_t>(n_jobs, 1), e.stream), "memset");
    unsigned long long total = 0;
    for (size_t i = 0; i < n_jobs; ++i) {
      size_t npix = size_t(jobs[i]->sd.width) * size_t(jobs[i]->sd.height);
      accs[i] = static_cast<unsigned long long*>(e.alloc(sizeof(unsigned long long) * 9 * npix));
      ck(cudaMemsetAsync(accs[i], 0, sizeof(unsigned long long) * 9 * npix, e.stream), "memset acc");
      table.push_back(job_entry(jobs[i], accs[i], done + i, total, passes[i]));
      total += table.back().n_samples;
    }
    e.set_jobs(table, total);
    cudaEvent_t a, b;
    ck(cudaEventCreate(&a), "event"); ck(cudaEventCreate(&b), "event");
    ck(cudaEventRecord(a, e.stream), "event");
    bool bound = false;
    e.run_wave(max_iter, &bound);
    ck(cudaEventRecord(b, e.stream), "event");
    ck(cudaEventSynchronize(b), "event");
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a); cudaEventDestroy(b);
    if (bound) throw ApiError{HASTY_ERR_CUDA, "batch stopped at its iteration bound"};
    // fold the fixed-point sums into each job's FP64 accumulators
    for (size_t i = 0; i < n_jobs; ++i) {
      hasty_job* j = jobs[i];
      launch_fixed_to_double(accs[i], j->sd.width * j->sd.height, j->acc[0], j->acc[1], j->acc[2], e.stream);
      j->samples_done += passes[i];
    }
    ck(cudaGetLastError(), "fold");
    unsigned long long st[MS_COUNT];
    ck(cudaStreamSynchronize(e.stream), "fold");
    e.stats(st);
    if (out) {
      std::memset(out, 0, sizeof(*out));
      out->device_ms = ms;
      out->wall_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
      out->samples = total;
      out->rays = st[MS_RAYS]; out->shaded = st[MS_SHADED]; out->nan_samples = st[MS_NAN];
      out->saturated = st[MS_SATURATED]; out->iterations = e.iterations; out->paths_in_flight = e.cap;
      out->engine_bytes = e.bytes;
    }
    return HASTY_OK;
  });
}

}  // extern "C"
