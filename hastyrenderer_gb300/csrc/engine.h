// Multi-job engine host side, shared by batching (engine.cpp) and serving
// (server.cpp). The engine owns one pool of path slots, a table of job slots,
// a ring of pass segments and a CUDA graph whose conditional while-node
// repeats one iteration (regenerate, trace, shade, condition) on the device
// until every issued sample is finished or the wave's iteration budget is
// spent. Jobs stay resident: scene, BVH and accumulators are buffers the
// caller owns; the engine only keeps pointers to them in its job table.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <deque>
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
  int job_slots = 0;
  uint32_t seg_cap = 0;
  JobDev* d_jobs = nullptr;
  SegDev* d_segs = nullptr;
  uint32_t* d_window = nullptr;
  unsigned long long* d_done = nullptr;   // per job slot: finished samples
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  uint32_t iterations = 0;
  // false: iterations are plain stream launches issued by the host, one at a
  // time (HASTY_ENGINE_LAUNCH=stream; profilers cannot see into graphs with
  // conditional nodes). Same kernels, same results.
  bool use_graph = true;
  // host view, as of the end of the last wave
  uint32_t seg_lo = 0, seg_hi = 0;
  std::deque<std::pair<unsigned long long, uint32_t>> spans;   // (begin, samples) of segments [seg_lo, seg_hi)
  unsigned long long total = 0;   // samples appended so far
  unsigned long long next = 0;    // samples issued so far
  uint32_t live = 0;              // paths in flight

  Engine() = default;
  Engine(const Engine&) = delete;
  Engine& operator=(const Engine&) = delete;
  ~Engine();

  void* alloc(size_t b);
  // capacity: path slots; slots: job-table entries; segments: ring size
  // (rounded up to a power of two).
  void init(hasty_ctx* c, int64_t capacity, int slots, uint32_t segments, uint32_t regen_below, uint32_t max_iter);
  // Writes job-table entry `slot` and clears its finished-sample counter.
  // Only for a slot no live path refers to.
  void set_job(int slot, const JobDev& j);
  unsigned long long* done_counter(int slot) const { return d_done + slot; }
  uint32_t free_segments() const { return seg_cap - (seg_hi - seg_lo); }
  // Appends one pass of job `slot` (npix samples) after the issued work.
  void append(int slot, uint32_t pass, uint32_t npix);
  // Makes appended segments visible to the device (call before run_wave).
  void publish();
  // One graph launch of up to n_iter iterations; synchronous. Returns true
  // while work remains.
  bool run_wave(uint32_t n_iter, bool* bound_hit);
  // run_wave in two halves, so that waves of several engines (one stream
  // each) run at the same time: launch_wave returns once the wave is queued
  // (graph mode; the host-driven stream mode runs it to the end), and
  // finish_wave waits for it and reads the engine's state back.
  void launch_wave(uint32_t n_iter);
  bool finish_wave(bool* bound_hit);
  // Resident blocks per SM of the persistent closest-hit kernel (0: all that
  // fit); set before init, for engines that share the GPU with another.
  int trace_blocks_per_sm = 0;
  bool busy() const { return live > 0 || next < total; }
  unsigned long long unissued() const { return total - next; }
  void read_done(std::vector<unsigned long long>& out);
  void stats(unsigned long long* out);

 private:
  std::vector<SegDev> staged;
  uint32_t wave_end = 0;
  void build_graph();
};

int64_t engine_pool_size(int64_t requested);
// Accumulator lanes of a job of npix pixels in a pool of cap paths: one lane
// per 256 samples of a pixel that can be in flight, 1..16 lanes. Only tiny
// frames get more than one: lanes multiply the job's accumulator footprint,
// and sums that fall out of L2 cost more than contended atomics.
uint32_t engine_lanes(int64_t cap, uint32_t npix);
uint32_t engine_regen_threshold(float fraction, int64_t cap);
// hasty_batch_render in HASTY_BATCH_REGEN mode (engine.cpp).
int batch_render_regen(hasty_ctx* ctx, hasty_job** jobs, const int32_t* passes, size_t n_jobs,
                       const hasty_batch_config* cfg, hasty_batch_stats* out);

}  // namespace hasty
