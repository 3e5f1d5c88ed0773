// Packed multi-job batches (batching and serving). A batch is filled with
// chunks of consecutive passes of several resident jobs, laid out one after
// another in the slots of one render lane; the lane runs the same wavefront
// kernels as the single-job path (ray generation, then per bounce closest
// hit, resolve, sample), the kernels finding each path's job through the
// chunk table passed as a kernel parameter. Lanes alternate on their own
// streams, so one batch's tracing overlaps another's shading; every batch's
// accumulation runs on one accumulation stream in batch order, and adds each
// pass into the job's FP64 sums one pass after the other. A job's image is
// therefore bit-identical to the single-job path's, whatever it is batched
// with.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "job.h"

namespace hasty {

constexpr int kMaxLanes = 4;

// A job as packed batches see it.
struct PackedJob {
  SceneDev sc;
  uint64_t seed = 0;
  double* acc[3] = {nullptr, nullptr, nullptr};   // FP64 sums: colour, normal, albedo (npix x 3 each)
  int32_t npix = 0;
  bool path_kernel = false;                      // rendered by the path kernel (use_path_kernel)
  bool simple_trace = false;                     // closest hits one ray per thread (simple_trace_bvh)
};

// Kernel class of a job; a batch holds jobs of one class: 0 wavefront with
// the persistent closest-hit kernel, 1 wavefront with one ray per thread
// (BVHs of a few nodes), 2 path kernel.
constexpr int kKernelClasses = 3;
inline int kernel_class(const PackedJob& j) { return j.path_kernel ? 2 : (j.simple_trace ? 1 : 0); }

// n_passes consecutive passes of job `job` from pass_base.
struct PackedChunk {
  int job;
  uint32_t pass_base;
  int32_t n_passes;
};

struct PackedLanes {
  hasty_ctx* ctx = nullptr;
  int n_lanes = 0;
  int64_t lane_paths = 0;                 // path slots of each lane
  int bvh_kind = 1;
  PathsDev pd[kMaxLanes] = {};
  PathsDev slots[kMaxLanes] = {};         // path-kernel slot pools
  cudaStream_t lane_stream[kMaxLanes] = {};
  cudaEvent_t lane_done[kMaxLanes] = {}, lane_free[kMaxLanes] = {};
  bool lane_free_valid[kMaxLanes] = {};
  cudaStream_t acc_stream = nullptr;      // accumulation, in batch order
  cudaEvent_t acc_ready = nullptr;
  unsigned long long* stats = nullptr;    // StatIndex counters of every lane
  std::vector<void*> allocs;
  int64_t bytes = 0;
  int next_lane = 0;
  // block shapes of the shading kernels and the closest-hit grid cap while
  // batches overlap (the autotuner's knobs; 0: defaults)
  int resolve_threads = 0, sample_threads = 0, trace_blocks_per_sm = 0;
  uint64_t batches = 0, launches = 0;

  PackedLanes() = default;
  PackedLanes(const PackedLanes&) = delete;
  PackedLanes& operator=(const PackedLanes&) = delete;
  ~PackedLanes();

  // lanes: 1..kMaxLanes; lane_paths: slots per lane (whole frames of every
  // job must fit: the caller checks).
  void init(hasty_ctx* c, int lanes, int64_t lane_paths);
  // Makes every lane wait for work already enqueued on `s` (accumulators
  // cleared there, for instance).
  void wait_for(cudaStream_t s);
  // Enqueues one batch on the next lane (asynchronous). `overlap`: other
  // batches run at the same time (the closest-hit grid then leaves room for
  // their shading). Chunks must fit one lane and number at most kMaxChunks.
  // A batch whose jobs all use the path kernel (use_path_kernel) runs the
  // path kernel, any other the wavefront; pack_batch keeps the two apart.
  // `start` (optional, a timing event) is recorded on the lane's stream when
  // the batch can start.
  void launch(const std::vector<PackedJob>& jobs, const std::vector<PackedChunk>& chunks, bool overlap,
              cudaEvent_t start = nullptr);
  void read_stats(unsigned long long* out);

 private:
  void* alloc(size_t b);
};

// Fills one batch: passes of the jobs in `order` (job indices), each job's
// next passes in order (pass_base[j], left[j] updated), up to `slots` path
// slots and kMaxChunks chunks, and (when job_samples > 0) at most
// job_samples camera samples of one job (one pass at least). A job whose
// next pass does not fit the space left is skipped for this batch. Returns
// the chunks (empty when nothing is left).
std::vector<PackedChunk> pack_batch(const std::vector<PackedJob>& jobs, const std::vector<int>& order,
                                    std::vector<uint32_t>& pass_base, std::vector<int32_t>& left, int64_t slots,
                                    int64_t job_samples = 0);
// Jobs of `order` in one kernel class (kernel_class), order kept.
std::vector<int> class_order(const std::vector<PackedJob>& jobs, const std::vector<int>& order, int cls);
// Cycles through the kernel classes between consecutive batches while more
// than one has passes left, so batches of different classes run side by side
// on the lanes (`turn`: the class to try first, advanced past the one taken).
std::vector<PackedChunk> pack_next(const std::vector<PackedJob>& jobs, const std::vector<int>& order,
                                   std::vector<uint32_t>& pass_base, std::vector<int32_t>& left, int64_t slots,
                                   int64_t job_samples, int& turn);

// Path slots of a lane: 16M camera samples (whole frames of the largest
// job at least), or `requested` when positive.
int64_t packed_lane_paths(int64_t requested, int64_t largest_frame);

}  // namespace hasty
