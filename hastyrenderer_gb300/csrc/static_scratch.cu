// One render pass that allocates no device memory.
//
// Some callers cannot call cudaMalloc while they render: a host application
// that hands all of the GPU's memory to its own allocator up front, a plugin
// host that forbids its plugins to allocate, or a real-time loop in which an
// allocation (which can synchronise the device) is not allowed.
// hasty_job_render_pass_static serves them. The scene is the job's (uploaded
// once by hasty_job_load), the output buffer is the caller's, and every
// scratch buffer of the wavefront (path state, rays, hits, queues, counters,
// statistics, normal and albedo sums) is carved from one file-scope device
// array, g_scratch below. The call makes no cudaMalloc, cudaFree or other
// allocating call.
//
// Limits. g_scratch is kStaticBytes (8 MiB), which holds the state of
// kStaticMaxPixels (16384) camera paths, e.g. a 128 x 128 frame; a larger
// frame is rejected with HASTY_ERR_ARG. Each device that runs this code
// reserves the array for the life of the process.
//
// Set-up. The first call on each device looks up the array's device address
// (cudaGetSymbolAddress) with that device current; make that first call
// before any stream capture begins. The address is kept for the life of the
// process: after cudaDeviceReset (or anything else that destroys and
// recreates the device's primary context) this entry point must not be
// called again in that process.
//
// Sharing. Every call uses the same array and the array keeps whatever the
// last call left in it. Each call clears what must start at zero (queue
// counters, statistics, the normal and albedo sums and the caller's output)
// before its kernels run. Calls whose GPU work overlaps (jobs rendering
// through this entry point on different streams, or from several host
// threads, at the same time) race on the array and produce garbage. Note
// that each job has its own stream and the call returns before its GPU work
// ends, so two calls on two different jobs from one host thread already
// overlap: call hasty_job_sync on the first job before calling on another.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <string>

#include "job.h"

namespace hasty {
namespace {

constexpr size_t kStaticBytes = size_t(8) << 20;
constexpr int kStaticMaxPixels = 16384;   // path state + 48 B of sums per pixel
constexpr int kMaxDevices = 64;
constexpr size_t kCarveAlign = 256;

// Bytes one call carves from g_scratch for a frame of npix pixels: the path
// state of npix slots (the same carving as every other path pool) and the
// normal and albedo sums, each block on a kCarveAlign boundary.
int64_t static_bytes_needed(int64_t npix) {
  return carved_bytes(npix, ST_COUNT, kCarveAlign, 2, sizeof(double) * 3 * size_t(npix));
}

static __device__ __align__(256) unsigned char g_scratch[kStaticBytes];

std::mutex g_mu;
unsigned char* g_scratch_addr[kMaxDevices] = {nullptr};

// Device address of g_scratch on `device` (which must be current).
unsigned char* scratch_address(int device) {
  std::lock_guard<std::mutex> lock(g_mu);
  if (device < 0 || device >= kMaxDevices) throw ApiError{HASTY_ERR_ARG, "device ordinal out of range"};
  if (!g_scratch_addr[device]) {
    void* p = nullptr;
    ck(cudaGetSymbolAddress(&p, g_scratch), "cudaGetSymbolAddress(static scratch)");
    if (!p) throw ApiError{HASTY_ERR_CUDA, "static scratch has no device address"};
    g_scratch_addr[device] = static_cast<unsigned char*>(p);
  }
  return g_scratch_addr[device];
}

}  // namespace
}  // namespace hasty

using namespace hasty;

extern "C" int hasty_job_render_pass_static(hasty_job* job, int pass, double* d_color) {
  return guarded([&] {
    if (!job) throw ApiError{HASTY_ERR_ARG, "null job handle"};
    if (!d_color) throw ApiError{HASTY_ERR_ARG, "null output buffer"};
    if (pass < 0) throw ApiError{HASTY_ERR_ARG, "negative pass index"};
    const int64_t npix64 = int64_t(job->sd.width) * int64_t(job->sd.height);
    if (npix64 <= 0 || npix64 > kStaticMaxPixels)
      throw ApiError{HASTY_ERR_ARG, "frame of " + std::to_string(npix64) +
                                        " pixels is outside the static scratch limit of 1.." +
                                        std::to_string(kStaticMaxPixels) + " pixels"};
    const int npix = int(npix64);
    ck(cudaSetDevice(job->ctx->device), "cudaSetDevice");
    unsigned char* base = scratch_address(job->ctx->device);
    size_t used = 0;
    auto carve = [&](size_t bytes) -> void* {
      size_t off = (used + kCarveAlign - 1) & ~(kCarveAlign - 1);
      if (off + bytes > kStaticBytes) throw ApiError{HASTY_ERR_ARG, "frame does not fit the static scratch"};
      used = off + bytes;
      return base + off;
    };
    const size_t sum_bytes = sizeof(double) * 3 * size_t(npix);
    PathsDev p{};
    alloc_paths_into(p, npix, ST_COUNT, carve, job->stream);   // carves and clears counters and statistics
    double* sum_normal = static_cast<double*>(carve(sum_bytes));
    double* sum_albedo = static_cast<double*>(carve(sum_bytes));
    ck(cudaMemsetAsync(d_color, 0, sum_bytes, job->stream), "clear output");
    ck(cudaMemsetAsync(sum_normal, 0, sum_bytes, job->stream), "clear scratch");
    ck(cudaMemsetAsync(sum_albedo, 0, sum_bytes, job->stream), "clear scratch");
    BatchDesc b;
    b.seed = job->seed;
    b.pass_base = uint32_t(pass);
    b.n_passes = 1;
    b.n_paths = npix;
    launch_raygen(job->sd, p, b, job->stream);
    for (int bounce = 0; bounce < job->sd.max_depth; ++bounce) {
      int q = bounce & 1;
      launch_trace(job->sd, p, q, 2 * npix, job->stream);
      launch_shade(job->sd, p, b, q, npix, job->stream);
    }
    launch_accumulate(job->sd, p, b, d_color, sum_normal, sum_albedo, job->stream);
    ck(cudaGetLastError(), "static render launch");
    return HASTY_OK;
  });
}

extern "C" int hasty_debug_static_scratch(int64_t* max_pixels, int64_t* bytes_needed, int64_t* capacity) {
  return guarded([&] {
    if (!max_pixels || !bytes_needed || !capacity) throw ApiError{HASTY_ERR_ARG, "null argument"};
    *max_pixels = kStaticMaxPixels;
    *bytes_needed = static_bytes_needed(kStaticMaxPixels);
    *capacity = int64_t(kStaticBytes);
    return HASTY_OK;
  });
}
