// C ABI of the GB300 path tracer (include/hasty_gpu.h): job lifecycle, device
// upload, batch orchestration and outputs. The pass loop replaces the
// reference's renderThread (core/src/PathTracing.cpp:98-160): instead of one
// CPU thread rendering whole 1-spp frames, a batch of passes is rendered as
// one wavefront of W*H*passes camera samples on the job's CUDA stream, and the
// per-sample results are folded into FP64 accumulators in pass order.
#include "hasty_gpu.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <exception>
#include <memory>
#include <mutex>
#include <string>
#include <sys/stat.h>
#include <system_error>
#include <thread>
#include <vector>

#include "bvh_build.h"
#include "job.h"
#include "image_out.h"
#include "scene_load.h"
#include "wavefront.h"

namespace hasty {
// integrator.cu
uint32_t bounds_status_integrator();
uint32_t bounds_status_trace();
uint32_t bounds_status_photon();
void launch_debug_bsdf(int which, const float* in, int n, const uint32_t* replay, int n_replay, float* out, cudaStream_t st);
// trace.cu
void host_trace_rays(int kind, const float4* nodes, const float4* tris, const float* rays, int64_t n, float4* hits);
}

using namespace hasty;

namespace hasty {
thread_local std::string g_error;
}

namespace {

}  // namespace

void hasty::carve_paths(PathsDev& p, int64_t cap, int n_stats, const std::function<void*(size_t)>& alloc,
                        unsigned long long* stats, int64_t media_blocks) {
  auto A = [&](size_t bytes) { return alloc(bytes); };
  p.capacity = int32_t(cap);
  size_t c = size_t(cap);
  p.rng = static_cast<uint64_t*>(A(c * sizeof(uint64_t)));
  p.thr = static_cast<float4*>(A(c * sizeof(float4)));
  p.rad = static_cast<float4*>(A(c * sizeof(float4)));
  p.pend_b = static_cast<float4*>(A(c * sizeof(float4)));
  p.nee_c = static_cast<float4*>(A(c * sizeof(float4)));
  p.nee_t = static_cast<float4*>(A(c * sizeof(float4)));
  p.med = static_cast<float4*>(A(c * kMaxMedia * sizeof(float4)));
  p.med_geom = static_cast<int32_t*>(A(c * kMaxMedia * sizeof(int32_t)));
  p.med_block = static_cast<int32_t*>(A(c * sizeof(int32_t)));
  p.med_pool_blocks = int32_t(media_blocks > 0 ? media_blocks : std::max<int64_t>(64, cap / 4));
  p.med_pool = static_cast<float4*>(A(size_t(p.med_pool_blocks) * kMediaBlock * sizeof(float4)));
  p.med_pool_geom = static_cast<int32_t*>(A(size_t(p.med_pool_blocks) * kMediaBlock * sizeof(int32_t)));
  p.ray_o = static_cast<float4*>(A(2 * c * sizeof(float4)));
  p.ray_d = static_cast<float4*>(A(2 * c * sizeof(float4)));
  p.hit = static_cast<float4*>(A(2 * c * sizeof(float4)));
  p.pq[0] = static_cast<int32_t*>(A(c * sizeof(int32_t)));
  p.pq[1] = static_cast<int32_t*>(A(c * sizeof(int32_t)));
  p.rq[0] = static_cast<int32_t*>(A(2 * c * sizeof(int32_t)));
  p.rq[1] = static_cast<int32_t*>(A(2 * c * sizeof(int32_t)));
  p.counts = static_cast<uint32_t*>(A(kCountSlots * sizeof(uint32_t)));
  p.sq = static_cast<int32_t*>(A(c * sizeof(int32_t)));
  p.out_color = static_cast<float4*>(A(c * sizeof(float4)));
  p.out_normal = static_cast<float4*>(A(c * sizeof(float4)));
  p.out_albedo = static_cast<float4*>(A(c * sizeof(float4)));
  p.stats = stats ? stats : static_cast<unsigned long long*>(A(size_t(n_stats) * sizeof(unsigned long long)));
}

void hasty::alloc_paths_into(PathsDev& p, int64_t cap, int n_stats, const std::function<void*(size_t)>& alloc, cudaStream_t st,
                             unsigned long long* stats) {
  carve_paths(p, cap, n_stats, alloc, stats);
  if (!stats) ck(cudaMemsetAsync(p.stats, 0, sizeof(unsigned long long) * size_t(n_stats), st), "memset stats");
  ck(cudaMemsetAsync(p.counts, 0, sizeof(uint32_t) * kCountSlots, st), "memset counts");
}

int64_t hasty::carved_bytes(int64_t cap, int n_stats, size_t align, size_t extra_blocks, size_t extra_bytes) {
  size_t used = 0;
  auto count = [&](size_t bytes) -> void* {
    used = ((used + align - 1) / align) * align + bytes;
    return reinterpret_cast<void*>(uintptr_t(align));   // never dereferenced
  };
  PathsDev p{};
  carve_paths(p, cap, n_stats, count, nullptr);
  for (size_t k = 0; k < extra_blocks; ++k) count(extra_bytes);
  return int64_t(used);
}

// Path-state buffers of the single-job path are allocated at the first
// render (jobs that only feed the multi-job engine never need them) and
// re-allocated when the paths-in-flight setting changes.
namespace {
// Frees the path buffers of p (not the statistics it points to).
void release_path_buffers(hasty_job& j, PathsDev& p) {
  void* bufs[] = {p.rng, p.thr, p.rad, p.pend_b, p.nee_c, p.nee_t, p.med, p.med_geom, p.med_block, p.med_pool,
                  p.med_pool_geom, p.ray_o, p.ray_d, p.hit,
                  p.pq[0], p.pq[1], p.rq[0], p.rq[1], p.counts, p.sq, p.out_color, p.out_normal, p.out_albedo};
  for (void* b : bufs) j.release(b);
  unsigned long long* stats = p.stats;
  p = PathsDev{};
  p.stats = stats;
}
}  // namespace

void hasty::ensure_paths(hasty_job& j, int64_t need) {
  for (int k = 0; k < 2; ++k) {
    if (!j.lane_stream[k]) ck(cudaStreamCreateWithFlags(&j.lane_stream[k], cudaStreamNonBlocking), "lane stream");
    if (!j.lane_done[k]) ck(cudaEventCreateWithFlags(&j.lane_done[k], cudaEventDisableTiming), "lane event");
    if (!j.lane_free[k]) ck(cudaEventCreateWithFlags(&j.lane_free[k], cudaEventDisableTiming), "lane event");
  }
  if (!j.main_ready) ck(cudaEventCreateWithFlags(&j.main_ready, cudaEventDisableTiming), "lane event");
  // buffers grow to what a call needs, up to the paths-in-flight setting
  need = std::max<int64_t>(1, std::min(need, j.capacity));
  if (j.pd.rng && j.pd.capacity >= need && j.pd.capacity <= j.capacity) return;
  ck(cudaStreamSynchronize(j.stream), "sync");
  for (cudaStream_t s : j.lane_stream) ck(cudaStreamSynchronize(s), "sync");
  release_path_buffers(j, j.pd);
  release_path_buffers(j, j.pd2);       // lane 1 is allocated again when next used
  unsigned long long* stats = j.pd.stats;
  alloc_paths_into(j.pd, need, ST_COUNT, [&](size_t b) { return static_cast<void*>(j.alloc<uint8_t>(b)); }, j.stream,
                   stats);
  j.lane_free_valid[0] = j.lane_free_valid[1] = false;
  j.lanes_wait_main = true;             // counters were cleared on `stream`
}

// Lane 1's path buffers, sharing lane 0's statistics.
void ensure_lane2(hasty_job& j) {
  if (j.pd2.rng && j.pd2.capacity == j.pd.capacity) return;
  release_path_buffers(j, j.pd2);
  alloc_paths_into(j.pd2, j.pd.capacity, ST_COUNT, [&](size_t b) { return static_cast<void*>(j.alloc<uint8_t>(b)); }, j.stream,
                   j.pd.stats);
  j.lane_free_valid[1] = false;
  j.lanes_wait_main = true;
}

namespace {

// Host half of the upload: BVH and CDF guide tables (no device work).
void prepare_scene(hasty_job& j) {
  if (j.prep) return;
  HostScene& h = j.host;
  std::unique_ptr<hasty_job::Prepared> p(new hasty_job::Prepared());
  bool binary = (j.ctx->flags & HASTY_CTX_BINARY_BVH) != 0;
  bool on_host = (j.ctx->flags & HASTY_CTX_HOST_BVH) != 0;
  if (!on_host) ck(cudaSetDevice(j.ctx->device), "cudaSetDevice");
  if (binary) {
    if (on_host) build_bvh_binary(h.tri_pos.data(), h.n_tris(), 4, p->bvh);
    else build_bvh_binary_gpu(h.tri_pos.data(), h.n_tris(), 4, p->bvh);
    if (p->bvh.depth > 60) throw ApiError{HASTY_ERR_LOAD, "BVH deeper than the traversal stack (64)"};
  } else {
    if (on_host) build_bvh_wide(h.tri_pos.data(), h.n_tris(), p->bvh);
    else build_bvh_wide_gpu(h.tri_pos.data(), h.n_tris(), p->bvh);
    if (p->bvh.depth > 30) throw ApiError{HASTY_ERR_LOAD, "wide BVH deeper than the traversal stack (32)"};
  }
  p->binary = binary;
  p->light_guide = build_cdf_guide(h.light_cdf, p->light_guide_log2);
  p->env_guide = build_cdf_guide(h.env_cdf, p->env_guide_log2);
  j.prep = std::move(p);
}

template <class T>
int64_t vec_bytes(const std::vector<T>& v) { return int64_t(v.size() * sizeof(T)); }

// Device bytes upload_scene allocates for a prepared job.
int64_t upload_bytes(const hasty_job& j) {
  const HostScene& h = j.host;
  const hasty_job::Prepared& p = *j.prep;
  return vec_bytes(h.tri_pos) + vec_bytes(h.tri_attr) + vec_bytes(h.normals) + vec_bytes(h.texcoords) +
         vec_bytes(p.bvh.nodes) + vec_bytes(p.bvh.tris) + vec_bytes(h.mats) + vec_bytes(h.textures) +
         vec_bytes(h.tex_pool) + vec_bytes(h.tex_pool8) + vec_bytes(h.light_tris) + vec_bytes(h.light_cdf) + vec_bytes(p.light_guide) +
         vec_bytes(h.env_texels) + vec_bytes(h.env_weights) + vec_bytes(h.env_cdf) + vec_bytes(p.env_guide);
}

void upload_scene(hasty_job& j) {
  prepare_scene(j);
  const auto u0 = std::chrono::steady_clock::now();
  HostScene& h = j.host;
  SceneDev& s = j.sd;
  hasty_job::Prepared& p = *j.prep;
  j.bvh_depth = p.bvh.depth; j.bvh_ms = p.bvh.build_ms; j.bvh_tree_ms = p.bvh.tree_ms;
  s.n_tris = int32_t(h.n_tris());
  s.tri_pos = j.upload(h.tri_pos);
  s.tri_attr = j.upload(h.tri_attr);
  s.normals = j.upload(h.normals);
  s.texcoords = j.upload(h.texcoords);
  s.n_texcoords = int64_t(h.texcoords.size());
  s.bvh_kind = p.binary ? 0 : 1;
  s.nodes = reinterpret_cast<const float4*>(j.upload(p.bvh.nodes));
  s.isect_tris = reinterpret_cast<const float4*>(j.upload(p.bvh.tris));
  s.n_nodes = int32_t(p.bvh.nodes.size() / (p.binary ? 16 : 20));
  s.mats = j.upload(h.mats);
  s.textures = j.upload(h.textures);
  s.n_mats = int32_t(h.mats.size());
  s.n_textures = int32_t(h.textures.size());
  s.tex_pool = j.upload(h.tex_pool);
  s.tex_pool8 = j.upload(h.tex_pool8);
  s.n_light_tris = int32_t(h.light_tris.size());
  s.light_tris = j.upload(h.light_tris);
  s.light_cdf = j.upload(h.light_cdf);
  s.light_guide = j.upload(p.light_guide);
  s.light_guide_log2 = p.light_guide_log2;
  s.light_pdf_area = h.light_tris.empty() ? 0.0f : 1.0f / h.total_light_area;
  EnvDev& e = s.env;
  e.is_texture = h.env_texture ? 1 : 0;
  for (int c = 0; c < 3; ++c) e.color[c] = h.bg[c];
  e.w = h.env_w; e.h = h.env_h;
  e.texels = j.upload(h.env_texels);
  e.weights = j.upload(h.env_weights);
  e.cdf = j.upload(h.env_cdf);
  e.guide = j.upload(p.env_guide);
  e.guide_log2 = p.env_guide_log2;
  e.value_sum = h.env_value_sum;
  s.cam = h.cam;
  const RenderSettingsH& st = h.settings;
  s.width = int32_t(st.width); s.height = int32_t(st.height);
  s.max_depth = st.max_depth; s.rr_start = st.roulette_start; s.rr_q = st.roulette_q;
  s.two_strategies = (h.has_light() && st.use_mis) ? 1 : 0;
  s.env_is_sampled = h.env_texture ? 1 : 0;
  s.p_surface = !h.env_texture ? 1.0f : (!h.light_tris.empty() ? 0.5f : 0.0f);   // Scene.cpp:545
  ck(cudaStreamSynchronize(j.stream), "sync upload");   // the host arrays may be freed after this
  j.upload_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - u0).count();
  j.prep.reset();
}

void clear_accumulators(hasty_job& j) {
  size_t n = size_t(j.sd.width) * size_t(j.sd.height) * 3;
  for (double* a : j.acc) ck(cudaMemsetAsync(a, 0, n * sizeof(double), j.stream), "memset acc");
  ck(cudaMemsetAsync(j.pd.stats, 0, sizeof(unsigned long long) * ST_COUNT, j.stream), "memset stats");
  j.lanes_wait_main = true;
  j.samples_done = 0;
  j.kernel_ms = j.trace_ms = j.shade_ms = j.path_ms = 0.0;
  j.trace_launches = j.kernel_launches = j.path_launches = 0;
}

// Up to 16M camera samples in flight per render lane (about 7 GB of path
// state each, allocated as far as a call needs it): fewer, larger batches
// per call. 1080p, 8 passes per call, two lanes (M samples/s): 2M paths 777,
// 4M 848, 8M 884, 16.6M (all 8 passes in one batch) 896.
int64_t default_capacity(int64_t npix) {
  int64_t cap = int64_t(1) << 24;
  if (npix > cap) cap = npix;
  return (cap / npix) * npix;
}

// Resident blocks per SM of the persistent closest-hit kernel while two
// render lanes run: fewer than fit (9 on GB300) leaves room for the other
// lane's shading blocks. Measured on the 1080p sphere field (M samples/s),
// 2-pass batches: all 822, 7: 829, 6: 834, 5: 836-840, 4: 822, 3: 788;
// 8-pass batches: all 883, 7: 897, 6: 897, 5: 900, 4: 903, 3: 865;
// with the 256/512-thread shading blocks: all 942, 7: 938, 6: 943, 5: 948,
// 4: 940.
constexpr int kLaneTraceBlocksPerSM = 5;
}  // namespace

// Largest scene the path kernel takes by default: none. Measured on GB300
// (M samples/s, path kernel vs wavefront): Cornell box 1024x768 475 vs 607,
// 128x128 389 vs 496; 64k-triangle field 1024x768 924 vs 2365; 1.02M
// triangles 256x192 318 vs 822, at 64, 96 or 128 registers per thread. Its
// path state stays in L2, but the wavefront's shading kernels are bound by
// load latency at 35-52% of HBM bandwidth, not by their traffic, and the
// path kernel loses more to idle lanes, block barriers and undivided
// traversal than it saves. HASTY_PATH_KERNEL_TRIS (or HASTY_CTX_PATH_KERNEL)
// selects it.
constexpr int64_t kPathKernelMaxTris = 0;

int64_t hasty::path_kernel_max_triangles() {
  static const int64_t v = [] {
    const char* e = std::getenv("HASTY_PATH_KERNEL_TRIS");
    return e ? std::max<int64_t>(0, std::atoll(e)) : kPathKernelMaxTris;
  }();
  return v;
}

bool hasty::use_path_kernel(const hasty_ctx* ctx, const SceneDev& sc) {
  if (sc.max_depth <= 0 || (ctx->flags & HASTY_CTX_WAVEFRONT)) return false;
  return (ctx->flags & HASTY_CTX_PATH_KERNEL) || int64_t(sc.n_tris) <= path_kernel_max_triangles();
}

void hasty::alloc_path_slots(PathsDev& p, const std::function<void*(size_t)>& alloc, unsigned long long* stats) {
  // a slot keeps its overflow block for all the paths it carries in a launch
  const int64_t n = path_slots();
  carve_paths(p, n, ST_COUNT, alloc, stats, std::max<int64_t>(64, n / 2));
}

// HASTY_LANE_TRACE_BLOCKS overrides it (0: no cap).
int hasty::lane_trace_blocks() {
  static const int v = [] {
    const char* e = std::getenv("HASTY_LANE_TRACE_BLOCKS");
    return e ? std::max(0, std::atoi(e)) : kLaneTraceBlocksPerSM;
  }();
  return v;
}

namespace {

// One batch of passes on render lane `lane` (the two lanes alternate; see
// hasty_job): ray generation and the bounces on the lane's stream, then the
// accumulation on the job's stream.
void render_batch(hasty_job& j, int n_passes, int lane, bool more_batches) {
  BatchDesc b;
  b.seed = j.seed;
  b.pass_base = uint32_t(j.samples_done);
  b.n_passes = n_passes;
  b.n_paths = n_passes * j.sd.width * j.sd.height;
  PathsDev& pd = lane ? j.pd2 : j.pd;
  cudaStream_t ls = j.lane_stream[lane];
  // cap the trace grid only while the other lane has work to overlap
  bool other_busy = more_batches;
  if (!other_busy && j.lane_free_valid[lane ^ 1]) {
    const cudaError_t qs = cudaEventQuery(j.lane_done[lane ^ 1]);
    if (qs == cudaErrorNotReady) {
      other_busy = true;
      (void)cudaGetLastError();        // "not ready" is an answer, not an error to report later
    }
  }
  const int trace_cap = (j.stage_timing || !other_busy) ? 0 : lane_trace_blocks();
  if (j.lane_free_valid[lane]) ck(cudaStreamWaitEvent(ls, j.lane_free[lane], 0), "lane wait");
  auto timed = [&](int stage, auto&& fn) {
    if (!j.stage_timing) { fn(); return; }
    cudaEvent_t a, c;
    ck(cudaEventCreate(&a), "event"); ck(cudaEventCreate(&c), "event");
    ck(cudaEventRecord(a, ls), "event record");
    fn();
    ck(cudaEventRecord(c, ls), "event record");
    j.pending_events.push_back({a, c, stage});
  };
  if (j.path_kernel) {
    PathsDev& slots = j.slots[lane];
    if (!slots.rng) {
      alloc_path_slots(slots, [&](size_t bytes) { return static_cast<void*>(j.alloc<uint8_t>(bytes)); }, j.pd.stats);
      ck(cudaMemsetAsync(slots.counts, 0, sizeof(uint32_t) * kCountSlots, ls), "memset counts");
    }
    timed(3, [&] { launch_paths(j.sd, b, slots, pd, ls); });
    j.path_launches += 1;
  } else {
    launch_raygen(j.sd, pd, b, ls);
    const int max_paths = b.n_paths;
    for (int bounce = 0; bounce < j.sd.max_depth; ++bounce) {
      int q = bounce & 1;
      timed(1, [&] { launch_trace(j.sd, pd, q, 2 * max_paths, ls, trace_cap); });
      timed(2, [&] { launch_shade(j.sd, pd, b, q, max_paths, ls); });
    }
    j.trace_launches += uint64_t(j.sd.max_depth);
  }
  ck(cudaEventRecord(j.lane_done[lane], ls), "lane event");
  ck(cudaStreamWaitEvent(j.stream, j.lane_done[lane], 0), "lane wait");
  launch_accumulate(j.sd, pd, b, j.acc[0], j.acc[1], j.acc[2], j.stream);
  ck(cudaGetLastError(), "kernel launch");
  ck(cudaEventRecord(j.lane_free[lane], j.stream), "lane event");
  j.lane_free_valid[lane] = true;
  // wavefront: raygen and accumulate, and per bounce trace, resolve, sample;
  // path kernel: it and accumulate
  j.kernel_launches += j.path_kernel ? 2u : uint64_t(2 + 3 * j.sd.max_depth);
  j.samples_done += n_passes;
}

hasty_job* as_job(hasty_job* j) {
  if (!j) throw ApiError{HASTY_ERR_ARG, "null job handle"};
  return j;
}

}  // namespace

std::unique_ptr<hasty_job> hasty::load_job_host(hasty_ctx* ctx, const std::string& path) {
  std::unique_ptr<hasty_job> j(new hasty_job());
  j->ctx = ctx;
  const auto t0 = std::chrono::steady_clock::now();
  load_render_job(path, j->host);
  j->parse_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  j->seed = j->host.settings.seed;
  return j;
}

void hasty::finish_job_load(hasty_job& job, bool plain) {
  hasty_job* j = &job;
  ck(cudaSetDevice(j->ctx->device), "cudaSetDevice");
  ck(cudaStreamCreateWithFlags(&j->stream, cudaStreamNonBlocking), "stream");
  upload_scene(*j);
  j->path_kernel = use_path_kernel(j->ctx, j->sd);
  int64_t npix = int64_t(j->sd.width) * j->sd.height;
  j->capacity = default_capacity(npix);
  if (plain) {
    j->pd.stats = j->alloc<unsigned long long>(ST_COUNT);
    for (double*& a : j->acc) a = j->alloc<double>(size_t(npix) * 3);
    j->est = j->alloc<float>(size_t(npix) * 3);
    clear_accumulators(*j);
  }
  ck(cudaStreamSynchronize(j->stream), "sync");
  // the host copies of the large arrays are not needed after upload
  std::vector<float>().swap(j->host.tri_pos);
  std::vector<float>().swap(j->host.env_texels);
  std::vector<float>().swap(j->host.tex_pool);
  std::vector<uint8_t>().swap(j->host.tex_pool8);
}

std::unique_ptr<hasty_job> hasty::load_job(hasty_ctx* ctx, const std::string& path, bool plain) {
  std::unique_ptr<hasty_job> j = load_job_host(ctx, path);
  finish_job_load(*j, plain);
  return j;
}

int64_t hasty::prepare_job_upload(hasty_job& j) {
  prepare_scene(j);
  return upload_bytes(j);
}

extern "C" {

int hasty_last_error(char* buf, size_t len) {
  if (!buf || len == 0) return HASTY_ERR_ARG;
  std::strncpy(buf, g_error.c_str(), len - 1);
  buf[len - 1] = 0;
  return HASTY_OK;
}

int hasty_version(int* major, int* minor) {
  if (major) *major = 0;
  if (minor) *minor = 1;
  return HASTY_OK;
}

int hasty_ctx_create(int device, uint32_t flags, hasty_ctx** out) {
  return guarded([&] {
    if (!out) throw ApiError{HASTY_ERR_ARG, "null output pointer"};
    int n = 0;
    ck(cudaGetDeviceCount(&n), "cudaGetDeviceCount");
    if (device < 0 || device >= n) throw ApiError{HASTY_ERR_ARG, "no CUDA device " + std::to_string(device)};
    ck(cudaSetDevice(device), "cudaSetDevice");
    auto* c = new hasty_ctx();
    c->device = device;
    c->flags = flags;
    ck(cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device), "attr");
    *out = c;
    return HASTY_OK;
  });
}

int hasty_ctx_destroy(hasty_ctx* ctx) { delete ctx; return HASTY_OK; }

int hasty_job_load(hasty_ctx* ctx, const char* path, hasty_job** out) {
  return guarded([&] {
    if (!ctx || !path || !out) throw ApiError{HASTY_ERR_ARG, "null argument"};
    *out = load_job(ctx, path, true).release();
    return HASTY_OK;
  });
}

int hasty_jobs_load(hasty_ctx* ctx, const char* const* paths, size_t n, int32_t threads, hasty_job** out) {
  return guarded([&] {
    if (!ctx || (n && (!paths || !out))) throw ApiError{HASTY_ERR_ARG, "null argument"};
    for (size_t i = 0; i < n; ++i) {
      if (!paths[i]) throw ApiError{HASTY_ERR_ARG, "null path"};
      out[i] = nullptr;
    }
    std::vector<std::unique_ptr<hasty_job>> jobs(n);
    std::atomic<size_t> next{0};
    std::atomic<bool> failed{false};
    std::mutex mu;
    std::exception_ptr first;   // the failure of the lowest-numbered failing job
    size_t first_i = n;
    auto worker = [&] {
      cudaSetDevice(ctx->device);
      for (;;) {
        const size_t i = next.fetch_add(1);
        if (i >= n || failed.load()) return;
        try {
          jobs[i] = load_job(ctx, paths[i], true);
        } catch (...) {
          std::lock_guard<std::mutex> lk(mu);
          if (i < first_i) { first_i = i; first = std::current_exception(); }
          failed = true;
        }
      }
    };
    size_t nt = threads > 0 ? size_t(threads) : size_t(std::max(1u, std::thread::hardware_concurrency()));
    nt = std::max<size_t>(1, std::min(nt, n));
    std::vector<std::thread> pool;
    for (size_t k = 1; k < nt; ++k) {
      try {
        pool.emplace_back(worker);
      } catch (const std::system_error&) {
        break;   // fewer threads: the ones running (and this one) take the rest
      }
    }
    worker();
    for (std::thread& t : pool) t.join();
    if (first) std::rethrow_exception(first);   // the loaded jobs are freed with `jobs`
    for (size_t i = 0; i < n; ++i) out[i] = jobs[i].release();
    return HASTY_OK;
  });
}

int hasty_job_destroy(hasty_job* job) { delete job; return HASTY_OK; }

int hasty_job_info_get(hasty_job* job, hasty_job_info* out) {
  return guarded([&] {
    as_job(job);
    if (!out) throw ApiError{HASTY_ERR_ARG, "null output"};
    const HostScene& h = job->host;
    out->width = int32_t(h.settings.width); out->height = int32_t(h.settings.height);
    out->num_samples = h.settings.num_samples; out->max_depth = h.settings.max_depth;
    out->roulette_start_depth = h.settings.roulette_start; out->roulette_q = h.settings.roulette_q;
    out->use_mis = h.settings.use_mis ? 1 : 0; out->seed = job->seed;
    out->n_triangles = int64_t(h.tri_attr.size()); out->n_light_triangles = int64_t(h.light_tris.size());
    out->n_shapes = int32_t(h.n_shapes); out->n_materials = int32_t(h.mats.size());
    out->env_is_texture = h.env_texture ? 1 : 0; out->exposure = h.cam.exposure;
    out->samples_done = job->samples_done; out->bvh_depth = job->bvh_depth; out->bvh_build_ms = job->bvh_ms;
    out->device_bytes = job->bytes;
    out->bvh_tree_ms = job->bvh_tree_ms;
    out->parse_ms = job->parse_ms;
    out->upload_ms = job->upload_ms;
    out->paths_in_flight = job->capacity;
    out->path_kernel = job->path_kernel ? 1 : 0;
    return HASTY_OK;
  });
}

int hasty_job_reset(hasty_job* job) {
  return guarded([&] {
    as_job(job);
    ck(cudaStreamSynchronize(job->stream), "sync");
    job->collect_events();
    clear_accumulators(*job);
    job->stop = false;
    ck(cudaStreamSynchronize(job->stream), "sync");
    return HASTY_OK;
  });
}

int hasty_job_set_seed(hasty_job* job, uint64_t seed) {
  int rc = hasty_job_reset(job);
  if (rc == HASTY_OK) job->seed = seed;
  return rc;
}

int hasty_job_set_paths_in_flight(hasty_job* job, int64_t paths) {
  return guarded([&] {
    as_job(job);
    int64_t npix = int64_t(job->sd.width) * job->sd.height;
    int64_t cap = paths <= 0 ? default_capacity(npix) : std::max<int64_t>(npix, (paths / npix) * npix);
    if (cap > int64_t(INT32_MAX) / 2) throw ApiError{HASTY_ERR_ARG, "too many paths in flight"};
    job->capacity = cap;   // the path buffers follow at the next render
    return HASTY_OK;
  });
}

int hasty_job_release_paths(hasty_job* job) {
  return guarded([&] {
    as_job(job);
    ck(cudaSetDevice(job->ctx->device), "cudaSetDevice");
    ck(cudaStreamSynchronize(job->stream), "sync");
    job->collect_events();
    release_path_buffers(*job, job->pd);
    release_path_buffers(*job, job->pd2);
    job->lane_free_valid[0] = job->lane_free_valid[1] = false;
    return HASTY_OK;
  });
}

int hasty_job_render_passes(hasty_job* job, int n_passes) {
  return guarded([&] {
    as_job(job);
    if (n_passes < 0) throw ApiError{HASTY_ERR_ARG, "negative pass count"};
    ck(cudaSetDevice(job->ctx->device), "cudaSetDevice");
    if (!job->pd.stats) throw ApiError{HASTY_ERR_ARG, "job was loaded for the multi-job engine only"};
    int64_t npix = int64_t(job->sd.width) * job->sd.height;
    if (n_passes > 0) ensure_paths(*job, std::min<int64_t>(job->capacity / npix, n_passes) * npix);
    int per_batch = int(std::max<int64_t>(1, job->pd.capacity / npix));
    int left = n_passes;
    if (left == 0) return HASTY_OK;
    // Device time of this call: from its first launch to its last
    // accumulation (consecutive calls chain on `stream`, so overlapped
    // batches are counted once).
    cudaEvent_t e0, e1;
    ck(cudaEventCreate(&e0), "event"); ck(cudaEventCreate(&e1), "event");
    ck(cudaEventRecord(e0, job->stream), "event record");
    if (job->lanes_wait_main) {
      ck(cudaEventRecord(job->main_ready, job->stream), "lane event");
      for (cudaStream_t ls : job->lane_stream) ck(cudaStreamWaitEvent(ls, job->main_ready, 0), "lane wait");
      job->lanes_wait_main = false;
    }
    while (left > 0) {
      if (job->stop.load()) break;
      int k = std::min(left, per_batch);
      // stage timing keeps one lane, so per-kernel times are not shared
      int lane = job->stage_timing ? 0 : job->next_lane;
      if (lane == 1) ensure_lane2(*job);
      if (job->lanes_wait_main) {          // lane 1 was just allocated on `stream`
        ck(cudaEventRecord(job->main_ready, job->stream), "lane event");
        ck(cudaStreamWaitEvent(job->lane_stream[1], job->main_ready, 0), "lane wait");
        job->lanes_wait_main = false;
      }
      render_batch(*job, k, lane, left > k);
      job->next_lane = lane ^ 1;
      left -= k;
    }
    ck(cudaEventRecord(e1, job->stream), "event record");
    job->pending_events.push_back({e0, e1, 0});
    if (job->stop.load()) throw ApiError{HASTY_ERR_STOPPED, "job stopped"};
    return HASTY_OK;
  });
}

int hasty_job_sync(hasty_job* job) {
  return guarded([&] {
    as_job(job);
    ck(cudaStreamSynchronize(job->stream), "cudaStreamSynchronize");
    job->collect_events();
    return HASTY_OK;
  });
}

int hasty_job_stop(hasty_job* job) {
  if (!job) return fail(HASTY_ERR_ARG, "null job handle");
  job->stop = true;
  return HASTY_OK;
}

int hasty_job_set_stage_timing(hasty_job* job, int on) {
  if (!job) return fail(HASTY_ERR_ARG, "null job handle");
  job->stage_timing = on != 0;
  return HASTY_OK;
}

int hasty_job_stats_get(hasty_job* job, hasty_stats* out) {
  return guarded([&] {
    as_job(job);
    if (!out) throw ApiError{HASTY_ERR_ARG, "null output"};
    ck(cudaStreamSynchronize(job->stream), "sync");
    job->collect_events();
    unsigned long long s[ST_COUNT];
    ck(cudaMemcpy(s, job->pd.stats, sizeof(s), cudaMemcpyDeviceToHost), "copy stats");
    out->rays = s[ST_RAYS]; out->shaded = s[ST_SHADED]; out->paths = s[ST_PATHS]; out->nan_samples = s[ST_NAN];
    out->media_overflow = s[ST_MEDIA_OVERFLOW]; out->trial_cap = s[ST_TRIAL_CAP];
    out->stack_overflow = s[ST_STACK_OVERFLOW];
    out->kernel_ms = job->kernel_ms;
    out->trace_ms = job->trace_ms; out->shade_ms = job->shade_ms;
    out->trace_launches = job->trace_launches; out->kernel_launches = job->kernel_launches;
    out->path_ms = job->path_ms; out->path_launches = job->path_launches;
    return HASTY_OK;
  });
}

int hasty_job_read_sums(hasty_job* job, int aov, double* host, size_t w, size_t h, int32_t* num_samples) {
  return guarded([&] {
    as_job(job);
    if (aov < 0 || aov > 2 || !host) throw ApiError{HASTY_ERR_ARG, "bad aov or buffer"};
    if (w != size_t(job->sd.width) || h != size_t(job->sd.height)) throw ApiError{HASTY_ERR_ARG, "buffer size does not match the frame"};
    ck(cudaStreamSynchronize(job->stream), "sync");
    job->collect_events();
    ck(cudaMemcpy(host, job->acc[aov], w * h * 3 * sizeof(double), cudaMemcpyDeviceToHost), "copy sums");
    if (num_samples) *num_samples = job->samples_done;
    return HASTY_OK;
  });
}

int hasty_job_read(hasty_job* job, int aov, float* host, size_t w, size_t h, int32_t* num_samples) {
  return guarded([&] {
    as_job(job);
    if (aov < 0 || aov > 2 || !host) throw ApiError{HASTY_ERR_ARG, "bad aov or buffer"};
    if (w != size_t(job->sd.width) || h != size_t(job->sd.height)) throw ApiError{HASTY_ERR_ARG, "buffer size does not match the frame"};
    int n = int(w * h * 3);
    float den = 1e-7f + float(job->samples_done);
    float scale = aov == HASTY_AOV_COLOR ? std::pow(2.0f, job->host.cam.exposure) : 1.0f;
    launch_estimate(job->acc[aov], n, den, scale, job->est, job->stream);
    ck(cudaGetLastError(), "estimate launch");
    ck(cudaMemcpyAsync(host, job->est, size_t(n) * sizeof(float), cudaMemcpyDeviceToHost, job->stream), "copy estimate");
    ck(cudaStreamSynchronize(job->stream), "sync");
    job->collect_events();
    if (num_samples) *num_samples = job->samples_done;
    return HASTY_OK;
  });
}

int hasty_job_write_outputs(hasty_job* job, const char* out_dir, int write_pfm) {
  return guarded([&] {
    as_job(job);
    if (!out_dir) throw ApiError{HASTY_ERR_ARG, "null directory"};
    struct stat sb;
    if (stat(out_dir, &sb) != 0 || !S_ISDIR(sb.st_mode)) throw ApiError{HASTY_ERR_IO, std::string("not a directory: ") + out_dir};
    size_t w = size_t(job->sd.width), h = size_t(job->sd.height);
    std::vector<float> img(w * h * 3);
    const char* names[3] = {"output", "outputNormal", "outputAlbedo"};
    for (int a = 0; a < 3; ++a) {
      int rc = hasty_job_read(job, a, img.data(), w, h, nullptr);
      if (rc != HASTY_OK) return rc;
      std::string base = std::string(out_dir) + "/" + names[a];
      if (!write_exr_rgb(base + ".exr", img.data(), int(w), int(h))) throw ApiError{HASTY_ERR_IO, "could not write " + base + ".exr"};
      if (write_pfm && !write_pfm_rgb(base + ".pfm", img.data(), int(w), int(h))) throw ApiError{HASTY_ERR_IO, "could not write " + base + ".pfm"};
    }
    return HASTY_OK;
  });
}

// Enqueues snapshot slot k of the AOVs in `mask`: the estimates on the job's
// stream behind every pass enqueued so far, their copy to pinned memory on
// the copy stream. Returns without waiting.
static void enqueue_snapshot(hasty_job& j, int k, uint32_t mask) {
  if (!j.acc[0]) throw ApiError{HASTY_ERR_ARG, "job was loaded for the multi-job engine only"};
  ck(cudaSetDevice(j.ctx->device), "cudaSetDevice");
  const size_t n = size_t(j.sd.width) * size_t(j.sd.height) * 3;
  hasty_job::Snapshot& s = j.snap[k];
  if (!s.dev) {
    s.dev = j.alloc<float>(3 * n);
    ck(cudaHostAlloc(reinterpret_cast<void**>(&s.host), 3 * n * sizeof(float), cudaHostAllocDefault), "cudaHostAlloc");
    ck(cudaEventCreateWithFlags(&s.copied, cudaEventDisableTiming), "event");
  }
  if (!j.copy_stream) {
    ck(cudaStreamCreateWithFlags(&j.copy_stream, cudaStreamNonBlocking), "stream");
    ck(cudaEventCreateWithFlags(&j.snap_est, cudaEventDisableTiming), "event");
  }
  // the slot's previous copy reads `dev`: the new estimates wait for it
  if (s.pending) ck(cudaStreamWaitEvent(j.stream, s.copied, 0), "snapshot wait");
  const float den = 1e-7f + float(j.samples_done);
  for (int a = 0; a < 3; ++a) {
    if (!(mask & (1u << a))) continue;
    const float scale = a == HASTY_AOV_COLOR ? std::pow(2.0f, j.host.cam.exposure) : 1.0f;
    launch_estimate(j.acc[a], int(n), den, scale, s.dev + size_t(a) * n, j.stream);
  }
  ck(cudaGetLastError(), "estimate launch");
  ck(cudaEventRecord(j.snap_est, j.stream), "event record");
  ck(cudaStreamWaitEvent(j.copy_stream, j.snap_est, 0), "snapshot wait");
  for (int a = 0; a < 3; ++a) {
    if (!(mask & (1u << a))) continue;
    ck(cudaMemcpyAsync(s.host + size_t(a) * n, s.dev + size_t(a) * n, n * sizeof(float), cudaMemcpyDeviceToHost,
                       j.copy_stream), "copy snapshot");
  }
  ck(cudaEventRecord(s.copied, j.copy_stream), "event record");
  s.pending = true;
  s.mask = mask;
  s.samples = j.samples_done;
}

static void check_out_dir(const char* out_dir) {
  if (!out_dir) throw ApiError{HASTY_ERR_ARG, "null directory"};
  struct stat sb;
  if (stat(out_dir, &sb) != 0 || !S_ISDIR(sb.st_mode)) throw ApiError{HASTY_ERR_IO, std::string("not a directory: ") + out_dir};
}

int hasty_job_snapshot(hasty_job* job, uint32_t aov_mask) {
  return guarded([&] {
    as_job(job);
    if (aov_mask == 0 || aov_mask > 7u) throw ApiError{HASTY_ERR_ARG, "bad aov mask"};
    enqueue_snapshot(*job, 0, aov_mask);
    return HASTY_OK;
  });
}

int hasty_job_snapshot_query(hasty_job* job, int* ready) {
  return guarded([&] {
    as_job(job);
    if (!ready) throw ApiError{HASTY_ERR_ARG, "null output"};
    const hasty_job::Snapshot& s = job->snap[0];
    if (!s.pending) throw ApiError{HASTY_ERR_ARG, "no snapshot was taken"};
    const cudaError_t e = cudaEventQuery(s.copied);
    if (e == cudaErrorNotReady) {
      (void)cudaGetLastError();        // "not ready" is an answer, not an error to report later
      *ready = 0;
    } else {
      ck(e, "snapshot query");
      *ready = 1;
    }
    return HASTY_OK;
  });
}

int hasty_job_snapshot_get(hasty_job* job, int aov, const float** out, int32_t* num_samples) {
  return guarded([&] {
    as_job(job);
    if (aov < 0 || aov > 2 || !out) throw ApiError{HASTY_ERR_ARG, "bad aov or output"};
    const hasty_job::Snapshot& s = job->snap[0];
    if (!s.pending) throw ApiError{HASTY_ERR_ARG, "no snapshot was taken"};
    if (!(s.mask & (1u << aov))) throw ApiError{HASTY_ERR_ARG, "aov not in the snapshot"};
    ck(cudaEventSynchronize(s.copied), "snapshot wait");
    *out = s.host + size_t(aov) * size_t(job->sd.width) * size_t(job->sd.height) * 3;
    if (num_samples) *num_samples = s.samples;
    return HASTY_OK;
  });
}

int hasty_job_write_outputs_async(hasty_job* job, const char* out_dir, int write_pfm) {
  return guarded([&] {
    as_job(job);
    check_out_dir(out_dir);
    if (job->writer.joinable()) job->writer.join();   // the previous write reads slot 1
    enqueue_snapshot(*job, 1, 7u);
    job->writer_rc = HASTY_OK;
    job->writer_err.clear();
    const int device = job->ctx->device;
    const int w = job->sd.width, h = job->sd.height;
    hasty_job::Snapshot* s = &job->snap[1];
    hasty_job* j = job;
    std::string dir(out_dir);
    job->writer = std::thread([j, s, device, w, h, dir, write_pfm] {
      const char* names[3] = {"output", "outputNormal", "outputAlbedo"};
      cudaError_t e = cudaSetDevice(device);
      if (e == cudaSuccess) e = cudaEventSynchronize(s->copied);
      if (e != cudaSuccess) {
        j->writer_rc = HASTY_ERR_CUDA;
        j->writer_err = std::string("snapshot wait: ") + cudaGetErrorString(e);
        return;
      }
      const size_t n = size_t(w) * size_t(h) * 3;
      for (int a = 0; a < 3; ++a) {
        const float* img = s->host + size_t(a) * n;
        const std::string base = dir + "/" + names[a];
        if (!write_exr_rgb(base + ".exr", img, w, h) || (write_pfm && !write_pfm_rgb(base + ".pfm", img, w, h))) {
          j->writer_rc = HASTY_ERR_IO;
          j->writer_err = "could not write " + base;
          return;
        }
      }
    });
    return HASTY_OK;
  });
}

int hasty_job_outputs_wait(hasty_job* job) {
  return guarded([&] {
    as_job(job);
    if (job->writer.joinable()) job->writer.join();
    if (job->writer_rc != HASTY_OK) {
      const int rc = job->writer_rc;
      job->writer_rc = HASTY_OK;
      throw ApiError{rc, job->writer_err};
    }
    return HASTY_OK;
  });
}

int hasty_debug_obj_digest(const char* path, int chunks, uint64_t* digest, int64_t* n_tris, int64_t* n_shapes) {
  return guarded([&] {
    if (!path || !digest || chunks < 0 || chunks > 4096) throw ApiError{HASTY_ERR_ARG, "bad argument"};
    *digest = obj_digest(path, size_t(chunks), n_tris, n_shapes);
    return HASTY_OK;
  });
}

int hasty_debug_intersect(hasty_job* job, const float* rays, size_t n, int32_t* tri, float* t, float* u, float* v) {
  return guarded([&] {
    as_job(job);
    if (n == 0) return HASTY_OK;
    if (!rays || !tri || !t || !u || !v) throw ApiError{HASTY_ERR_ARG, "null buffer"};
    if (n > size_t(INT32_MAX)) throw ApiError{HASTY_ERR_ARG, "too many rays"};
    float* dr = nullptr; float4* dh = nullptr;
    ck(cudaMalloc(&dr, n * 6 * sizeof(float)), "cudaMalloc rays");
    cudaError_t e = cudaMalloc(&dh, n * sizeof(float4));
    if (e != cudaSuccess) { cudaFree(dr); ck(e, "cudaMalloc hits"); }
    std::vector<float4> hh(n);
    cudaError_t err = cudaMemcpyAsync(dr, rays, n * 6 * sizeof(float), cudaMemcpyHostToDevice, job->stream);
    if (err == cudaSuccess) { launch_trace_rays(job->sd, dr, int(n), dh, job->stream); err = cudaGetLastError(); }
    if (err == cudaSuccess) err = cudaMemcpyAsync(hh.data(), dh, n * sizeof(float4), cudaMemcpyDeviceToHost, job->stream);
    if (err == cudaSuccess) err = cudaStreamSynchronize(job->stream);
    cudaFree(dr); cudaFree(dh);
    ck(err, "debug intersect");
    for (size_t i = 0; i < n; ++i) {
      int32_t id; std::memcpy(&id, &hh[i].w, 4);
      tri[i] = id; t[i] = hh[i].x; u[i] = hh[i].y; v[i] = hh[i].z;
    }
    return HASTY_OK;
  });
}

int hasty_debug_wide_emit_check(int device, const char* job_path, int64_t* info, int32_t* identical) {
  return guarded([&] {
    if (!job_path || !identical) throw ApiError{HASTY_ERR_ARG, "null argument"};
    ck(cudaSetDevice(device), "cudaSetDevice");
    HostScene h;
    load_render_job(job_path, h);
    *identical = check_wide_emit_gpu(h.tri_pos.data(), h.n_tris(), info) ? 1 : 0;
    return HASTY_OK;
  });
}

int hasty_debug_host_trace(const char* job_path, int kind, const float* rays, size_t n, int32_t* tri, float* t, float* u,
                           float* v, int64_t* info) {
  return guarded([&] {
    if (!job_path || (n && (!rays || !tri || !t || !u || !v)) || (kind != 0 && kind != 1))
      throw ApiError{HASTY_ERR_ARG, "bad argument"};
    HostScene h;
    load_render_job(job_path, h);
    BvhHost bvh;
    if (kind == 0) build_bvh_binary(h.tri_pos.data(), h.n_tris(), 4, bvh);
    else build_bvh_wide(h.tri_pos.data(), h.n_tris(), bvh);
    std::vector<float4> nodes(bvh.nodes.size() / 4), tris(bvh.tris.size() / 4);
    std::memcpy(nodes.data(), bvh.nodes.data(), bvh.nodes.size() * sizeof(float));
    std::memcpy(tris.data(), bvh.tris.data(), bvh.tris.size() * sizeof(float));
    std::vector<float4> hits(n);
    host_trace_rays(kind, nodes.data(), tris.data(), rays, int64_t(n), hits.data());
    for (size_t i = 0; i < n; ++i) {
      int32_t id; std::memcpy(&id, &hits[i].w, 4);
      tri[i] = id; t[i] = hits[i].x; u[i] = hits[i].y; v[i] = hits[i].z;
    }
    if (info) { info[0] = int64_t(h.n_tris()); info[1] = int64_t(nodes.size() / (kind == 1 ? 5 : 4)); info[2] = bvh.depth; }
    return HASTY_OK;
  });
}

int hasty_debug_tri_ids(hasty_job* job, int32_t* geom, int32_t* prim, size_t n) {
  return guarded([&] {
    as_job(job);
    if (n != job->host.tri_attr.size()) throw ApiError{HASTY_ERR_ARG, "n must equal the triangle count"};
    for (size_t i = 0; i < n; ++i) { geom[i] = int32_t(job->host.tri_attr[i].geom); prim[i] = int32_t(job->host.tri_attr[i].prim); }
    return HASTY_OK;
  });
}

int hasty_debug_bounds_status(uint32_t* flags) {
#ifdef HASTY_DEBUG_BOUNDS
  if (!flags) return fail(HASTY_ERR_ARG, "null argument");
  *flags = hasty::bounds_status_integrator() | hasty::bounds_status_trace() | hasty::bounds_status_photon();
  return HASTY_OK;
#else
  (void)flags;
  return fail(HASTY_ERR_MISSING, "bounds checks are compiled into the bounds-checked build only "
                                 "(python -m hastyrenderer_gb300.build --debug-bounds)");
#endif
}

int hasty_debug_bsdf(int which, const float* in, size_t n_cases, const uint32_t* replay, size_t n_replay, float* out) {
  return guarded([&] {
    if (which < 0 || which > 2 || !in || !out || (n_replay && !replay)) throw ApiError{HASTY_ERR_ARG, "bad argument"};
    if (n_cases == 0) return HASTY_OK;
    if (n_replay == 0) throw ApiError{HASTY_ERR_ARG, "replay stream must not be empty"};
    float *din = nullptr, *dout = nullptr; uint32_t* drep = nullptr;
    ck(cudaMalloc(&din, n_cases * 33 * sizeof(float)), "cudaMalloc");
    cudaError_t err = cudaMalloc(&dout, n_cases * 12 * sizeof(float));
    if (err == cudaSuccess) err = cudaMalloc(&drep, n_cases * n_replay * sizeof(uint32_t));
    if (err == cudaSuccess) err = cudaMemcpy(din, in, n_cases * 33 * sizeof(float), cudaMemcpyHostToDevice);
    if (err == cudaSuccess) err = cudaMemcpy(drep, replay, n_cases * n_replay * sizeof(uint32_t), cudaMemcpyHostToDevice);
    if (err == cudaSuccess) { launch_debug_bsdf(which, din, int(n_cases), drep, int(n_replay), dout, 0); err = cudaGetLastError(); }
    if (err == cudaSuccess) err = cudaMemcpy(out, dout, n_cases * 12 * sizeof(float), cudaMemcpyDeviceToHost);
    cudaFree(din); cudaFree(dout); cudaFree(drep);
    ck(err, "debug bsdf");
    return HASTY_OK;
  });
}

}  // extern "C"
