// Photon mapper, host side and C ABI (include/hasty_gpu.h, hasty_pm_*): the
// loop of the reference's renderPhotonThread (core/src/PhotonMapping.cpp:
// 814-935) for one render thread, with the photon tracing and the per-pixel
// gather on the GPU (photon.cu). The host keeps what the reference computes
// sequentially in float: the footprint angle of each pixel, the fill of
// pixels without a footprint, the hash-cell size, and the photon map's cell
// order (photons sorted by cell, then by emission index and depth, which is
// the order the reference's hash cells list them in).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

#include "job.h"
#include "photon.h"
#include "scene_load.h"

namespace hasty {

struct PmDev {
  uint32_t W = 0, H = 0;
  bool initialised = false;
  uint32_t iteration = 0;
  PmPixelsDev px{};
  unsigned long long* stats = nullptr;     // [0] media overflow, [1] trial cap
  // photon buffers (grown on demand)
  PhotonRec* append = nullptr;
  size_t append_cap = 0;
  uint32_t* append_count = nullptr;
  uint32_t* fetch = nullptr;               // emission counter of the photon kernel
  uint8_t* stored = nullptr;
  size_t stored_cap = 0;
  PhotonRec* sorted = nullptr;
  size_t sorted_cap = 0;
  int4* cells = nullptr;
  size_t cells_cap = 0;
  int32_t* cell_count = nullptr;
  size_t counts_cap = 0;
  int32_t* n_cells = nullptr;
  // map build (photon_build.cu)
  PmStatus* status = nullptr;              // device
  PmStatus* status_host = nullptr;         // pinned
  uint32_t* base = nullptr;                // first slot of each emission
  size_t base_cap = 0;
  uint32_t* scratch = nullptr;
  size_t scratch_cap = 0;
  uint32_t* src = nullptr;                 // append index of each slot
  size_t src_cap = 0;
  int32_t* coords = nullptr;               // hash cell of each slot, three planes
  size_t coords_cap = 0;
  uint32_t* perm[2] = {nullptr, nullptr};
  size_t perm_cap[2] = {0, 0};
  uint32_t* flag = nullptr;
  size_t flag_cap = 0;
  uint32_t* cell_of = nullptr;
  size_t cell_of_cap = 0;
  uint32_t* hist = nullptr;
  size_t hist_cap = 0;
  ~PmDev() { if (status_host) cudaFreeHost(status_host); }
  std::vector<float> radii;                // host copy of the radius image
  // last iteration
  uint64_t emitted = 0, photons = 0;
  float cell = 0.0f;
  double device_ms = 0.0, host_ms = 0.0, photon_ms = 0.0, gather_ms = 0.0, cell_ms = 0.0, map_ms = 0.0;
  uint64_t last_emitted = 0;               // sizes the next iteration's first photon batch
};

void destroy_pm(PmDev* pm) { delete pm; }

namespace {


// Camera::computeRayAngle (Camera.cpp:83-98); q = tan(fov / 2) as the camera
// evaluates it.
float ray_angle(float q, float x, float y, float W, float H) {
  float lx1 = (x + 0.5f - 0.5f * W) / W * 2.0f;
  float ly1 = (y + 0.5f - 0.5f * H) / W * 2.0f;
  float lx2 = (x - 0.5f - 0.5f * W) / W * 2.0f;
  float ly2 = (y - 0.5f - 0.5f * H) / W * 2.0f;
  float ax = std::fabs(std::atan(q * lx1) - std::atan(q * lx2));
  float ay = std::fabs(std::atan(q * ly1) - std::atan(q * ly2));
  return 0.5f * ax + 0.5f * ay;
}

// getCloseNonNegative (PhotonMapping.cpp:653-678), img[x + y * W]; the
// reference's fourth candidate per step is computed and never tested.
float close_non_negative(const std::vector<float>& img, int W, int H, int i, int j) {
  auto inside = [&](int x, int y) { return x >= 0 && y >= 0 && x < W && y < H; };
  auto at = [&](int x, int y) { return img[size_t(y) * size_t(W) + size_t(x)]; };
  for (int k = 1; k < std::max(H, W); ++k) {
    for (int m = 0; m <= k * 2; m++) {
      int i2 = i - k, j2 = j - k + m;
      if (inside(i2, j2) && at(i2, j2) > 0.0f) return at(i2, j2);
      i2 = i - k + m; j2 = j - k;
      if (inside(i2, j2) && at(i2, j2) > 0.0f) return at(i2, j2);
      i2 = i + k; j2 = j - k + m;
      if (inside(i2, j2) && at(i2, j2) > 0.0f) return at(i2, j2);
    }
  }
  return 1e-3f;
}

// computeCellSize (PhotonMapping.cpp:522-576): float sums in the reference's
// order (x outer, y inner).
float cell_size_for(const std::vector<float>& radii, uint32_t W, uint32_t H) {
  auto p3 = [](float f) { return f * (f * f); };     // powci<3>
  float sum = 0.0f;
  for (uint32_t i = 0; i < W; i++)
    for (uint32_t j = 0; j < H; j++) sum += radii[size_t(j) * W + i];
  const float a = 5.0f, density = 1e5f;
  float cs = sum / float(W * H);
  auto cost = [&](float c) {
    float s = 0.0f;
    for (uint32_t i = 0; i < W; i++)
      for (uint32_t j = 0; j < H; j++) {
        float r = radii[size_t(j) * W + i];
        s += a * p3(r / c) + p3(std::max(r, c)) * density;
      }
    return s;
  };
  // The reference evaluates cost(cs), then up to 10 trials cs *= 1.5 while
  // they improve, then up to 10 trials cs *= 0.6666. The trial values along
  // that path are fixed in advance, so their costs are evaluated at once on
  // several threads and the same decisions are taken afterwards.
  auto costs_of = [&](const std::vector<float>& c) {
    std::vector<float> out(c.size());
    std::vector<std::thread> th;
    for (size_t k = 1; k < c.size(); ++k) th.emplace_back([&, k] { out[k] = cost(c[k]); });
    if (!c.empty()) out[0] = cost(c[0]);
    for (std::thread& t : th) t.join();
    return out;
  };
  std::vector<float> up(11);
  up[0] = cs;
  for (int k = 1; k <= 10; ++k) up[size_t(k)] = up[size_t(k) - 1] * 1.5f;
  std::vector<float> cu = costs_of(up);
  float best = cu[0];
  size_t at = 0;
  for (size_t k = 1; k <= 10; ++k) {
    if (!(cu[k] < best)) break;
    best = cu[k]; at = k;
  }
  cs = up[at];
  std::vector<float> down(10);
  down[0] = cs * 0.6666f;
  for (int k = 1; k < 10; ++k) down[size_t(k)] = down[size_t(k) - 1] * 0.6666f;
  std::vector<float> cd = costs_of(down);
  for (size_t k = 0; k < 10; ++k) {
    if (!(cd[k] < best)) break;
    best = cd[k]; cs = down[k];
  }
  return cs;
}

template <class T>
T* grow(hasty_job& j, T* old, size_t& cap, size_t need, size_t keep) {
  if (need <= cap) return old;
  size_t n = std::max(need, cap + cap / 2);
  T* p = j.alloc<T>(n);
  if (old && keep) ck(cudaMemcpyAsync(p, old, keep * sizeof(T), cudaMemcpyDeviceToDevice, j.stream), "grow");
  if (old) { ck(cudaStreamSynchronize(j.stream), "grow"); j.release(old); }
  cap = n;
  return p;
}

PmDev& pm_state(hasty_job& j) {
  if (!j.pm) {
    auto* pm = new PmDev();
    j.pm = pm;
    const uint32_t W = uint32_t(j.sd.width), H = uint32_t(j.sd.height);
    const size_t n = size_t(W) * H;
    pm->W = W; pm->H = H;
    pm->px.radius = j.alloc<float>(n);
    pm->px.N = j.alloc<float>(n);
    pm->px.Ne = j.alloc<float>(n);
    pm->px.flux = j.alloc<float4>(n);
    pm->px.lsum = j.alloc<float4>(n);
    pm->px.radii = j.alloc<float>(n);
    pm->px.color = j.alloc<float>(3 * n);
    pm->px.normal = j.alloc<float>(3 * n);
    pm->px.albedo = j.alloc<float>(3 * n);
    pm->stats = j.alloc<unsigned long long>(2);
    pm->append_count = j.alloc<uint32_t>(1);
    pm->fetch = j.alloc<uint32_t>(1);
    pm->n_cells = j.alloc<int32_t>(1);
    pm->status = j.alloc<PmStatus>(1);
    ck(cudaHostAlloc(reinterpret_cast<void**>(&pm->status_host), sizeof(PmStatus), cudaHostAllocDefault), "cudaHostAlloc");
  }
  return *j.pm;
}

// Pixel statistics cleared and the radius image set up (renderPhotonThread,
// PhotonMapping.cpp:828-833: footprint radii x 10 with a surface light, else 1).
void pm_init(hasty_job& j, PmDev& pm) {
  const uint32_t W = pm.W, H = pm.H;
  const size_t n = size_t(W) * H;
  std::vector<float> minus1(n, -1.0f);
  ck(cudaMemcpyAsync(pm.px.radius, minus1.data(), n * sizeof(float), cudaMemcpyHostToDevice, j.stream), "pm init");
  ck(cudaMemsetAsync(pm.px.N, 0, n * sizeof(float), j.stream), "pm init");
  ck(cudaMemsetAsync(pm.px.Ne, 0, n * sizeof(float), j.stream), "pm init");
  ck(cudaMemsetAsync(pm.px.flux, 0, n * sizeof(float4), j.stream), "pm init");
  ck(cudaMemsetAsync(pm.px.lsum, 0, n * sizeof(float4), j.stream), "pm init");
  ck(cudaMemsetAsync(pm.px.color, 0, 3 * n * sizeof(float), j.stream), "pm init");
  ck(cudaMemsetAsync(pm.px.normal, 0, 3 * n * sizeof(float), j.stream), "pm init");
  ck(cudaMemsetAsync(pm.px.albedo, 0, 3 * n * sizeof(float), j.stream), "pm init");
  ck(cudaMemsetAsync(pm.stats, 0, 2 * sizeof(unsigned long long), j.stream), "pm init");
  pm.radii.assign(n, 1.0f);
  if (j.sd.n_light_tris > 0) {
    float* dist = j.alloc<float>(n);
    launch_pm_footprint(j.sd, j.seed, dist, j.stream);
    ck(cudaGetLastError(), "footprint launch");
    std::vector<float> d(n);
    ck(cudaMemcpyAsync(d.data(), dist, n * sizeof(float), cudaMemcpyDeviceToHost, j.stream), "footprint");
    ck(cudaStreamSynchronize(j.stream), "footprint");
    j.release(dist);
    const float q = j.sd.cam.q;
    for (uint32_t y = 0; y < H; y++)
      for (uint32_t x = 0; x < W; x++) {
        const size_t p = size_t(y) * W + x;
        float fp = -1.0f;                       // computeRadiusPixelFootPrint's default
        if (d[p] >= 0.0f) {
          float angle = ray_angle(q, float(x) + 0.5f, float(y) + 0.5f, float(W), float(H));
          fp = 0.5f * d[p] * std::tan(angle);
        }
        pm.radii[p] = 10.0f * fp;
      }
    for (uint32_t y = 0; y < H; y++)
      for (uint32_t x = 0; x < W; x++)
        if (pm.radii[size_t(y) * W + x] < 0.0f)
          pm.radii[size_t(y) * W + x] = close_non_negative(pm.radii, int(W), int(H), int(x), int(y));
  }
  ck(cudaMemcpyAsync(pm.px.radii, pm.radii.data(), n * sizeof(float), cudaMemcpyHostToDevice, j.stream), "radii");
  ck(cudaStreamSynchronize(j.stream), "pm init");
  pm.initialised = true;
  pm.iteration = 0;
}

// One iteration of renderPhotonThread's loop (PhotonMapping.cpp:848-931).
// The GPU traces photon batches and scans their store counts; the hash-cell
// size is computed on the host meanwhile (it needs only the radii of the
// previous iteration); then the photon map is built and gathered on the GPU.
void pm_iteration(hasty_job& j, PmDev& pm) {
  const uint32_t W = pm.W, H = pm.H, t = pm.iteration;
  const auto h0 = std::chrono::steady_clock::now();
  cudaEvent_t ev[6];
  for (cudaEvent_t& e : ev) ck(cudaEventCreate(&e), "event");
  auto elapsed = [&](int a, int b) {
    float ms = 0.f;
    ck(cudaEventElapsedTime(&ms, ev[a], ev[b]), "event time");
    return double(ms);
  };
  double photon_ms = 0.0, cell_ms = 0.0;
  float cell = 0.0f;
  bool have_cell = false;
  auto compute_cell = [&] {
    const auto c0 = std::chrono::steady_clock::now();
    cell = cell_size_for(pm.radii, W, H);
    cell_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - c0).count();
    have_cell = true;
  };
  uint32_t emitted = 0, kept = 0, appended = 0;
  const int count_threshold = int(0.5f * float(H) * float(W));
  if (j.sd.n_light_tris > 0 && count_threshold > 0) {
    const int trace_threshold = int(10.f * float(H) * float(W));
    const int depth_slots = std::max(1, j.sd.max_depth - 1);   // photons one emitted photon can store
    const float min_q = 1.0f - std::pow(0.1f, 1.0f / j.sd.max_depth);
    uint32_t first = 0;
    // first batch: what the previous iteration needed (+10%), else 2x the stored target
    size_t chunk = std::max<size_t>(size_t(1) << 16, pm.last_emitted ? size_t(pm.last_emitted * 1.1) + 1024
                                                                     : 2 * size_t(count_threshold));
    ck(cudaMemsetAsync(pm.append_count, 0, sizeof(uint32_t), j.stream), "photon count");
    ck(cudaMemsetAsync(pm.status, 0, sizeof(PmStatus), j.stream), "photon status");
    for (;;) {
      const uint32_t n = uint32_t(std::min<uint64_t>(chunk, uint64_t(trace_threshold) - first));
      pm.append = grow(j, pm.append, pm.append_cap, size_t(appended) + size_t(n) * depth_slots, appended);
      pm.stored = grow(j, pm.stored, pm.stored_cap, n, 0);
      pm.base = grow(j, pm.base, pm.base_cap, size_t(first) + n, first);
      pm.scratch = grow(j, pm.scratch, pm.scratch_cap, size_t(n) / 2048 + 2, 0);
      PmEmitOut out{pm.append, pm.append_count, uint32_t(pm.append_cap), pm.stored, pm.stats, pm.fetch};
      ck(cudaEventRecord(ev[0], j.stream), "event");
      launch_pm_emit(j.sd, j.seed, t, first, n, min_q, out, j.stream);
      launch_pm_emit_scan(pm.stored, n, first, uint32_t(count_threshold), pm.base, pm.scratch, pm.status, j.stream);
      ck(cudaGetLastError(), "photon launch");
      ck(cudaEventRecord(ev[1], j.stream), "event");
      ck(cudaMemcpyAsync(&pm.status->appended, pm.append_count, sizeof(uint32_t), cudaMemcpyDeviceToDevice, j.stream),
         "photon count");
      ck(cudaMemcpyAsync(pm.status_host, pm.status, sizeof(PmStatus), cudaMemcpyDeviceToHost, j.stream), "photon status");
      ck(cudaEventRecord(ev[2], j.stream), "event");
      if (!have_cell) compute_cell();           // overlaps the photon tracing
      ck(cudaEventSynchronize(ev[2]), "photons");
      photon_ms += elapsed(0, 1);
      appended = pm.status_host->appended;
      if (appended > pm.append_cap) throw ApiError{HASTY_ERR_CUDA, "photon buffer overflow"};
      // the reference emits photon i while fewer than count_threshold are stored
      if (pm.status_host->done) { emitted = pm.status_host->emitted; kept = pm.status_host->kept; break; }
      first += n;
      if (first >= uint32_t(trace_threshold)) { emitted = first; kept = pm.status_host->cum; break; }
      chunk *= 2;
    }
  }
  if (!have_cell) compute_cell();
  // Photon map: the kept photons in emission order (slot = the emission's
  // first slot + the photon's index within it), then a stable radix sort by
  // hash cell, so each cell lists its photons in the order the reference
  // stored them.
  const uint32_t cap = std::max<uint32_t>(kept, 1u);
  const uint32_t tiles = pm_sort_tiles(cap);
  pm.src = grow(j, pm.src, pm.src_cap, cap, 0);
  pm.perm[0] = grow(j, pm.perm[0], pm.perm_cap[0], cap, 0);
  pm.perm[1] = grow(j, pm.perm[1], pm.perm_cap[1], cap, 0);
  pm.flag = grow(j, pm.flag, pm.flag_cap, cap, 0);
  pm.cell_of = grow(j, pm.cell_of, pm.cell_of_cap, cap, 0);
  pm.hist = grow(j, pm.hist, pm.hist_cap, size_t(256) * tiles, 0);
  pm.scratch = grow(j, pm.scratch, pm.scratch_cap, size_t(cap) / 2048 + size_t(tiles) / 8 + 2, 0);
  pm.sorted = grow(j, pm.sorted, pm.sorted_cap, cap, 0);
  pm.cells = grow(j, pm.cells, pm.cells_cap, cap, 0);
  pm.cell_count = grow(j, pm.cell_count, pm.counts_cap, cap, 0);
  // coordinates: three planes of `coords_cap / 3` slots
  if (pm.coords_cap < 3 * size_t(cap)) {
    j.release(pm.coords);
    pm.coords = nullptr;
    pm.coords_cap = 0;
    pm.coords = grow(j, pm.coords, pm.coords_cap, 3 * size_t(cap), 0);
  }
  const uint32_t plane = uint32_t(pm.coords_cap / 3);
  ck(cudaEventRecord(ev[3], j.stream), "event");
  launch_pm_place(pm.append, appended, pm.base, emitted, pm.status, cell, pm.src, pm.coords, plane, j.stream);
  ck(cudaGetLastError(), "photon map launch");
  const uint32_t* perm = nullptr;
  if (kept > 1) {
    ck(cudaMemcpyAsync(pm.status_host, pm.status, sizeof(PmStatus), cudaMemcpyDeviceToHost, j.stream), "cell bounds");
    ck(cudaStreamSynchronize(j.stream), "cell bounds");
    int which = 0;
    for (int axis = 2; axis >= 0; --axis) {      // least significant key first: z, y, x
      const uint32_t range = uint32_t(int64_t(pm.status_host->hi[axis]) - int64_t(pm.status_host->lo[axis]));
      for (int shift = 0; shift < 32 && (range >> shift) != 0; shift += 8) {
        launch_pm_sort_pass(pm.coords + size_t(axis) * plane, pm.status_host->lo[axis], shift, kept, perm,
                            pm.perm[which], pm.hist, pm.scratch, j.stream);
        perm = pm.perm[which];
        which ^= 1;
      }
    }
  }
  launch_pm_cells(pm.append, pm.src, pm.coords, plane, kept, perm, pm.sorted, pm.flag, pm.cell_of, pm.scratch,
                  pm.cells, pm.cell_count, pm.n_cells, j.stream);
  ck(cudaGetLastError(), "photon map launch");
  ck(cudaEventRecord(ev[4], j.stream), "event");
  PmMapDev map{pm.sorted, pm.cells, pm.cell_count, pm.n_cells, cell};
  const float ox = halton_value(2, t), oy = halton_value(3, t);
  launch_pm_gather(j.sd, map, pm.px, j.seed, t, ox, oy, int(emitted), pm.stats, j.stream);
  ck(cudaGetLastError(), "gather launch");
  ck(cudaEventRecord(ev[5], j.stream), "event");
  const size_t n = size_t(W) * H;
  ck(cudaMemcpyAsync(pm.radii.data(), pm.px.radii, n * sizeof(float), cudaMemcpyDeviceToHost, j.stream), "radii");
  ck(cudaStreamSynchronize(j.stream), "radii");
  const double map_ms = elapsed(3, 4), gather_ms = elapsed(4, 5);
  for (cudaEvent_t e : ev) cudaEventDestroy(e);
  const double dev_ms = photon_ms + map_ms + gather_ms;
  pm.emitted = emitted;
  pm.photons = kept;
  pm.cell = cell;
  pm.iteration = t + 1;
  pm.device_ms += dev_ms;
  pm.photon_ms += photon_ms;
  pm.gather_ms += gather_ms;
  pm.map_ms += map_ms;
  pm.cell_ms += cell_ms;
  pm.last_emitted = emitted;
  pm.host_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - h0).count() - dev_ms;
}

hasty_job* pm_job(hasty_job* j) {
  if (!j) throw ApiError{HASTY_ERR_ARG, "null job handle"};
  if (j->sd.max_depth > kPmMaxDepth)
    throw ApiError{HASTY_ERR_ARG, "photon mapping supports max_depth <= " + std::to_string(kPmMaxDepth)};
  ck(cudaSetDevice(j->ctx->device), "cudaSetDevice");
  return j;
}

}  // namespace
}  // namespace hasty

using namespace hasty;

extern "C" {

int hasty_pm_render(hasty_job* job, int iterations) {
  return guarded([&] {
    pm_job(job);
    if (iterations < 0) throw ApiError{HASTY_ERR_ARG, "negative iteration count"};
    ck(cudaStreamSynchronize(job->stream), "sync");
    PmDev& pm = pm_state(*job);
    if (!pm.initialised) pm_init(*job, pm);
    for (int k = 0; k < iterations; ++k) {
      if (job->stop.load()) throw ApiError{HASTY_ERR_STOPPED, "job stopped"};
      pm_iteration(*job, pm);
    }
    return HASTY_OK;
  });
}

int hasty_pm_reset(hasty_job* job) {
  return guarded([&] {
    pm_job(job);
    if (job->pm) job->pm->initialised = false;
    return HASTY_OK;
  });
}

int hasty_pm_read(hasty_job* job, int aov, float* host, size_t w, size_t h) {
  return guarded([&] {
    pm_job(job);
    if (aov < 0 || aov > 2 || !host) throw ApiError{HASTY_ERR_ARG, "bad aov or buffer"};
    if (w != size_t(job->sd.width) || h != size_t(job->sd.height)) throw ApiError{HASTY_ERR_ARG, "buffer size does not match the frame"};
    if (!job->pm || !job->pm->initialised) throw ApiError{HASTY_ERR_ARG, "no photon-mapping iteration rendered"};
    const float* src = aov == 0 ? job->pm->px.color : (aov == 1 ? job->pm->px.normal : job->pm->px.albedo);
    ck(cudaMemcpyAsync(host, src, w * h * 3 * sizeof(float), cudaMemcpyDeviceToHost, job->stream), "read");
    ck(cudaStreamSynchronize(job->stream), "read");
    if (aov == HASTY_AOV_COLOR) {            // image *= 2^exposure, PhotonMappingViewer.cpp:154
      const float scale = std::pow(2.0f, job->host.cam.exposure);
      for (size_t k = 0; k < w * h * 3; ++k) host[k] *= scale;
    }
    return HASTY_OK;
  });
}

int hasty_pm_read_radii(hasty_job* job, float* host, size_t w, size_t h) {
  return guarded([&] {
    pm_job(job);
    if (!host) throw ApiError{HASTY_ERR_ARG, "null buffer"};
    if (w != size_t(job->sd.width) || h != size_t(job->sd.height)) throw ApiError{HASTY_ERR_ARG, "buffer size does not match the frame"};
    if (!job->pm || !job->pm->initialised) throw ApiError{HASTY_ERR_ARG, "no photon-mapping iteration rendered"};
    std::memcpy(host, job->pm->radii.data(), w * h * sizeof(float));
    return HASTY_OK;
  });
}

int hasty_pm_stats_get(hasty_job* job, hasty_pm_stats* out) {
  return guarded([&] {
    pm_job(job);
    if (!out) throw ApiError{HASTY_ERR_ARG, "null argument"};
    std::memset(out, 0, sizeof(*out));
    if (!job->pm) return HASTY_OK;
    const PmDev& pm = *job->pm;
    out->iterations = int32_t(pm.iteration);
    out->photons_emitted = int64_t(pm.emitted);
    out->photons_stored = int64_t(pm.photons);
    out->cell_size = pm.cell;
    out->device_ms = pm.device_ms;
    out->host_ms = pm.host_ms;
    unsigned long long st[2] = {0, 0};
    if (pm.stats) {
      ck(cudaMemcpyAsync(st, pm.stats, sizeof(st), cudaMemcpyDeviceToHost, job->stream), "stats");
      ck(cudaStreamSynchronize(job->stream), "stats");
    }
    out->media_overflow = st[0];
    out->trial_cap = st[1];
    out->photon_ms = pm.photon_ms;
    out->gather_ms = pm.gather_ms;
    out->cell_ms = pm.cell_ms;
    out->map_ms = pm.map_ms;
    return HASTY_OK;
  });
}

int hasty_debug_pm_map(hasty_job* job, float* xyz, uint32_t* emission, uint32_t* index, int32_t* cells,
                       int64_t* n_photons, int64_t* n_cells, float* cell) {
  return guarded([&] {
    pm_job(job);
    if (!n_photons || !n_cells || !cell) throw ApiError{HASTY_ERR_ARG, "null count output"};
    if (!job->pm || !job->pm->initialised || job->pm->iteration == 0)
      throw ApiError{HASTY_ERR_ARG, "no photon-mapping iteration rendered"};
    const PmDev& pm = *job->pm;
    int32_t nc = 0;
    ck(cudaMemcpyAsync(&nc, pm.n_cells, sizeof(int32_t), cudaMemcpyDeviceToHost, job->stream), "map");
    ck(cudaStreamSynchronize(job->stream), "map");
    *n_photons = int64_t(pm.photons);
    *n_cells = nc;
    *cell = pm.cell;
    if (xyz && emission && index && pm.photons) {
      std::vector<PhotonRec> ph(pm.photons);
      ck(cudaMemcpyAsync(ph.data(), pm.sorted, ph.size() * sizeof(PhotonRec), cudaMemcpyDeviceToHost, job->stream), "map");
      ck(cudaStreamSynchronize(job->stream), "map");
      for (size_t q = 0; q < ph.size(); ++q) {
        xyz[3 * q] = ph[q].xn.x; xyz[3 * q + 1] = ph[q].xn.y; xyz[3 * q + 2] = ph[q].xn.z;
        std::memcpy(&emission[q], &ph[q].wi.w, 4);
        std::memcpy(&index[q], &ph[q].flux.w, 4);
      }
    }
    if (cells && nc > 0) {
      std::vector<int4> c(static_cast<size_t>(nc));
      std::vector<int32_t> cnt(static_cast<size_t>(nc));
      ck(cudaMemcpyAsync(c.data(), pm.cells, c.size() * sizeof(int4), cudaMemcpyDeviceToHost, job->stream), "map");
      ck(cudaMemcpyAsync(cnt.data(), pm.cell_count, cnt.size() * sizeof(int32_t), cudaMemcpyDeviceToHost, job->stream), "map");
      ck(cudaStreamSynchronize(job->stream), "map");
      for (size_t k = 0; k < c.size(); ++k) {
        cells[5 * k] = c[k].x; cells[5 * k + 1] = c[k].y; cells[5 * k + 2] = c[k].z;
        cells[5 * k + 3] = c[k].w; cells[5 * k + 4] = cnt[k];
      }
    }
    return HASTY_OK;
  });
}

}  // extern "C"
