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
  uint8_t* stored = nullptr;
  size_t stored_cap = 0;
  PhotonRec* sorted = nullptr;
  size_t sorted_cap = 0;
  int4* cells = nullptr;
  size_t cells_cap = 0;
  int32_t* cell_count = nullptr;
  size_t counts_cap = 0;
  std::vector<float> radii;                // host copy of the radius image
  // last iteration
  uint64_t emitted = 0, photons = 0;
  float cell = 0.0f;
  double device_ms = 0.0, host_ms = 0.0, photon_ms = 0.0, gather_ms = 0.0;
  uint64_t last_emitted = 0;               // sizes the next iteration's first photon batch
};

void destroy_pm(PmDev* pm) { delete pm; }

namespace {

int32_t floor_i32(double x) { int i = (int)x; return i - (i > x); }     // VMath.h floor_int32

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
void pm_iteration(hasty_job& j, PmDev& pm) {
  const uint32_t W = pm.W, H = pm.H, t = pm.iteration;
  const auto h0 = std::chrono::steady_clock::now();
  double dev_ms = 0.0;
  cudaEvent_t e0, e1;
  ck(cudaEventCreate(&e0), "event"); ck(cudaEventCreate(&e1), "event");
  double photon_ms = 0.0, gather_ms = 0.0;
  auto time_device = [&](double& part, auto&& fn) {
    ck(cudaEventRecord(e0, j.stream), "event");
    fn();
    ck(cudaEventRecord(e1, j.stream), "event");
    ck(cudaEventSynchronize(e1), "event");
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    dev_ms += ms;
    part += ms;
  };
  const float cell = cell_size_for(pm.radii, W, H);
  uint64_t emitted = 0, kept = 0;
  std::vector<uint64_t> base;          // first emission-order slot of each emitted photon
  std::vector<PhotonRec> host_ph;
  if (j.sd.n_light_tris > 0) {
    const int trace_threshold = int(10.f * float(H) * float(W));
    const int count_threshold = int(0.5f * float(H) * float(W));
    const int depth_slots = std::max(1, j.sd.max_depth - 1);   // photons one emitted photon can store
    const float min_q = 1.0f - std::pow(0.1f, 1.0f / j.sd.max_depth);
    uint64_t first = 0, cum = 0;
    uint32_t appended = 0;
    base.clear();
    // first batch: what the previous iteration needed (+10%), else 2x the stored target
    size_t chunk = std::max<size_t>(size_t(1) << 16, pm.last_emitted ? size_t(pm.last_emitted * 1.1) + 1024
                                                                     : 2 * size_t(count_threshold));
    ck(cudaMemsetAsync(pm.append_count, 0, sizeof(uint32_t), j.stream), "photon count");
    bool done = count_threshold <= 0;
    std::vector<uint8_t> stored;
    while (!done && first < uint64_t(trace_threshold)) {
      const uint32_t n = uint32_t(std::min<uint64_t>(chunk, uint64_t(trace_threshold) - first));
      pm.append = grow(j, pm.append, pm.append_cap, size_t(appended) + size_t(n) * depth_slots, appended);
      pm.stored = grow(j, pm.stored, pm.stored_cap, n, 0);
      PmEmitOut out{pm.append, pm.append_count, uint32_t(pm.append_cap), pm.stored, pm.stats};
      time_device(photon_ms, [&] {
        launch_pm_emit(j.sd, j.seed, t, uint32_t(first), n, min_q, out, j.stream);
        ck(cudaGetLastError(), "photon launch");
      });
      stored.resize(n);
      ck(cudaMemcpyAsync(stored.data(), pm.stored, n, cudaMemcpyDeviceToHost, j.stream), "photon counts");
      ck(cudaMemcpyAsync(&appended, pm.append_count, sizeof(uint32_t), cudaMemcpyDeviceToHost, j.stream), "photon count");
      ck(cudaStreamSynchronize(j.stream), "photons");
      if (appended > pm.append_cap) throw ApiError{HASTY_ERR_CUDA, "photon buffer overflow"};
      // the reference emits photon i while fewer than count_threshold are stored
      for (uint32_t k = 0; k < n && !done; ++k) {
        base.push_back(cum);
        cum += stored[k];
        if (cum >= uint64_t(count_threshold)) { emitted = first + k + 1; done = true; }
      }
      kept = cum;
      if (!done) { first += n; emitted = first; }
      chunk *= 2;
    }
    host_ph.resize(appended);
    if (appended)
      ck(cudaMemcpyAsync(host_ph.data(), pm.append, appended * sizeof(PhotonRec), cudaMemcpyDeviceToHost, j.stream), "photons");
    ck(cudaStreamSynchronize(j.stream), "photons");
  }
  // Photon map: the photons of the emitted range in emission order (slot =
  // the emission's first slot + the photon's index within it), then a stable
  // radix sort by hash cell, so each cell lists its photons in the order the
  // reference stored them.
  std::vector<PhotonRec> ordered(kept);
  for (const PhotonRec& r : host_ph) {
    uint32_t emit, k;
    std::memcpy(&emit, &r.wi.w, 4);
    std::memcpy(&k, &r.flux.w, 4);
    if (emit < emitted) ordered[base[emit] + k] = r;
  }
  const size_t np = ordered.size();
  std::vector<int32_t> cxyz(3 * np);
  int32_t lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
  for (size_t q = 0; q < np; ++q) {
    const float* x = &ordered[q].xn.x;
    for (int a = 0; a < 3; ++a) {
      int32_t c = floor_i32(x[a] / cell);
      cxyz[3 * q + a] = c;
      if (q == 0 || c < lo[a]) lo[a] = c;
      if (q == 0 || c > hi[a]) hi[a] = c;
    }
  }
  const uint64_t nx = uint64_t(int64_t(hi[0]) - lo[0] + 1), ny = uint64_t(int64_t(hi[1]) - lo[1] + 1),
                 nz = uint64_t(int64_t(hi[2]) - lo[2] + 1);
  const bool fits = double(nx) * double(ny) * double(nz) < 9.0e18;      // linear cell key fits 64 bits
  std::vector<uint64_t> key(np);
  std::vector<uint32_t> perm(np), tmp(np);
  for (size_t q = 0; q < np; ++q) perm[q] = uint32_t(q);
  if (fits) {
    for (size_t q = 0; q < np; ++q)
      key[q] = (uint64_t(int64_t(cxyz[3 * q]) - lo[0]) * ny + uint64_t(int64_t(cxyz[3 * q + 1]) - lo[1])) * nz +
               uint64_t(int64_t(cxyz[3 * q + 2]) - lo[2]);
    uint64_t maxkey = 0;
    for (uint64_t k : key) maxkey = std::max(maxkey, k);
    for (int shift = 0; shift < 64 && (maxkey >> shift) != 0; shift += 16) {     // LSD radix, stable
      std::vector<uint32_t> hist(65537, 0);
      for (size_t q = 0; q < np; ++q) hist[((key[perm[q]] >> shift) & 0xFFFFu) + 1]++;
      for (size_t b = 1; b < hist.size(); ++b) hist[b] += hist[b - 1];
      for (size_t q = 0; q < np; ++q) tmp[hist[(key[perm[q]] >> shift) & 0xFFFFu]++] = perm[q];
      perm.swap(tmp);
    }
  } else {                                                 // huge cell ranges: compare the coordinates
    std::stable_sort(perm.begin(), perm.end(), [&](uint32_t a, uint32_t b) {
      for (int c = 0; c < 3; ++c)
        if (cxyz[3 * a + c] != cxyz[3 * b + c]) return cxyz[3 * a + c] < cxyz[3 * b + c];
      return false;
    });
    for (size_t q = 0; q < np; ++q)   // equal coordinates <=> equal key (cell boundaries below)
      key[perm[q]] = q > 0 && std::equal(&cxyz[3 * perm[q]], &cxyz[3 * perm[q]] + 3, &cxyz[3 * perm[q - 1]])
                         ? key[perm[q - 1]] : uint64_t(q);
  }
  std::vector<PhotonRec> sorted(np);
  std::vector<int4> cells;
  std::vector<int32_t> counts;
  for (size_t q = 0; q < np; ++q) {
    const uint32_t src = perm[q];
    sorted[q] = ordered[src];
    if (q == 0 || key[src] != key[perm[q - 1]]) {
      cells.push_back(make_int4(cxyz[3 * src], cxyz[3 * src + 1], cxyz[3 * src + 2], int(q)));
      counts.push_back(0);
    }
    counts.back() += 1;
  }
  pm.sorted = grow(j, pm.sorted, pm.sorted_cap, std::max<size_t>(1, sorted.size()), 0);
  pm.cells = grow(j, pm.cells, pm.cells_cap, std::max<size_t>(1, cells.size()), 0);
  pm.cell_count = grow(j, pm.cell_count, pm.counts_cap, std::max<size_t>(1, cells.size()), 0);
  if (!sorted.empty())
    ck(cudaMemcpyAsync(pm.sorted, sorted.data(), sorted.size() * sizeof(PhotonRec), cudaMemcpyHostToDevice, j.stream), "photon map");
  if (!cells.empty()) {
    ck(cudaMemcpyAsync(pm.cells, cells.data(), cells.size() * sizeof(int4), cudaMemcpyHostToDevice, j.stream), "photon map");
    ck(cudaMemcpyAsync(pm.cell_count, counts.data(), counts.size() * sizeof(int32_t), cudaMemcpyHostToDevice, j.stream), "photon map");
  }
  PmMapDev map{pm.sorted, pm.cells, pm.cell_count, int32_t(cells.size()), cell};
  const float ox = halton_value(2, t), oy = halton_value(3, t);
  time_device(gather_ms, [&] {
    launch_pm_gather(j.sd, map, pm.px, j.seed, t, ox, oy, int(emitted), pm.stats, j.stream);
    ck(cudaGetLastError(), "gather launch");
  });
  const size_t n = size_t(W) * H;
  ck(cudaMemcpyAsync(pm.radii.data(), pm.px.radii, n * sizeof(float), cudaMemcpyDeviceToHost, j.stream), "radii");
  ck(cudaStreamSynchronize(j.stream), "radii");
  cudaEventDestroy(e0); cudaEventDestroy(e1);
  pm.emitted = emitted;
  pm.photons = np;
  pm.cell = cell;
  pm.iteration = t + 1;
  pm.device_ms += dev_ms;
  pm.photon_ms += photon_ms;
  pm.gather_ms += gather_ms;
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
    return HASTY_OK;
  });
}

}  // extern "C"
