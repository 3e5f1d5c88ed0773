// Oracle (test infrastructure only): drives the reference's photon mapper,
// core/src/PhotonMapping.cpp, compiled unmodified in this translation unit
// (its PhotonMap class and free functions are not declared in a header) and
// linked with the rest of the reference build in oracle/_ref/. One function of
// that file binds a temporary LightRayInfo to a non-const reference (an MSVC
// extension, PhotonMapping.cpp:610); the macro below makes GCC do the same
// without changing the source. It composes renderPhotonThread's loop
// (PhotonMapping.cpp:814-935) for one thread from the reference's own pieces
// (computeRadiusPixelFootPrint, getCloseNonNegative, computeCellSize,
// sampleLightRay, tracePhoton, PhotonMap, pathTraceWithCausticsMap,
// PMRenderJob's statistics) with random streams keyed per photon and per
// pixel (hor_rng.hpp) instead of one sequential stream per thread.
#include <Hasty/Json.h>
#include <Hasty/MIS.h>
#include <Hasty/PhotonMapping.h>
#include <Hasty/Scene.h>

#include <cstring>

#include "port/hor_io.hpp"
#include "port/hor_rng.hpp"

template <class T> T& hasty_lvalue(T&& x) { return x; }
#define sampleBRDFConcentrated(c, l, h, a) sampleBRDFConcentrated(c, hasty_lvalue(l), h, a)
#include "../src/PhotonMapping.cpp"
#undef sampleBRDFConcentrated

using namespace Hasty;

namespace {
struct RefPm {
  PMRenderJob job;
  uint64_t seed = 0;
  bool initialised = false;
  uint32_t iteration = 0;
  Image1f radii;
  Image3f color, normal, albedo;
  uint64_t emitted = 0, stored = 0;
  float cell = 0.0f;
};

void init(RefPm& r) {
  RenderSettings& st = r.job.renderSettings;
  Scene& scene = *r.job.scene;
  const uint32_t W = st.width, H = st.height;
  r.color.setZero(W, H); r.normal.setZero(W, H); r.albedo.setZero(W, H);
  r.radii.setConstant(W, H, 1.f);
  if (scene.hasSurfaceLight()) {      // computeInitialRadii(context, W, H, 10.0f), keyed per pixel
    r.radii.setConstant(W, H, -1.0f);
    for (uint32_t j = 0; j < H; j++)
      for (uint32_t i = 0; i < W; i++) {
        RNG rng(hor::path_key(r.seed, j * W + i, hor::kFootprintPass));
        RenderContext ctx(scene, rng, st);
        r.radii(i, j) = 10.0f * computeRadiusPixelFootPrint(ctx, -1.0f, i, j, W, H, true);
      }
    for (uint32_t j = 0; j < H; j++)
      for (uint32_t i = 0; i < W; i++)
        if (r.radii(i, j) < 0.0f) r.radii(i, j) = getCloseNonNegative(r.radii, i, j);
  }
  r.initialised = true;
}

void iterate(RefPm& r) {
  RenderSettings& st = r.job.renderSettings;
  Scene& scene = *r.job.scene;
  const uint32_t W = st.width, H = st.height, t = r.iteration;
  RenderJobSample sample = r.job.fetchSample();
  PhotonMap photonMap;
  photonMap.clear(true, computeCellSize(r.radii));
  if (scene.hasSurfaceLight()) {
    int tracethreshold = 10.f * st.height * st.width;
    int countThreshold = 0.5f * st.height * st.width;
    for (int i = 0; i < tracethreshold && photonMap.photonCount() < countThreshold; i++) {
      RNG rng(hor::photon_key(r.seed, uint32_t(i), t));
      RenderContext ctx(scene, rng, st);
      Vec3f flux;
      Ray ray = scene.sampleLightRay(rng, flux);
      photonMap.increaseEmittedCount();
      tracePhoton(ctx, photonMap, ray, flux, true);
    }
  }
  photonMap.build();
  r.emitted = photonMap.emittedCount();
  r.stored = photonMap.photonCount();
  for (uint32_t j = 0; j < H; j++)
    for (uint32_t i = 0; i < W; i++) {
      RNG rng(hor::path_key(r.seed, j * W + i, t));
      RenderContext ctx(scene, rng, st);
      Vec2f p0 = Vec2f(float(i), float(j));
      Ray ray = scene.camera.computeRay(rng, p0 + sample.offset, float(W), float(H));
      float radius = r.job.lock(i, j, r.radii(i, j));
      Vec3f normal, albedo;
      LightRayInfo lightRay;
      PathTraceWithCausticsMapResult res = pathTraceWithCausticsMap(ctx, photonMap, lightRay, ray, nullptr, normal, albedo,
                                                                    radius, 0);
      Vec3f L = res.LLight + res.LRest + res.LSpecular;
      Vec3f Lnew;
      if (L != L || res.photonFlux != res.photonFlux) Lnew = r.job.unlock(i, j);
      else Lnew = r.job.unlockAndUpdateStatistic(i, j, res.photonFlux, L, res.M, photonMap.emittedCount(), radius);
      r.radii(i, j) = radius;
      r.color(i, j) = Lnew; r.normal(i, j) = normal; r.albedo(i, j) = albedo;
    }
  r.iteration = t + 1;
}
}  // namespace

extern "C" {

void* ref_pm_load(const char* job_path, char* err, int errlen) {
  auto* r = new RefPm();
  try {
    r->job.loadJSON(job_path);
    hor::Json j = hor::read_json_file(job_path);
    if (const hor::Json* g = j.find("gb300")) if (g->contains("seed")) r->seed = uint64_t(g->at("seed").as_number());
    return r;
  } catch (const std::exception& e) {
    if (err && errlen > 0) { std::strncpy(err, e.what(), size_t(errlen - 1)); err[errlen - 1] = 0; }
    delete r;
    return nullptr;
  }
}

void ref_pm_free(void* p) { delete static_cast<RefPm*>(p); }

// Same layout as hor_pm_iterate (oracle/port/oracle_capi.cpp).
int ref_pm_iterate(void* p, int n, float* color, float* normal, float* albedo, float* radii, int64_t* info) {
  RefPm& r = *static_cast<RefPm*>(p);
  if (!r.initialised) init(r);
  for (int k = 0; k < n; ++k) iterate(r);
  const uint32_t W = r.job.renderSettings.width, H = r.job.renderSettings.height;
  for (uint32_t j = 0; j < H; j++)
    for (uint32_t i = 0; i < W; i++) {
      size_t q = size_t(j) * W + i;
      for (int c = 0; c < 3; ++c) {
        if (color) color[3 * q + c] = r.color(i, j)[c];
        if (normal) normal[3 * q + c] = r.normal(i, j)[c];
        if (albedo) albedo[3 * q + c] = r.albedo(i, j)[c];
      }
      if (radii) radii[q] = r.radii(i, j);
    }
  if (info) {
    info[0] = int64_t(r.emitted); info[1] = int64_t(r.stored); info[2] = r.iteration;
    info[3] = 0;
  }
  return 0;
}

}  // extern "C"
