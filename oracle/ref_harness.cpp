// Oracle (test infrastructure only): drives the reference's own integrator,
// compiled unmodified from its sources (core/src/*.cpp) against the stand-in
// headers in oracle/shims/. Used on the development machine to pin the CPU
// restatement (oracle/port) and to write the golden fixtures under
// tests/golden/. Built by oracle/Makefile into oracle/_ref/.
//
// It provides (1) the stand-in implementations of the absent dependencies'
// entry points (shishua, Embree) and (2) a C API mirroring oracle_capi.cpp:
// ref_load / ref_render / ref_render_samples / ref_kat.
#include <Hasty/BRDF.h>
#include <Hasty/Camera.h>
#include <Hasty/Environment.h>
#include <Hasty/LightRayInfo.h>
#include <Hasty/MIS.h>
#include <Hasty/PathTracing.h>
#include <Hasty/Random.h>
#include <Hasty/RenderJob.h>
#include <Hasty/Sample.h>
#include <Hasty/Scene.h>

#include <atomic>
#include <cstring>
#include <thread>

#include "port/hor_bvh.hpp"
#include "port/hor_io.hpp"
#include "port/hor_rng.hpp"

// ------------------------------------------------------------- shishua ----
namespace {
thread_local const uint32_t* g_replay = nullptr;
thread_local size_t g_replay_n = 0;
}  // namespace

extern "C" void prng_init(struct prng_state* s, uint64_t seed[4]) {
  std::memset(s, 0, sizeof(*s));
  if (g_replay) { s->replay = 1; s->replay_pos = 0; return; }
  hor::Pcg32 p; p.seed_key(seed[0]);
  s->state = p.state; s->inc = p.inc;
}

extern "C" void prng_gen(struct prng_state* s, uint8_t* buf, size_t size) {
  size_t n = size / 4;
  for (size_t i = 0; i < n; ++i) {
    uint32_t v;
    if (s->replay) { v = g_replay[s->replay_pos % g_replay_n]; s->replay_pos++; }
    else { hor::Pcg32 p; p.state = s->state; p.inc = s->inc; v = p.next(); s->state = p.state; }
    std::memcpy(buf + 4 * i, &v, 4);
  }
}

// -------------------------------------------------------------- Embree ----
struct RTCDeviceTy { int dummy; };
struct RTCGeometryTy {
  std::vector<float> verts;
  std::vector<unsigned> idx;
};
struct RTCSceneTy {
  std::vector<RTCGeometryTy*> geoms;
  std::vector<float> tri_pos;
  std::vector<unsigned> tri_geom, tri_prim;
  hor::Bvh2 bvh;
};

RTCDevice rtcNewDevice(const char*) { return new RTCDeviceTy(); }
void rtcReleaseDevice(RTCDevice d) { delete d; }
RTCScene rtcNewScene(RTCDevice) { return new RTCSceneTy(); }
void rtcReleaseScene(RTCScene s) { for (auto* g : s->geoms) delete g; delete s; }
RTCGeometry rtcNewGeometry(RTCDevice, enum RTCGeometryType) { return new RTCGeometryTy(); }
void* rtcSetNewGeometryBuffer(RTCGeometry g, enum RTCBufferType type, unsigned int, enum RTCFormat, size_t, size_t count) {
  if (type == RTC_BUFFER_TYPE_VERTEX) { g->verts.assign(3 * count, 0.f); return g->verts.data(); }
  g->idx.assign(3 * count, 0u);
  return g->idx.data();
}
void rtcCommitGeometry(RTCGeometry) {}
unsigned int rtcAttachGeometry(RTCScene s, RTCGeometry g) { s->geoms.push_back(g); return unsigned(s->geoms.size() - 1); }
void rtcReleaseGeometry(RTCGeometry) {}
void rtcCommitScene(RTCScene s) {
  for (size_t gi = 0; gi < s->geoms.size(); ++gi) {
    const RTCGeometryTy* g = s->geoms[gi];
    for (size_t f = 0; f < g->idx.size() / 3; ++f) {
      for (int k = 0; k < 3; ++k)
        for (int c = 0; c < 3; ++c) s->tri_pos.push_back(g->verts[3 * size_t(g->idx[3 * f + k]) + c]);
      s->tri_geom.push_back(unsigned(gi)); s->tri_prim.push_back(unsigned(f));
    }
  }
  s->bvh.build(s->tri_pos.data(), s->tri_geom.size());
}
void rtcInitIntersectContext(struct RTCIntersectContext* c) { std::memset(c, 0, sizeof(*c)); }
void rtcIntersect1(RTCScene s, struct RTCIntersectContext*, struct RTCRayHit* rh) {
  float o[3] = {rh->ray.org_x, rh->ray.org_y, rh->ray.org_z};
  float d[3] = {rh->ray.dir_x, rh->ray.dir_y, rh->ray.dir_z};
  hor::BvhHit h = s->bvh.intersect(o, d, rh->ray.tnear, rh->ray.tfar);
  if (h.prim < 0) return;
  rh->ray.tfar = h.t;
  rh->hit.u = h.u; rh->hit.v = h.v;
  rh->hit.Ng_x = h.ng[0]; rh->hit.Ng_y = h.ng[1]; rh->hit.Ng_z = h.ng[2];
  rh->hit.geomID = s->tri_geom[size_t(h.prim)];
  rh->hit.primID = s->tri_prim[size_t(h.prim)];
}

// ----------------------------------------------------------- harness ----
using namespace Hasty;

namespace {
struct RefJob {
  RenderJob job;
  uint64_t seed = 0;
};

void put3(float* o, const Vec3f& v) { o[0] = v[0]; o[1] = v[1]; o[2] = v[2]; }

struct ReplayGuard {
  ReplayGuard(const uint32_t* v, size_t n) { g_replay = v; g_replay_n = n; }
  ~ReplayGuard() { g_replay = nullptr; g_replay_n = 0; }
};

// Position in the replayed list of the next value the RNG would hand out.
float draws_of(RNG& rng, const uint32_t* replay, int n) {
  uint32_t nxt = rng();
  for (int i = 0; i < n; ++i) if (replay[i] == nxt) return float(i);
  return -1.0f;
}

Vec3f v3(const float* p) { return Vec3f(p[0], p[1], p[2]); }
}  // namespace

namespace Hasty { float smithGGX(float nv, float tv, float bv, float alpha_t, float alpha_b); }

extern "C" {

void* ref_load(const char* job_path, char* err, int errlen) {
  auto* r = new RefJob();
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

void ref_free(void* p) { delete static_cast<RefJob*>(p); }

static Vec3f ref_sample(RefJob& r, uint32_t x, uint32_t y, uint32_t pass, const Vec2f& offset, Vec3f& normal, Vec3f& albedo) {
  RenderSettings& st = r.job.renderSettings;
  Scene& scene = *r.job.scene;
  RNG rng(hor::path_key(r.seed, y * st.width + x, pass));
  RenderContext ctx(scene, rng, st);
  Vec2f p0 = Vec2f(float(x), float(y));
  Ray ray = scene.camera.computeRay(rng, p0 + offset, float(st.width), float(st.height));
  LightRayInfo info;
  normal = Vec3f::Zero(); albedo = Vec3f::Zero();
  return estimateRadiance(ctx, info, ray, normal, albedo, 0);
}

static std::vector<Vec2f> halton_offsets(int pass0, int npasses) {
  HaltonSequence2 seq;
  std::vector<Vec2f> out;
  for (int k = 0; k < pass0 + npasses; ++k) { Vec2f o = seq(); if (k >= pass0) out.push_back(o); }
  return out;
}

int ref_render(void* p, int pass0, int npasses, int x0, int y0, int w, int h, int nthreads,
               double* color, double* color_sq, double* normal, double* albedo, uint64_t* nan_count) {
  RefJob& r = *static_cast<RefJob*>(p);
  std::vector<Vec2f> offs = halton_offsets(pass0, npasses);
  if (nthreads < 1) nthreads = int(std::max(1u, std::thread::hardware_concurrency()));
  std::atomic<int> next_row{0};
  std::atomic<uint64_t> nans{0};
  auto work = [&]() {
    for (;;) {
      int row = next_row.fetch_add(1);
      if (row >= h) break;
      for (int xx = 0; xx < w; ++xx) {
        double c[3] = {0, 0, 0}, c2[3] = {0, 0, 0}, nn[3] = {0, 0, 0}, aa[3] = {0, 0, 0};
        for (int k = 0; k < npasses; ++k) {
          Vec3f n, a;
          Vec3f L = ref_sample(r, uint32_t(x0 + xx), uint32_t(y0 + row), uint32_t(pass0 + k), offs[size_t(k)], n, a);
          if (L != L) { nans++; continue; }
          for (int q = 0; q < 3; ++q) { c[q] += L[q]; c2[q] += double(L[q]) * L[q]; nn[q] += n[q]; aa[q] += a[q]; }
        }
        size_t kk = 3 * (size_t(row) * w + xx);
        for (int q = 0; q < 3; ++q) {
          if (color) color[kk + q] = c[q];
          if (color_sq) color_sq[kk + q] = c2[q];
          if (normal) normal[kk + q] = nn[q];
          if (albedo) albedo[kk + q] = aa[q];
        }
      }
    }
  };
  std::vector<std::thread> th;
  for (int t = 1; t < nthreads; ++t) th.emplace_back(work);
  work();
  for (auto& t : th) t.join();
  if (nan_count) *nan_count = nans;
  return 0;
}

int ref_render_samples(void* p, int pass, int x0, int y0, int w, int h, float* color, float* normal, float* albedo) {
  RefJob& r = *static_cast<RefJob*>(p);
  Vec2f off = halton_offsets(pass, 1)[0];
  for (int yy = 0; yy < h; ++yy)
    for (int xx = 0; xx < w; ++xx) {
      Vec3f n, a;
      Vec3f L = ref_sample(r, uint32_t(x0 + xx), uint32_t(y0 + yy), uint32_t(pass), off, n, a);
      size_t k = 3 * (size_t(yy) * w + xx);
      put3(color + k, L); put3(normal + k, n); put3(albedo + k, a);
    }
  return 0;
}

// Same input/output layouts as hor_kat in oracle/port/oracle_capi.cpp.
int ref_kat(int which, const float* in, const uint32_t* replay, int nreplay, float* out) {
  ReplayGuard guard(replay, size_t(nreplay));
  RNG rng(0);
  try {
    switch (which) {
      case 0: case 1: case 2: {
        SurfaceInteraction it;
        it.geomID = 0; it.primID = 0; it.h = 0.0f;
        it.x = v3(in); it.normalGeometric = v3(in + 3); it.normalShadingDefault = v3(in + 6);
        it.tangent = v3(in + 9); it.bitangent = v3(in + 12);
        it.materialId = 0; it.barycentricCoordinates = Vec3f(1.0f, 0.0f, 0.0f);
        PrincipledBRDF brdf(std::make_unique<ConstantTexture3f>(v3(in + 15)), std::make_unique<ConstantTexture1f>(in[20]),
                            std::make_unique<ConstantTexture1f>(in[18]), in[19], in[23], nullptr, in[21], in[22], in[24] != 0.0f);
        Vec3f wo = v3(in + 25), wi = v3(in + 28);
        int wl = int(in[31]); float eta = in[32];
        if (which == 0) {
          SampleResult s = brdf.sample(rng, it, wo, wl, eta, false, ShaderEvalFlag::ALL);
          out[0] = s.outside ? 1.f : 0.f; put3(out + 1, s.direction); put3(out + 4, s.throughputDiffuse);
          put3(out + 7, s.throughputConcentrated); out[10] = s.pdfOmega; out[11] = draws_of(rng, replay, nreplay);
          return 12;
        }
        if (which == 1) {
          MaterialEvalResult e = brdf.evaluate(it, wo, wi, eta, false, ShaderEvalFlag::ALL);
          put3(out, e.fDiffuse); put3(out + 3, e.fConcentrated); put3(out + 6, e.normalShading);
          return 9;
        }
        out[0] = brdf.evaluateSamplePDF(it, wo, wi, eta);
        return 1;
      }
      case 3: { float pdf; Vec2f s = sampleCircularNGonUniformly(rng, int(in[0]), in[1], pdf); out[0] = s[0]; out[1] = s[1]; out[2] = pdf; out[3] = draws_of(rng, replay, nreplay); return 4; }
      case 4: { float pdf; Vec3f d = sampleHemisphereCosImportance(rng, v3(in), pdf); put3(out, d); out[3] = pdf; out[4] = draws_of(rng, replay, nreplay); return 5; }
      case 5: { Vec3f b = sampleTriangleUniformly(rng); put3(out, b); out[3] = draws_of(rng, replay, nreplay); return 4; }
      case 6: {
        Vec3f n = v3(in), t = v3(in + 5), b = v3(in + 8), wo = v3(in + 11);
        float pdf; Vec3f d = sampleGGXVNDFGlobal(rng, n, in[3], in[4], t, b, wo, pdf);
        put3(out, d); out[3] = pdf; out[4] = sampleGGXVNDFGlobalDensity(n, in[3], in[4], t, b, wo, d);
        out[5] = draws_of(rng, replay, nreplay);
        return 6;
      }
      case 7: out[0] = fresnelDielectric(in[0], in[1], in[2], in[3]); return 1;
      case 8: { Vec3f wt = Vec3f::Zero(); bool ok = computeRefractionDirection(v3(in), v3(in + 3), in[6], in[7], wt); out[0] = ok; put3(out + 1, wt); return 4; }
      case 9: { float pdf; Vec3f v = sampleSphereSurfaceUniformly(rng, pdf); put3(out, v); out[3] = pdf; out[4] = draws_of(rng, replay, nreplay); return 5; }
      case 10: {
        RotationBetweenTwoVectors<float, Vec3f> rot(v3(in), v3(in + 3));
        Vec3f x = v3(in + 6);
        put3(out, applyRotation(rot, x)); put3(out + 3, applyRotationInverse(rot, x));
        return 6;
      }
      case 11: out[0] = Hasty::smithGGX(in[0], in[1], in[2], in[3], in[4]); out[1] = DGGX(in[0], in[1], in[2], in[3], in[4]); return 2;
      case 12: { float pdf; Vec3f d = sampleDGGX(rng, v3(in), in[3], v3(in + 4), pdf); put3(out, d); out[3] = pdf; out[4] = sampleDGGXDensity(v3(in), in[3], v3(in + 4), d); out[5] = draws_of(rng, replay, nreplay); return 6; }
      case 13: { float pdf; Vec3f d = sampleCosineLobe(rng, v3(in), in[3], pdf); put3(out, d); out[3] = pdf; out[4] = evaluateCosineLobePDF(v3(in), in[3], d); out[5] = draws_of(rng, replay, nreplay); return 6; }
      case 14: { float pdf; Vec3f v = sampleHemisphereSurfaceUniformly(rng, v3(in), pdf); put3(out, v); out[3] = pdf; out[4] = draws_of(rng, replay, nreplay); return 5; }
      case 15: out[0] = evaluateHemisphereCosImportancePDF(v3(in), v3(in + 3)); return 1;
      default: return -1;
    }
  } catch (const std::exception&) {
    return -2;
  }
}

}  // extern "C"
