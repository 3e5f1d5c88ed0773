// Oracle (test infrastructure only): C entry points of the CPU oracle,
// loaded with ctypes by tests/, __graft_entry__.smoke() and bench.py's
// CPU-baseline leg. Nothing in the product links against this library.
#include "oracle_core.hpp"
#include "oracle_pm.hpp"
#include <atomic>
#include <cstring>
#include <thread>

using namespace hor;

namespace {
struct Handle { Scene sc; };

void fill_err(char* err, int n, const std::string& m) {
  if (err && n > 0) { std::strncpy(err, m.c_str(), size_t(n - 1)); err[n - 1] = 0; }
}

Interaction kat_interaction(const float* in) {
  Interaction it;
  it.x = V3(in[0], in[1], in[2]);
  it.ng = V3(in[3], in[4], in[5]);
  it.ns_default = V3(in[6], in[7], in[8]);
  it.tangent = V3(in[9], in[10], in[11]);
  it.bitangent = V3(in[12], in[13], in[14]);
  it.material = 0;
  return it;
}
Material kat_material(const float* in) {
  Material m;
  m.albedo = V3(in[15], in[16], in[17]);
  m.metallic = in[18]; m.specular = in[19]; m.roughness = in[20];
  m.anisotropy = in[21]; m.transmission = in[22]; m.ior = in[23]; m.vary_ior = in[24] != 0.0f;
  { const float um[3] = {0.65f, 0.55f, 0.45f}; set_ior_bands(m, false, 0.0f, um); }
  return m;
}
void put3(float* o, const V3& v) { o[0] = v.x; o[1] = v.y; o[2] = v.z; }
}  // namespace

extern "C" {

void* hor_load(const char* job_path, char* err, int errlen) {
  try {
    auto* h = new Handle();
    h->sc.load_job(job_path);
    return h;
  } catch (const std::exception& e) {
    fill_err(err, errlen, e.what());
    return nullptr;
  }
}

void hor_free(void* p) { delete static_cast<Handle*>(p); }

// out: width, height, num_samples, max_depth, n_tris, n_light_tris, env_is_texture,
//      use_mis, roulette_start, n_shapes, n_materials, seed
void hor_info(void* p, int64_t* out) {
  const Scene& s = static_cast<Handle*>(p)->sc;
  out[0] = s.settings.width; out[1] = s.settings.height; out[2] = s.settings.num_samples;
  out[3] = s.settings.max_depth; out[4] = int64_t(s.tris.size()); out[5] = int64_t(s.light_tris.size());
  out[6] = s.env.is_texture; out[7] = s.settings.use_mis; out[8] = s.settings.roulette_start;
  out[9] = int64_t(s.shape_first.size()); out[10] = int64_t(s.mats.size()); out[11] = int64_t(s.settings.seed);
}

void hor_set_seed(void* p, uint64_t seed) { static_cast<Handle*>(p)->sc.settings.seed = seed; }

// Process-wide test switch: per-sample math-library results moved by one ulp
// (see nudge_ulp in oracle_core.hpp).
void hor_set_ulp_nudge(int on) { g_ulp_nudge = on != 0; }

// Sums over passes [pass0, pass0+npasses) for the pixel window (x0,y0,w,h):
// color (NaN samples dropped, as PathTracing.cpp:132-142), its square,
// normal and albedo AOVs. Buffers are w*h*3 doubles, row-major.
// stats[6]: rays, nan samples, bvh nodes visited, triangle tests, shaded vertices, paths.
// Rows y0, y0 + row_stride, ..., (h rows) of the same window; the buffers
// hold the h rendered rows.
int hor_render_rows(void* p, int pass0, int npasses, int x0, int y0, int w, int h, int row_stride, int nthreads,
                    double* color, double* color_sq, double* normal, double* albedo, uint64_t* stats);

int hor_render(void* p, int pass0, int npasses, int x0, int y0, int w, int h, int nthreads,
               double* color, double* color_sq, double* normal, double* albedo, uint64_t* stats) {
  return hor_render_rows(p, pass0, npasses, x0, y0, w, h, 1, nthreads, color, color_sq, normal, albedo, stats);
}

int hor_render_rows(void* p, int pass0, int npasses, int x0, int y0, int w, int h, int row_stride, int nthreads,
                    double* color, double* color_sq, double* normal, double* albedo, uint64_t* stats) {
  const Scene& sc = static_cast<Handle*>(p)->sc;
  if (row_stride < 1) return -1;
  if (nthreads < 1) nthreads = int(std::max(1u, std::thread::hardware_concurrency()));
  std::atomic<int> next_row{0};
  std::vector<RenderStats> per(static_cast<size_t>(nthreads));
  auto work = [&](int tid) {
    RenderStats& st = per[size_t(tid)];
    for (;;) {
      int row = next_row.fetch_add(1);
      if (row >= h) break;
      for (int xx = 0; xx < w; ++xx) {
        size_t k = 3 * (size_t(row) * w + xx);
        double c[3] = {0, 0, 0}, c2[3] = {0, 0, 0}, nn[3] = {0, 0, 0}, aa[3] = {0, 0, 0};
        for (int ps = pass0; ps < pass0 + npasses; ++ps) {
          V3 n, a;
          V3 L = render_sample(sc, uint32_t(x0 + xx), uint32_t(y0 + row * row_stride), uint32_t(ps), n, a, st);
          if (L != L) { st.nan++; continue; }
          for (int q = 0; q < 3; ++q) { c[q] += L[q]; c2[q] += double(L[q]) * L[q]; nn[q] += n[q]; aa[q] += a[q]; }
        }
        for (int q = 0; q < 3; ++q) {
          if (color) color[k + q] = c[q];
          if (color_sq) color_sq[k + q] = c2[q];
          if (normal) normal[k + q] = nn[q];
          if (albedo) albedo[k + q] = aa[q];
        }
      }
    }
  };
  std::vector<std::thread> th;
  for (int t = 1; t < nthreads; ++t) th.emplace_back(work, t);
  work(0);
  for (auto& t : th) t.join();
  if (stats) {
    RenderStats tot;
    for (auto& s : per) { tot.rays += s.rays; tot.nan += s.nan; tot.nodes += s.nodes; tot.tris += s.tris; tot.shaded += s.shaded; tot.paths += s.paths; }
    stats[0] = tot.rays; stats[1] = tot.nan; stats[2] = tot.nodes; stats[3] = tot.tris; stats[4] = tot.shaded; stats[5] = tot.paths;
  }
  return 0;
}

// Per-sample values of one pass (NaN kept), float32, w*h*3 each.
int hor_render_samples(void* p, int pass, int x0, int y0, int w, int h, float* color, float* normal, float* albedo) {
  const Scene& sc = static_cast<Handle*>(p)->sc;
  RenderStats st;
  for (int yy = 0; yy < h; ++yy)
    for (int xx = 0; xx < w; ++xx) {
      V3 n, a;
      V3 L = render_sample(sc, uint32_t(x0 + xx), uint32_t(y0 + yy), uint32_t(pass), n, a, st);
      size_t k = 3 * (size_t(yy) * w + xx);
      for (int q = 0; q < 3; ++q) { color[k + q] = L[q]; normal[k + q] = n[q]; albedo[k + q] = a[q]; }
    }
  return 0;
}

// rays: n x 6 floats (origin, direction). mode 0: BVH (FP32), 1: brute force (FP64),
// 2: brute force with the FP32 triangle test.
// Outputs: triangle index (global, shape-major order; -1 miss), t, u, v.
// stats[2]: nodes visited, triangle tests (mode 0).
int hor_intersect(void* p, const float* rays, int64_t n, int mode, int32_t* prim, float* t, float* u, float* v, uint64_t* stats) {
  const Scene& sc = static_cast<Handle*>(p)->sc;
  BvhStats st;
  for (int64_t i = 0; i < n; ++i) {
    const float* r = rays + 6 * i;
    BvhHit hh = mode == 0 ? sc.bvh.intersect(r, r + 3, 1e-6f, INFINITY, &st)
               : mode == 2 ? sc.bvh.intersect_brute(r, r + 3, 1e-6f, INFINITY)
                           : sc.bvh.intersect_fp64(r, r + 3, 1e-6f, INFINITY);
    prim[i] = hh.prim; t[i] = hh.t; u[i] = hh.u; v[i] = hh.v;
  }
  if (stats) { stats[0] = st.nodes; stats[1] = st.tris; }
  return 0;
}

void hor_tri_ids(void* p, int32_t* geom, int32_t* prim) {
  const Scene& sc = static_cast<Handle*>(p)->sc;
  for (size_t i = 0; i < sc.tris.size(); ++i) { geom[i] = int32_t(sc.tris[i].geom); prim[i] = int32_t(sc.tris[i].prim); }
}

// The first n outputs of the path's stream.
void hor_rng_stream(uint64_t seed, uint32_t pixel, uint32_t pass, int n, uint32_t* out) {
  Rng r(path_key(seed, pixel, pass));
  for (int i = 0; i < n; ++i) out[i] = r.next_u32();
}

float hor_halton(uint32_t base, uint32_t k) { return halton(base, k); }

// The reference's unit tests (apps/Tests.cpp:40-232) as loops over the
// oracle's routines, seeded with the project stream of `seed`. Writes the
// quantities each test asserts on; returns the number written.
//   0 rodriguesRotation (Tests.cpp:40-52): max |x - R^-1 R x| over n trials
//   1 sphericalCoordinates (:54-74): max |d - to(from(d))|, min/max theta, phi
//   2 sampleCosineLobe (:76-90): max rel |pdf - evalpdf|, max ||w|-1|
//   3 sampleHemisphereCosImportance (:93-106): same quantities
//   4 DGGX (:107-131): MC estimate of int D(h) (n.h) dh (alpha 0.3)
//   5 sampleDGGX (:132-147): max rel |pdf - density|
//   6 sampleDGGX2 (:148-168): MC estimate of E[cos/pdf] (alpha 1)
//   7 sampleGGXVNDFGlobal (:169-187): max rel |pdf - density|, min pdf
//   8 sampleGGXVNDFGlobal2 (:188-210): MC estimate of E[cos/pdf] (alpha 1)
//   9 refraction (:212-232): max |wi - wi2|, |F1 - F2|
int hor_property(int which, int64_t n, uint64_t seed, double* out) {
  Rng r(path_key(seed, 0, 0));
  float pd;
  switch (which) {
    case 0: {
      double m = 0;
      for (int64_t i = 0; i < n; ++i) {
        V3 a = sample_sphere_uniformly(r, pd), b = sample_sphere_uniformly(r, pd);
        Rotation rot(a, b);
        V3 x(r.uniform01f(), r.uniform01f(), r.uniform01f());
        V3 y = rot.apply_inverse(rot.apply(x));
        m = std::max(m, double(norm(x - y)));
      }
      out[0] = m; return 1;
    }
    case 1: {
      double m = 0, tmin = 1e9, tmax = -1e9, pmin = 1e9, pmax = -1e9;
      for (int64_t i = 0; i < n; ++i) {
        V3 d = sample_sphere_uniformly(r, pd);
        float th, ph; sph_from_dir(d, th, ph);
        SphDir back = sph_to_dir(th, ph);
        m = std::max(m, double(norm(d - back.dir)));
        tmin = std::min(tmin, double(th)); tmax = std::max(tmax, double(th));
        pmin = std::min(pmin, double(ph)); pmax = std::max(pmax, double(ph));
      }
      out[0] = m; out[1] = tmin; out[2] = tmax; out[3] = pmin; out[4] = pmax; return 5;
    }
    case 2: case 3: {
      double mrel = 0, mlen = 0;
      for (int64_t i = 0; i < n; ++i) {
        V3 lobe = sample_sphere_uniformly(r, pd);
        float p1, p2; V3 w;
        if (which == 2) { float e = 1.0f + r.uniform01f() * 10.0f; w = sample_cosine_lobe(r, lobe, e, p1); p2 = eval_cosine_lobe_pdf(lobe, e, w); }
        else { w = sample_hemisphere_cos(r, lobe, p1); p2 = eval_hemisphere_cos_pdf(lobe, w); }
        mrel = std::max(mrel, std::fabs(double(p1) - p2) / std::max(1.0, std::fabs(double(p2))));
        mlen = std::max(mlen, std::fabs(double(norm(w)) - 1.0));
      }
      out[0] = mrel; out[1] = mlen; return 2;
    }
    case 4: {
      float alpha = 0.3f;
      V3 nrm = sample_sphere_uniformly(r, pd);
      V3 wo = sample_hemisphere_uniformly(r, nrm, pd);
      V3 t = any_orthonormal(nrm), b = cross(nrm, t);
      double sum = 0; float mind = 1;
      for (int64_t i = 0; i < n; ++i) {
        wo = sample_hemisphere_uniformly(r, nrm, pd);
        float d = dggx(dot(nrm, wo), dot(t, wo), dot(b, wo), alpha, alpha);
        mind = std::min(mind, d);
        sum += double(d) * dot(nrm, wo) / pd;
      }
      out[0] = sum / double(n); out[1] = mind; return 2;
    }
    case 5: {
      double mrel = 0;
      for (int64_t i = 0; i < n; ++i) {
        float alpha = std::max(1e-2f, r.uniform01f());
        V3 nrm = sample_sphere_uniformly(r, pd);
        V3 wo = sample_hemisphere_uniformly(r, nrm, pd);
        float p1; V3 wi = sample_dggx(r, nrm, alpha, wo, p1);
        float p2 = sample_dggx_density(nrm, alpha, wo, wi);
        mrel = std::max(mrel, std::fabs(double(p1) - p2) / std::max(1.0, std::fabs(double(p2))));
      }
      out[0] = mrel; return 1;
    }
    case 6: case 8: {
      float alpha = 1.0f;
      V3 nrm = sample_sphere_uniformly(r, pd);
      V3 wo = nrm;
      double sum = 0; float minp = 1e30f;
      for (int64_t i = 0; i < n; ++i) {
        float p; V3 wi;
        if (which == 6) wi = sample_dggx(r, nrm, alpha, wo, p);
        else { V3 t = any_orthonormal(nrm), b = cross(nrm, t); wi = sample_ggx_vndf_global(r, nrm, alpha, alpha, t, b, wo, p); }
        minp = std::min(minp, p);
        sum += std::max(0.0f, dot(nrm, wi)) / p;
      }
      out[0] = sum / double(n); out[1] = minp; return 2;
    }
    case 7: {
      double mrel = 0; float minp = 1e30f;
      for (int64_t i = 0; i < n; ++i) {
        float alpha = std::max(1e-2f, r.uniform01f());
        V3 nrm = sample_sphere_uniformly(r, pd);
        V3 wo = sample_hemisphere_uniformly(r, nrm, pd);
        V3 t = any_orthonormal(nrm), b = cross(nrm, t);
        float p1; V3 wi = sample_ggx_vndf_global(r, nrm, alpha, alpha, t, b, wo, p1);
        float p2 = sample_ggx_vndf_global_density(nrm, alpha, alpha, t, b, wo, wi);
        minp = std::min(minp, p1);
        mrel = std::max(mrel, std::fabs(double(p1) - p2) / std::max(1.0, std::fabs(double(p2))));
      }
      out[0] = mrel; out[1] = minp; return 2;
    }
    case 9: {
      V3 nrm = normalize(V3(0.1f, 0.2f, 1.0f)), wi = normalize(V3(0.15f, 0.05f, 1.0f)), wo, wi2;
      refraction_direction(wi, nrm, 1.45f, 1.0f, wo);
      refraction_direction(wo, -nrm, 1.0f, 1.45f, wi2);
      out[0] = norm(wi - wi2);
      out[1] = std::fabs(fresnel_dielectric(0.3f, 0.6f, 1.0f, 1.4f) - fresnel_dielectric(0.6f, 0.3f, 1.4f, 1.0f));
      return 2;
    }
    default: return -1;
  }
}

// Known-answer entry points with replayed uniforms; layouts are listed in
// tests/golden/make_golden.py. Returns the number of outputs written.
int hor_kat(int which, const float* in, const uint32_t* replay, int nreplay, float* out) {
  Rng r = Rng::from_replay(replay, size_t(nreplay));
  try {
    switch (which) {
      case 0: case 1: case 2: {
        Interaction it = kat_interaction(in);
        Material m = kat_material(in);
        std::vector<Texture> tex;
        MaterialCtx mc{&m, &tex};
        V3 wo(in[25], in[26], in[27]), wi(in[28], in[29], in[30]);
        int wl = int(in[31]); float eta_out = in[32];
        if (which == 0) {
          SampleResult s = mc.sample(r, it, wo, wl, eta_out);
          out[0] = s.outside ? 1.f : 0.f; put3(out + 1, s.dir); put3(out + 4, s.thrD); put3(out + 7, s.thrC);
          out[10] = s.pdf; out[11] = float(r.replay_pos);
          return 12;
        }
        if (which == 1) { EvalResult e = mc.evaluate(it, wo, wi, eta_out); put3(out, e.fD); put3(out + 3, e.fC); put3(out + 6, e.ns); return 9; }
        out[0] = mc.sample_pdf(it, wo, wi, eta_out);
        return 1;
      }
      case 3: { float pdf; V2 s = sample_ngon_uniformly(r, int(in[0]), in[1], pdf); out[0] = s.x; out[1] = s.y; out[2] = pdf; out[3] = float(r.replay_pos); return 4; }
      case 4: { float pdf; V3 d = sample_hemisphere_cos(r, V3(in[0], in[1], in[2]), pdf); put3(out, d); out[3] = pdf; out[4] = float(r.replay_pos); return 5; }
      case 5: { V3 b = sample_triangle_uniformly(r); put3(out, b); out[3] = float(r.replay_pos); return 4; }
      case 6: {
        V3 n(in[0], in[1], in[2]), t(in[5], in[6], in[7]), b(in[8], in[9], in[10]), wo(in[11], in[12], in[13]);
        float pdf; V3 d = sample_ggx_vndf_global(r, n, in[3], in[4], t, b, wo, pdf);
        put3(out, d); out[3] = pdf; out[4] = sample_ggx_vndf_global_density(n, in[3], in[4], t, b, wo, d); out[5] = float(r.replay_pos);
        return 6;
      }
      case 7: out[0] = fresnel_dielectric(in[0], in[1], in[2], in[3]); return 1;
      case 8: { V3 wt(0, 0, 0); bool ok = refraction_direction(V3(in[0], in[1], in[2]), V3(in[3], in[4], in[5]), in[6], in[7], wt); out[0] = ok; put3(out + 1, wt); return 4; }
      case 9: { float pdf; V3 v = sample_sphere_uniformly(r, pdf); put3(out, v); out[3] = pdf; out[4] = float(r.replay_pos); return 5; }
      case 10: { Rotation rot(V3(in[0], in[1], in[2]), V3(in[3], in[4], in[5])); V3 x(in[6], in[7], in[8]); put3(out, rot.apply(x)); put3(out + 3, rot.apply_inverse(x)); return 6; }
      case 11: out[0] = smith_ggx(in[0], in[1], in[2], in[3], in[4]); out[1] = dggx(in[0], in[1], in[2], in[3], in[4]); return 2;
      case 12: { V3 n(in[0], in[1], in[2]), d1(in[4], in[5], in[6]); float pdf; V3 d = sample_dggx(r, n, in[3], d1, pdf); put3(out, d); out[3] = pdf; out[4] = sample_dggx_density(n, in[3], d1, d); out[5] = float(r.replay_pos); return 6; }
      case 13: { V3 l(in[0], in[1], in[2]); float pdf; V3 d = sample_cosine_lobe(r, l, in[3], pdf); put3(out, d); out[3] = pdf; out[4] = eval_cosine_lobe_pdf(l, in[3], d); out[5] = float(r.replay_pos); return 6; }
      case 14: { float pdf; V3 v = sample_hemisphere_uniformly(r, V3(in[0], in[1], in[2]), pdf); put3(out, v); out[3] = pdf; out[4] = float(r.replay_pos); return 5; }
      case 15: { out[0] = eval_hemisphere_cos_pdf(V3(in[0], in[1], in[2]), V3(in[3], in[4], in[5])); return 1; }
      default: return -1;
    }
  } catch (const std::exception&) {
    return -2;
  }
}

// ---- photon mapper (oracle_pm.hpp) ----------------------------------------
void* hor_pm_new(void* p) {
  auto* st = new PmState();
  return st;
}
void hor_pm_free(void* s) { delete static_cast<PmState*>(s); }
// Runs n more iterations; writes the current colour / normal / albedo images
// (W*H*3 floats), the radii (W*H) and info = {emitted, stored, iteration} +
// the cell size (as float bits in info[3]) of the last iteration.
int hor_pm_iterate(void* p, void* s, int n, float* color, float* normal, float* albedo, float* radii, int64_t* info) {
  const Scene& sc = static_cast<Handle*>(p)->sc;
  PmState& st = *static_cast<PmState*>(s);
  try {
    if (!st.initialised) pm_init(sc, st);
    for (int k = 0; k < n; ++k) pm_iteration(sc, st);
  } catch (const std::exception&) {
    return -1;
  }
  const size_t np = size_t(st.W) * st.H;
  if (color) std::memcpy(color, st.color.data(), 3 * np * sizeof(float));
  if (normal) std::memcpy(normal, st.normal.data(), 3 * np * sizeof(float));
  if (albedo) std::memcpy(albedo, st.albedo.data(), 3 * np * sizeof(float));
  if (radii) std::memcpy(radii, st.radii.data(), np * sizeof(float));
  if (info) {
    info[0] = int64_t(st.emitted); info[1] = int64_t(st.stored); info[2] = st.iteration;
    uint32_t cb; std::memcpy(&cb, &st.cell, 4); info[3] = cb;
  }
  return 0;
}
// Initial radii only (before the first iteration).
int hor_pm_init_radii(void* p, void* s, float* radii) {
  const Scene& sc = static_cast<Handle*>(p)->sc;
  PmState& st = *static_cast<PmState*>(s);
  pm_init(sc, st);
  std::memcpy(radii, st.radii.data(), size_t(st.W) * st.H * sizeof(float));
  return 0;
}

}  // extern "C"
