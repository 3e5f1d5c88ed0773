// Oracle (test infrastructure only): the photon mapper restated; see
// oracle_pm.hpp. Operation order follows core/src/PhotonMapping.cpp line by
// line (same float/double promotions), built with -ffp-contract=off.
#include "oracle_pm.hpp"

#include <cmath>
#include <stdexcept>

namespace hor {
namespace {

bool same_prim(const Hit& a, const Hit& b) {      // isSelfIntersection, PathTracing.h:41-45
  return a.geomID == b.geomID && a.primID == b.primID;
}

bool has_diffuse_lobe(const Scene& sc, const Hit& h) { return sc.ctx(h.it).has_diffuse_lobe(h.it); }

// Scene::sampleBRDFConcentrated (Scene.cpp:339-352).
SampleResult sample_concentrated(const Scene& sc, Rng& r, LightRayInfo& lr, const Hit& h, bool adjoint) {
  MaterialCtx mc = sc.ctx(h.it);
  float prob;
  int wl = lr.sample_wavelength(r, mc.mat->vary_ior, prob);
  float eta_out = lr.outside_ior(h);
  SampleResult s = mc.sample(r, h.it, h.wfrom, wl, eta_out, kEvalConcentrated, adjoint);
  s.thrD = s.thrD / prob;
  s.thrC = s.thrC / prob;
  return s;
}

// MISSampleResult of one strategy (MIS.cpp:6-54): the light strategy
// evaluates the BSDF toward a light sample, the BSDF strategy samples the
// BSDF (all lobes) and traces the sampled ray.
struct MisSample { V3 o, d; LightRayInfo lr; Hit hit; V3 thrD, thrC; float pdf = 0.0f; };

MisSample mis_sample(const Scene& sc, Rng& r, const LightRayInfo& lr, const V3& rd, const Hit& hit, bool light) {
  MisSample ms;
  ms.lr = lr;
  if (light) {
    bool vis;
    sc.sample_light_ray(r, hit.it, ms.pdf, ms.o, ms.d, ms.hit, vis, nullptr);
    if (!vis || ms.pdf == 0.0f) { ms.thrD = ms.thrC = V3(0, 0, 0); ms.pdf = 0.0f; return ms; }
    EvalResult ev = sc.ctx(hit.it).evaluate(hit.it, -rd, ms.d, ms.lr.outside_ior(hit));
    float m = std::fabs(dot(ms.d, hit.it.ng)) / ms.pdf;
    ms.thrD = ev.fD * m;
    ms.thrC = ev.fC * m;
    return ms;
  }
  MaterialCtx mc = sc.ctx(hit.it);
  float prob;
  int wl = ms.lr.sample_wavelength(r, mc.mat->vary_ior, prob);
  float eta_out = ms.lr.outside_ior(hit);
  SampleResult s = mc.sample(r, hit.it, hit.wfrom, wl, eta_out);
  s.thrD = s.thrD / prob;
  s.thrC = s.thrC / prob;
  if (s.pdf == 0.0f) { ms.thrD = ms.thrC = V3(0, 0, 0); ms.pdf = 0.0f; return ms; }
  ms.o = sc.ray_x(hit.it, s.outside);
  ms.d = s.dir;
  ms.thrD = s.thrD; ms.thrC = s.thrC; ms.pdf = s.pdf;
  sc.ray_hit(ms.o, ms.d, ms.hit, nullptr);
  return ms;
}

float powci3(float f) { return f * (f * f); }     // powci<3>, VMath.h:29-46

}  // namespace

void PhotonMap::build() {
  for (uint32_t i = 0; i < photons.size(); ++i) cells[index(photons[i].x)].push_back(i);
}

void PhotonMap::radius_search(const V3& c, float radius, std::vector<uint32_t>& out) const {
  out.clear();
  float rsq = radius * radius;
  std::array<int32_t, 3> lo = index(c - V3::fill(radius)), hi = index(c + V3::fill(radius));
  for (int32_t i = lo[0]; i <= hi[0]; i++)
    for (int32_t j = lo[1]; j <= hi[1]; j++)
      for (int32_t k = lo[2]; k <= hi[2]; k++) {
        auto it = cells.find({i, j, k});
        if (it == cells.end()) continue;
        for (uint32_t idx : it->second)
          if (norm_sq(photons[idx].x - c) <= rsq) out.push_back(idx);
      }
}

void trace_photon(const Scene& sc, Rng& r, PhotonMap& pm, V3 o, V3 d, const V3& flux0, uint32_t emit_index) {
  V3 flux = flux0;
  LightRayInfo lr;
  Hit hit;
  sc.ray_hit(o, d, hit, nullptr);
  if (!hit.hit) return;
  flux = cwise(flux, beers_law(lr.transmittance, norm(hit.it.x - o)));
  const int max_depth = sc.settings.max_depth;
  for (int depth = 0; depth < max_depth; depth++) {
    if (!finite3(flux)) break;
    if (has_diffuse_lobe(sc, hit) && depth > 0)
      pm.photons.push_back(Photon{-d, dot(hit.it.ng, hit.wfrom), hit.it.x, flux, emit_index, uint32_t(depth)});
    SampleResult s = sample_concentrated(sc, r, lr, hit, true);
    V3 tt = s.thrD + s.thrC;
    if (tt == V3(0, 0, 0)) break;
    V3 o2 = sc.ray_x(hit.it, s.outside), d2 = s.dir;
    Hit hit2;
    sc.ray_hit(o2, d2, hit2, nullptr);
    if (!hit2.hit || same_prim(hit, hit2)) break;
    lr.update_media(sc, hit, s.dir);
    tt = cwise(tt, beers_law(lr.transmittance, norm(hit2.it.x - o2)));
    float minQ = 1.0f - std::pow(0.1f, 1.0f / max_depth);
    float q = std::max(minQ, 1.0f - norm(tt));
    if (r.uniform01f() <= q) break;
    flux = cwise(flux, tt) / (1.0f - q);
    hit = hit2; o = o2; d = d2;
  }
}

PmResult path_trace_caustics(const Scene& sc, Rng& r, const PhotonMap& pm, LightRayInfo& lr, const V3& ro, const V3& rd,
                             const Hit* pre, V3& normal, V3& albedo, float& radius, int depth,
                             std::vector<uint32_t>& scratch) {
  PmResult res;
  if (depth >= sc.settings.max_depth) return res;
  Hit local;
  if (!pre) sc.ray_hit(ro, rd, local, nullptr);
  const Hit& hit = pre ? *pre : local;
  if (!hit.hit) {
    res.LRest = cwise(beers_law(lr.transmittance, 1e6f), sc.env.eval(rd));
    normal = V3(0, 0, 0);
    albedo = res.LRest;
    return res;
  }
  if (depth == 0) { normal = hit.it.ns_default; albedo = sc.albedo(hit.it); }
  V3 thr = beers_law(lr.transmittance, norm(hit.it.x - ro));
  if (sc.is_surface_light(hit)) {
    res.LLight = res.LLight + cwise(thr, sc.emission(-rd, hit));
    return res;
  }
  if (has_diffuse_lobe(sc, hit)) {                 // photonMapFluxEstimate, PhotonMapping.cpp:271-302
    if (radius <= 0.0f) throw std::runtime_error("photon gather radius <= 0 (the reference falls back to a kd-tree)");
    pm.radius_search(hit.it.x, radius, scratch);
    V3 est(0, 0, 0);
    MaterialCtx mc = sc.ctx(hit.it);
    for (uint32_t idx : scratch) {
      const Photon& ph = pm.photons[idx];
      EvalResult ev = mc.evaluate(hit.it, hit.wfrom, ph.wi, 1.0f, kEvalDiffuse);
      float fc = std::fabs(dot(ph.wi, hit.it.ng)) / (1e-7f + std::fabs(ph.ngwi));
      est = est + cwise(ph.flux * fc, ev.fD + ev.fC);
    }
    res.M += int(scratch.size());
    res.photonFlux = res.photonFlux + cwise(thr, est);
  }
  bool two = sc.has_light() && sc.settings.use_mis;      // SamplingStrategies, MIS.cpp:60-72
  int nstrat = two ? 2 : 1;
  float q = depth >= sc.settings.roulette_start ? sc.settings.roulette_q : 0.0f;
  if (r.uniform01f() <= q) return res;
  thr = thr / (1.0f - q);
  float pdfs[2] = {0.0f, 0.0f};
  for (int s = 0; s < nstrat; ++s) {
    const bool light = two && s == 0;
    MisSample ms = mis_sample(sc, r, lr, rd, hit, light);
    pdfs[s] = ms.pdf;
    if ((ms.thrD + ms.thrC) == V3(0, 0, 0) || same_prim(hit, ms.hit)) continue;
    for (int j = 0; j < nstrat; ++j) {
      if (j == s) continue;
      if (two && j == 0) pdfs[j] = sc.light_ray_density(hit.it, ms.o, ms.d, ms.hit);
      else pdfs[j] = sc.ctx(hit.it).sample_pdf(hit.it, hit.wfrom, ms.d, ms.lr.outside_ior(hit));
    }
    float ssum = 0.0f;
    for (int j = 0; j < nstrat; ++j) ssum += pdfs[j] * pdfs[j];
    float w = pdfs[s] * pdfs[s] / ssum;
    ms.lr.update_media(sc, hit, ms.d);
    V3 tD = cwise(thr, ms.thrD) * w;
    V3 tC = cwise(thr, ms.thrC) * w;
    V3 t2 = tD + tC;
    V3 n2, a2;
    PmResult rs = path_trace_caustics(sc, r, pm, ms.lr, ms.o, ms.d, &ms.hit, n2, a2, radius, depth + 1, scratch);
    res.LSpecular = res.LSpecular + cwise(rs.LLight + rs.LSpecular, tC);
    res.LCaustic = res.LCaustic + cwise(rs.LSpecular, tD);
    res.LRest = res.LRest + (cwise(rs.LRest, t2) + cwise(rs.LLight, tD));
    res.photonFlux = res.photonFlux + cwise(rs.photonFlux, t2);
    res.M += rs.M;
  }
  return res;
}

float cell_size_for(const std::vector<float>& radii, uint32_t W, uint32_t H) {
  float sum = 0.0f;
  for (uint32_t i = 0; i < W; i++)
    for (uint32_t j = 0; j < H; j++) sum += radii[size_t(j) * W + i];
  const float a = 5.0f;
  const float density = 1e5f;
  float cs = sum / float(W * H);
  auto cost = [&](float c) {
    float s = 0.0f;
    for (uint32_t i = 0; i < W; i++)
      for (uint32_t j = 0; j < H; j++) {
        float rr = radii[size_t(j) * W + i];
        s += a * powci3(rr / c) + powci3(std::max(rr, c)) * density;
      }
    return s;
  };
  float best = cost(cs);
  for (int k = 0; k < 10; k++) {
    bool changed = false;
    float trial = cs * 1.5f;
    float tc = cost(trial);
    if (tc < best) { cs = trial; best = tc; changed = true; }
    if (!changed) break;
  }
  for (int k = 0; k < 10; k++) {
    bool changed = false;
    float trial = cs * 0.6666f;
    float tc = cost(trial);
    if (tc < best) { cs = trial; best = tc; changed = true; }
    if (!changed) break;
  }
  return cs;
}

float footprint_radius(const Scene& sc, Rng& r, float default_r, int i, int j, int W, int H) {
  float px = float(i) + 0.5f, py = float(j) + 0.5f;
  V3 o, d;
  sc.camera.compute_ray(r, px, py, float(W), float(H), o, d);
  Hit hit;
  sc.ray_hit(o, d, hit, nullptr);
  if (!hit.hit) return default_r;
  float angle = sc.camera.ray_angle(px, py, float(W), float(H));
  float dist = norm(sc.camera.pos - hit.it.x);
  if (!has_diffuse_lobe(sc, hit)) {
    for (int k = 0; k < sc.settings.max_depth; k++) {
      if (has_diffuse_lobe(sc, hit)) break;
      SampleResult s;
      int tries = 0;
      do {
        LightRayInfo fresh;
        s = sample_concentrated(sc, r, fresh, hit, false);
        tries += 1;
      } while (s.thrC == V3(0, 0, 0) && tries < 3);
      if (s.thrC == V3(0, 0, 0)) break;
      V3 o2 = sc.ray_x(hit.it, s.outside);
      Hit hit2;
      sc.ray_hit(o2, s.dir, hit2, nullptr);
      if (!hit2.hit || same_prim(hit, hit2)) return default_r;
      dist += norm(hit.it.x - hit2.it.x);
      hit = hit2;
    }
  }
  return 0.5f * dist * std::tan(angle);
}

float close_non_negative(const std::vector<float>& img, int W, int H, int i, int j) {
  auto inside = [&](int x, int y) { return x >= 0 && y >= 0 && x < W && y < H; };
  auto at = [&](int x, int y) { return img[size_t(y) * size_t(W) + size_t(x)]; };
  int k = 1;
  while (k < std::max(H, W)) {
    for (int m = 0; m <= k * 2; m++) {
      int i2 = i - k, j2 = j - k + m;
      if (inside(i2, j2) && at(i2, j2) > 0.0f) return at(i2, j2);
      i2 = i - k + m; j2 = j - k;
      if (inside(i2, j2) && at(i2, j2) > 0.0f) return at(i2, j2);
      i2 = i + k; j2 = j - k + m;
      if (inside(i2, j2) && at(i2, j2) > 0.0f) return at(i2, j2);
      // the reference computes a fourth candidate (i - k + m, j + k) here and never tests it
    }
    k += 1;
  }
  return 1e-3f;
}

void pm_init(const Scene& sc, PmState& st) {
  const uint32_t W = sc.settings.width, H = sc.settings.height;
  st.W = W; st.H = H;
  st.px.assign(size_t(W) * H, PmPixel());
  st.color.assign(size_t(W) * H * 3, 0.0f);
  st.normal.assign(size_t(W) * H * 3, 0.0f);
  st.albedo.assign(size_t(W) * H * 3, 0.0f);
  st.radii.assign(size_t(W) * H, 1.0f);
  if (sc.has_surface_light()) {                     // computeInitialRadii(context, W, H, 10), :680-705
    for (uint32_t j = 0; j < H; j++)
      for (uint32_t i = 0; i < W; i++) {
        Rng r(path_key(sc.settings.seed, j * W + i, kFootprintPass));
        st.radii[size_t(j) * W + i] = 10.0f * footprint_radius(sc, r, -1.0f, int(i), int(j), int(W), int(H));
      }
    for (uint32_t j = 0; j < H; j++)
      for (uint32_t i = 0; i < W; i++)
        if (st.radii[size_t(j) * W + i] < 0.0f)
          st.radii[size_t(j) * W + i] = close_non_negative(st.radii, int(W), int(H), int(i), int(j));
  }
  st.initialised = true;
  st.iteration = 0;
}

void pm_iteration(const Scene& sc, PmState& st) {
  if (!st.initialised) pm_init(sc, st);
  const uint32_t W = st.W, H = st.H, t = st.iteration;
  const uint64_t seed = sc.settings.seed;
  PhotonMap pm;
  pm.clear(cell_size_for(st.radii, W, H));
  if (sc.has_surface_light()) {
    const int trace_threshold = int(10.f * float(H) * float(W));
    const int count_threshold = int(0.5f * float(H) * float(W));
    for (int i = 0; i < trace_threshold && pm.photons.size() < size_t(count_threshold); i++) {
      Rng r(photon_key(seed, uint32_t(i), t));
      V3 flux, o, d;
      sc.sample_emission_ray(r, flux, o, d);
      pm.emitted += 1;
      trace_photon(sc, r, pm, o, d, flux, uint32_t(i));
    }
  }
  pm.build();
  st.emitted = pm.emitted;
  st.stored = pm.photons.size();
  st.cell = pm.cell;
  const float ox = halton(2, t), oy = halton(3, t);
  std::vector<uint32_t> scratch;
  for (uint32_t j = 0; j < H; j++)
    for (uint32_t i = 0; i < W; i++) {
      const size_t p = size_t(j) * W + i;
      Rng r(path_key(seed, uint32_t(p), t));
      V3 o, d;
      sc.camera.compute_ray(r, float(i) + ox, float(j) + oy, float(W), float(H), o, d);
      PmPixel& px = st.px[p];
      if (px.radius == -1.0f) px.radius = st.radii[p];        // PMRenderJob::lock
      float radius = px.radius;
      V3 normal(0, 0, 0), albedo(0, 0, 0);
      LightRayInfo lr;
      PmResult res = path_trace_caustics(sc, r, pm, lr, o, d, nullptr, normal, albedo, radius, 0, scratch);
      V3 L = res.LLight + res.LRest + res.LSpecular;
      V3 Lnew;
      if (L != L || res.photonFlux != res.photonFlux) {
        Lnew = px.LSum / (1e-7f + float(px.Nd));               // PMRenderJob::unlock
      } else {                                                // PMRenderJob::unlockAndUpdateStatistic
        const float alpha = 0.4f;
        const int M = res.M, NeInI = int(pm.emitted);
        px.LSum = px.LSum + L;
        px.Nd += 1;
        V3 Lflux(0, 0, 0);
        if (px.radius < 0.0f) {
          if (!(radius < 0.0f)) {
            px.radius = radius;
            px.N += alpha * M;
            px.Ne += NeInI;
            px.flux = res.photonFlux;
            Lflux = px.Ne == 0 ? V3(0, 0, 0) : px.flux / (px.radius * px.radius * float(kPi) * px.Ne);
          }
        } else {
          float rold = px.radius;
          float Ni = px.N;
          if (Ni + M > 0) px.radius *= std::sqrt((Ni + alpha * M) / (Ni + M));
          px.N += alpha * M;
          px.Ne += NeInI;
          px.flux = (px.flux + res.photonFlux) * (px.radius * px.radius) / (rold * rold);
          Lflux = px.Ne == 0 ? V3(0, 0, 0) : px.flux / (px.radius * px.radius * float(kPi) * px.Ne);
          radius = px.radius;
        }
        Lnew = Lflux + px.LSum / float(px.Nd);
      }
      st.radii[p] = radius;
      for (int c = 0; c < 3; ++c) {
        st.color[3 * p + c] = Lnew[c];
        st.normal[3 * p + c] = normal[c];
        st.albedo[3 * p + c] = albedo[c];
      }
    }
  st.iteration = t + 1;
}

}  // namespace hor
