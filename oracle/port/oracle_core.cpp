// Oracle (test infrastructure only). See oracle_core.hpp.
#include "oracle_core.hpp"
#include <cstdio>
#include <numeric>
#include <stdexcept>

namespace hor {

bool g_ulp_nudge = false;

// ============================================================ sampling ====
V2 sample_disk_uniformly(Rng& r, float& pdf) {
  float alpha = r.uniform01f() * float(2.0 * kPi);
  float rad = std::sqrt(r.uniform01f());
  pdf = float(kInvPi);
  return V2{rad * ncos(alpha), rad * nsin(alpha)};
}

V2 sample_ngon_uniformly(Rng& r, int blades, float rotation, float& pdf) {
  float per = float(2.0 * kPi / blades);
  float nx = std::cos(per * 0.5f), ny = std::sin(per * 0.5f);
  float d = -nx;
  V2 s;
  bool outside;
  do {
    s = sample_disk_uniformly(r, pdf);
    float rad = std::sqrt(s.x * s.x + s.y * s.y);
    float ang = natan2(s.y, s.x);
    ang -= rotation;
    ang += float(2.0 * kPi) * (1.0f + FLT_EPSILON);
    ang = std::fmod(ang, per);
    float px = rad * ncos(ang), py = rad * nsin(ang);
    outside = (nx * px + ny * py + d) > 0.0f;
  } while (outside);
  float area_sector = 0.5 * std::sin(per);
  float area = blades * area_sector;
  pdf = 1.0 / area;
  return s;
}

V3 sample_sphere_uniformly(Rng& r, float& pdf) {
  pdf = 0.25f * float(kInvPi);
  for (;;) {
    V3 v(r.uniformm11f(), r.uniformm11f(), r.uniformm11f());  // argument order as the reference's compiler
    float rsq = norm_sq(v);
    if (rsq <= 1.0 && rsq > 1e-6f) return v / std::sqrt(rsq);
  }
}

V3 sample_hemisphere_uniformly(Rng& r, const V3& n, float& pdf) {
  pdf = 0.5f * float(kInvPi);
  for (;;) {
    V3 v(r.uniformm11f(), r.uniformm11f(), r.uniformm11f());
    float rsq = norm_sq(v);
    if (rsq <= 1.0f && rsq > 1e-6f && dot(v, n) >= 0.0f) return v / std::sqrt(rsq);
  }
}

V3 sample_hemisphere_cos(Rng& r, const V3& n, float& pdf) {
  V3 dir; float c;
  do {
    float xi1 = r.uniform01f();
    float xi2 = r.uniform01f();
    float phi = 2.0f * float(kPi) * xi2;
    c = std::sqrt(xi1);
    float s = std::sqrt(1.0f - xi1);
    float cp = ncos(phi), sp = nsin(phi);
    V3 rv(s * cp, s * sp, c);
    Rotation rot(V3(0, 0, 1), n);
    dir = normalize(rot.apply(rv));
    c = dot(dir, n);
  } while (c <= 0.0f);
  pdf = float(kInvPi) * c;
  return dir;
}

float eval_hemisphere_cos_pdf(const V3& n, const V3& d) {
  float c = dot(n, d);
  if (c < 0.0f) return 0.0f;
  return float(kInvPi) * c;
}

V3 sample_cosine_lobe(Rng& r, const V3& lobe, float e, float& pdf) {
  V3 dir; float c;
  do {
    float xi1 = r.uniform01f();
    float xi2 = r.uniform01f();
    float phi = 2.0f * float(kPi) * xi2;
    c = npow(xi1, 1.0f / (e + 1.0f));
    float s = std::sqrt(1.0f - c * c);
    float cp = ncos(phi), sp = nsin(phi);
    V3 rv(s * cp, s * sp, c);
    Rotation rot(V3(0, 0, 1), lobe);
    dir = normalize(rot.apply(rv));
    c = dot(dir, lobe);
  } while (c <= 0.0f);
  pdf = (e + 1.0f) * 0.5f * float(kInvPi) * npow(c, e);
  return dir;
}

float eval_cosine_lobe_pdf(const V3& lobe, float e, const V3& d) {
  float c = dot(lobe, d);
  if (c < 0.0f) return 0.0f;
  return (e + 1.0f) * 0.5f * float(kInvPi) * npow(c, e);
}

V3 sample_triangle_uniformly(Rng& r) {
  float s = r.uniform01f();
  float t = std::sqrt(r.uniform01f());
  float b1 = 1.0f - t;
  float b3 = t * s;
  float b2 = std::max(0.0f, 1.0f - b1 - b3);
  return V3(b1, b2, b3);
}

// ================================================================ BSDF ====
bool refraction_direction(const V3& wi, const V3& n, float ei, float et, V3& wt) {
  float rel = ei / et;
  float ci = dot(wi, n);
  float si2 = std::max(0.f, 1.f - ci * ci);
  float st2 = (rel * rel) * si2;
  if (st2 >= 1.0f) return false;
  float ct = std::sqrt(1.0f - st2);
  wt = normalize((-rel) * wi + (rel * ci - ct) * n);
  return true;
}

bool refraction_cos_t(float ci, float ei, float et, float& ct) {
  float rel = ei / et;
  float si2 = std::max(0.f, 1.f - ci * ci);
  float st2 = (rel * rel) * si2;
  if (st2 >= 1.0f) return false;
  ct = std::sqrt(1.0f - st2);
  return true;
}

V3 refraction_direction_from_angles(const V3& wi, const V3& n, float ratio, float ci, float ct) {
  return normalize((-ratio) * wi + (ratio * ci - ct) * n);
}

float fresnel_dielectric(float ci, float ct, float ei, float et) {
  float rp = (et * ci - ei * ct) / (et * ci + ei * ct);
  float ro = (ei * ci - et * ct) / (ei * ci + et * ct);
  return 0.5f * (rp * rp + ro * ro);
}

float dggx_iso(float nh, float a) {
  float q = (nh * nh) * (a * a - 1.0f) + 1.0f;
  return a * a / (1e-7f + float(kPi) * (q * q));
}

V3 sample_dggx(Rng& r, const V3& n, float a, const V3& d1, float& pdf) {
  if (dot(d1, n) < 0.0f) { pdf = 1.0f; return -n; }
  V3 h;
  do {
    float xi1 = r.uniform01f();
    float xi2 = r.uniform01f();
    float phi = 2.0f * float(kPi) * xi2;
    float c = std::sqrt((1.0f - xi1) / (xi1 * (a * a - 1.0f) + 1.0f));
    float s = std::sqrt(1.0f - c * c);
    float cp = ncos(phi), sp = nsin(phi);
    V3 rv(s * cp, s * sp, c);
    Rotation rot(V3(0, 0, 1), n);
    h = normalize(rot.apply(rv));
  } while (dot(h, n) <= 0.0f);
  V3 d2 = normalize(reflect_across(d1, h));
  float nh = dot(n, h);
  float q = (nh * nh) * (a * a - 1.0f) + 1.0f;
  float ph = a * a * nh / (float(kPi) * (q * q));
  pdf = ph / std::fabs(4.0f * dot(d1, h));
  return d2;
}

float sample_dggx_density(const V3& n, float a, const V3& d1, const V3& d2) {
  V3 h = normalize(d1 + d2);
  float nh = std::fabs(dot(n, h));
  float q = (nh * nh) * (a * a - 1.0f) + 1.0f;
  float ph = a * a * nh / (float(kPi) * (q * q));
  return ph / (1e-7f + std::fabs(4.0f * dot(d1, h)));
}

float dggx(float nh, float th, float bh, float at, float ab) {
  return float(kInvPi) / (at * ab * sq(sq(th / at) + sq(bh / ab) + sq(nh)));
}

float smith_ggx(float nv, float tv, float bv, float at, float ab) {
  float lambda = 0.5f * (std::sqrt(1.0f + (sq(at * tv) + sq(ab * bv)) / sq(nv)) - 1.0f);
  return 1.0f / (1.0f + lambda);
}

V3 sample_ggx_vndf(const V3& wo, float ax, float ay, float xi1, float xi2) {
  V3 vh = normalize(V3(ax * wo.x, ay * wo.y, wo.z));
  V3 t1 = cross(vh, V3(0, 0, 1));
  if (norm_sq(t1) < 1e-12f) t1 = V3(1, 0, 0);
  else t1 = normalize(t1);
  V3 t2 = cross(t1, vh);
  float rr = std::sqrt(xi1);
  float a = 1.0f / (1.0f + vh.z);
  float phi = float(kPi) * ((xi2 < a) ? (xi2 / a) : (1.0f + (xi2 - a) / (1.0f - a)));
  float p1 = rr * ncos(phi);
  float p2 = rr * nsin(phi) * (xi2 < a ? 1.0f : vh.z);
  float p3 = std::sqrt(std::max(0.0f, 1.0f - p1 * p1 - p2 * p2));
  V3 nh = p1 * t1 + p2 * t2 + p3 * vh;
  return normalize(V3(ax * nh.x, ay * nh.y, std::max(0.0f, nh.z)));
}

V3 sample_ggx_vndf_global(Rng& r, const V3& n, float at, float ab, const V3& t, const V3& b, const V3& d1, float& pdf) {
  if (dot(d1, n) <= 0.0f) { pdf = 0.0f; return -n; }
  V3 ng;
  do {
    V3 ve(dot(t, d1), dot(b, d1), dot(n, d1));
    // BRDF.cpp:199 passes two uniform01f(rng) calls as arguments; the
    // reference's compiler (GCC, right-to-left) draws the second first.
    float xi2 = r.uniform01f();
    float xi1 = r.uniform01f();
    V3 ne = sample_ggx_vndf(ve, at, ab, xi1, xi2);
    ng = normalize(t * ne.x + b * ne.y + n * ne.z);
  } while (dot(ng, d1) <= 0.0f);
  V3 d2 = normalize(reflect_across(d1, ng));
  float g1 = smith_ggx(dot(n, d1), dot(t, d1), dot(b, d1), at, ab);
  float d = dggx(dot(n, ng), dot(t, ng), dot(b, ng), at, ab);
  float ph = g1 * dot(d1, ng) * d / dot(d1, n);
  pdf = ph / (1e-7f + 4.0f * std::fabs(dot(d1, ng)));
  return d2;
}

float sample_ggx_vndf_global_density(const V3& n, float at, float ab, const V3& t, const V3& b, const V3& d1, const V3& d2) {
  if (dot(d1, n) <= 0.0f) return 0.0f;
  V3 ng = normalize(d1 + d2);
  float g1 = smith_ggx(dot(n, d1), dot(t, d1), dot(b, d1), at, ab);
  float d = dggx(dot(n, ng), dot(t, ng), dot(b, ng), at, ab);
  float ph = g1 * std::max(0.0f, dot(d1, ng)) * d / dot(d1, n);
  return ph / (1e-7f + 4.0f * std::fabs(dot(d1, ng)));
}

static inline float normal_scale(const V3& wi, const V3& ns, const V3& ng) {
  return std::fabs(dot(wi, ns)) / (1e-7f + std::fabs(dot(wi, ng)));
}

float compute_alpha(float rough) {
  float a = rough * rough;
  if (a < 1e-2f && a != 0.0f) a = 1e-2f;
  return a;
}

ProbResult compute_probability(float m, float s, float t, float cos_o, float eo, float er, int flags) {
  ProbResult p;
  p.cosT = 0.0f;
  p.refr = refraction_cos_t(cos_o, eo, er, p.cosT);
  p.FD = p.refr ? fresnel_dielectric(cos_o, p.cosT, eo, er) : 1.0f;
  float mD = (1.0f - t) * (1.0f - m) * (1.0f - 0.5f * s);
  float mS = mixf(mixf(0.5f * s, p.FD, t), 1.0f, m);
  float mR = (1.0 - p.FD) * t * (1.0 - m);
  if (!(flags & kEvalDiffuse)) mD = 0.0f;
  if (!(flags & kEvalConcentrated)) { mS = 0.0f; mR = 0.0f; }
  float sum = mD + mS + mR;
  p.none = sum == 0.0f;
  if (p.none) { p.pD = p.pS = p.pR = 0.0f; }
  else { p.pD = mD / sum; p.pS = mS / sum; p.pR = mR / sum; }
  return p;
}

void anisotropy_params(const Interaction& it, const V3& ns, float alpha, float aniso, float& at, float& ab, V3& t, V3& b) {
  float aspect = std::sqrt(1.0f - 0.9f * aniso);
  at = alpha / aspect;
  ab = alpha * aspect;
  Rotation rot(it.ng, ns);
  t = rot.apply(it.tangent);
  b = rot.apply(it.bitangent);
}

V3 evaluate_diffuse(float nsWi, const V3& albedo, float nscale, float m, float s, float t) {
  if (nsWi < 0.0f) return V3(0, 0, 0);
  float k = float(kInvPi) * nscale * (1.0f - 0.5f * s);
  double kd = double(k) * (1.0 - t) * (1.0 - m);
  return albedo * float(kd);
}

V3 evaluate_concentrated(float nsWi, const V3& albedo, float m, float s, float t, const V3& wo, const V3& wi,
                         float alpha, float at, float ab, const V3& tan, const V3& bit, const V3& ns,
                         float nscale, bool force, const V3& FD) {
  if (nsWi < 0.0f) return V3(0, 0, 0);
  V3 h = normalize(wo + wi);
  float lh = std::fabs(dot(wi, h));
  float c5 = pow5(1.0f - lh);
  float nh = dot(ns, h);
  float nv = std::fabs(dot(ns, wo));
  float nl = std::fabs(dot(ns, wi));
  float go = smith_ggx(nv, dot(tan, wo), dot(bit, wo), at, ab);
  float gi = smith_ggx(nl, dot(tan, wi), dot(bit, wi), at, ab);
  float G = go * gi;
  float D = (alpha == 0.0f) ? (force ? 4.0f * nl : 0.0f) : dggx(nh, dot(tan, h), dot(bit, h), at, ab);
  float spec_diel = 0.5f * s;
  V3 spec_trans(0, 0, 0);
  V3 spec_metal = albedo * (1.0f - c5) + V3(1, 1, 1) * c5;
  if (t > 0.0f) {
    if (alpha != 0.0f) throw std::runtime_error("not implemented");
    spec_trans = force ? FD : V3(0, 0, 0);
  }
  return mixv(mixv(V3::fill(spec_diel), spec_trans, t), spec_metal, m) * (D * G * nscale / std::fabs(1e-7f + 4.0f * nv * nl));
}

SampleResult principled_sample(Rng& r, const Interaction& it, const V3& wo, const V3& ns, const V3& albedo,
                               float m, float s, float rough, float aniso, float t, int wavelength,
                               float eta_out, float eta_mat, int flags, bool adjoint) {
  SampleResult res;
  float ngwo = dot(it.ng, wo);
  float nswo = dot(ns, wo);
  float alpha = compute_alpha(rough);
  res.outside = ngwo >= 0.0f;
  float eo = res.outside ? eta_out : eta_mat;
  float er = res.outside ? eta_mat : eta_out;
  ProbResult p = compute_probability(m, s, t, nswo, eo, er, flags);
  if (p.none) {
    res.dir = V3(1, 0, 0); res.thrD = V3(0, 0, 0); res.thrC = V3(0, 0, 0); res.pdf = 0.0f;
    return res;
  }
  V3 FD = V3::fill(p.FD);
  V3 mask(1, 1, 1);
  if (wavelength != -1) { mask = V3(0, 0, 0); mask[wavelength] = 1.0f; }
  float at, ab; V3 tan, bit;
  anisotropy_params(it, ns, alpha, aniso, at, ab, tan, bit);
  V3 fD(0, 0, 0), fC(0, 0, 0);
  float xi = r.uniform01f();
  int strat = xi < p.pR ? 3 : (xi < (p.pR + p.pS) ? 2 : 1);
  if (strat == 2) {
    if (alpha == 0.0f) {
      res.dir = reflect_across(wo, ns);
      res.pdf = 1e12f;
      float nswi = dot(ns, res.dir);
      float nsc = normal_scale(res.dir, ns, it.ng);
      fC = 1e12f / p.pS * evaluate_concentrated(nswi, albedo, m, s, t, wo, res.dir, alpha, at, ab, tan, bit, ns, nsc, true, FD);
    } else {
      float pdf_spec;
      res.dir = sample_ggx_vndf_global(r, ns, at, ab, tan, bit, wo, pdf_spec);
      float pdf_diff = eval_hemisphere_cos_pdf(ns, res.dir);
      res.pdf = p.pS * pdf_spec + p.pD * pdf_diff;
      float nswi = dot(ns, res.dir);
      float nsc = normal_scale(res.dir, ns, it.ng);
      fD = evaluate_diffuse(nswi, albedo, nsc, m, s, t);
      fC = evaluate_concentrated(nswi, albedo, m, s, t, wo, res.dir, alpha, at, ab, tan, bit, ns, nsc, false, FD);
    }
  } else if (strat == 1) {
    float pdf_diff;
    res.dir = sample_hemisphere_cos(r, ns, pdf_diff);
    float nswi = dot(ns, res.dir);
    float nsc = normal_scale(res.dir, ns, it.ng);
    if (alpha == 0.0f) {
      res.pdf = p.pD * pdf_diff;
      fD = evaluate_diffuse(nswi, albedo, nsc, m, s, t);
    } else {
      float pdf_spec = sample_ggx_vndf_global_density(ns, at, ab, tan, bit, wo, res.dir);
      res.pdf = p.pS * pdf_spec + (1.0f - p.pS) * pdf_diff;
      fD = evaluate_diffuse(nswi, albedo, nsc, m, s, t);
      fC = evaluate_concentrated(nswi, albedo, m, s, t, wo, res.dir, alpha, at, ab, tan, bit, ns, nsc, false, FD);
    }
  } else {
    res.outside = !res.outside;
    res.pdf = 1e12f;
    if (!p.refr) {
      res.dir = V3(1, 0, 0);
    } else {
      float ratio = eo / er;
      res.dir = refraction_direction_from_angles(wo, ns, ratio, nswo, p.cosT);
      float scale = adjoint ? 1.0f : sq(ratio);
      float fc = res.pdf / p.pR * scale * (1.0f - p.FD) / std::fabs(dot(res.dir, it.ng));
      fC = fc * mask;
    }
  }
  float mm = std::fabs(dot(res.dir, it.ng)) / res.pdf;
  res.thrD = fD * mm;
  res.thrC = fC * mm;
  return res;
}

// ------------------------------------------------------------ textures ----
static inline float clampf(float v, float lo, float hi) { return v < lo ? lo : (v > hi ? hi : v); }  // VMath.h:716-719

void Texture::lookup(float u0, float v0, float* out) const {
  float u = clampU ? clampf(u0, 0.0f, 1.0f - FLT_EPSILON) : fmod1p1(u0);
  float omv = clampV ? clampf(1.0f - v0, 0.0f, 1.0f - FLT_EPSILON) : fmod1p1(1.0f - v0);
  int col = int(u * float(w));
  int row = int(omv * float(h));
  // u*W can round up to W for widths that are not powers of two; the
  // reference then reads past the row. The oracle clamps to the last texel.
  col = col >= w ? w - 1 : col;
  row = row >= h ? h - 1 : row;
  const float* p = &data[(size_t(row) * w + col) * ch];
  for (int c = 0; c < ch; ++c) out[c] = p[c];
}

V3 MaterialCtx::albedo(const Interaction& it) const {
  if (mat->albedo_tex < 0) return mat->albedo;
  if (!it.has_uv) return V3(1.0f, 0.0f, 0.7f);           // Texture.h:98-101
  float c[3]; (*tex)[mat->albedo_tex].lookup(it.uv[0], it.uv[1], c);
  return V3(c[0], c[1], c[2]);
}
float MaterialCtx::roughness(const Interaction& it) const {
  if (mat->roughness_tex < 0) return mat->roughness;
  if (!it.has_uv) return -1.0f;
  float c; (*tex)[mat->roughness_tex].lookup(it.uv[0], it.uv[1], &c);
  return c;
}
float MaterialCtx::metallic(const Interaction& it) const {
  if (mat->metallic_tex < 0) return mat->metallic;
  if (!it.has_uv) return -1.0f;
  float c; (*tex)[mat->metallic_tex].lookup(it.uv[0], it.uv[1], &c);
  return c;
}
float MaterialCtx::ior(int wl) const {       // BRDF.cpp:589-603 (bands precomputed at load)
  if (!mat->vary_ior) return mat->ior;
  if (wl >= 0 && wl < 3) return mat->ior_band[wl];
  return std::numeric_limits<float>::quiet_NaN();
}

void set_ior_bands(Material& m, bool cauchy, float b, const float* band_um) {
  const float ratio[3] = {1.43f / 1.45f, 1.45f / 1.45f, 1.47f / 1.45f};
  for (int k = 0; k < 3; ++k) {
    float lam = band_um[k];
    m.ior_band[k] = cauchy ? m.ior + b / (lam * lam) : m.ior * ratio[k];
  }
}
V3 MaterialCtx::shading_normal(const Interaction& it, const V3& wo, float ngwo) const {
  float side = ngwo < 0.0f ? -1.0f : 1.0f;
  V3 ns;
  if (mat->normal_tex >= 0) {
    V3 col(1.0f, 0.0f, 0.7f);
    if (it.has_uv) { float c[3]; (*tex)[mat->normal_tex].lookup(it.uv[0], it.uv[1], c); col = V3(c[0], c[1], c[2]); }
    V3 tn = 2.0f * col - V3(1, 1, 1);
    ns = normalize(it.tangent * tn.x + it.bitangent * tn.y + it.ng * tn.z);
  } else {
    ns = it.ns_default;
  }
  float side_s = dot(ns, wo) < 0.0f ? -1.0f : 1.0f;
  if (side != side_s) ns = it.ng;
  return ns * side;
}
EvalResult MaterialCtx::evaluate(const Interaction& it, const V3& wo, const V3& wi, float eta_out, int flags) const {
  (void)eta_out;
  float ngwo = dot(it.ng, wo);
  V3 ns = shading_normal(it, wo, ngwo);
  float nswi = dot(ns, wi);
  EvalResult r; r.ns = ns;
  V3 alb = albedo(it);
  float rough = roughness(it);
  float alpha = compute_alpha(rough);
  float m = metallic(it);
  float s = mat->specular, an = mat->anisotropy, t = mat->transmission;
  float nsc = normal_scale(wi, ns, it.ng);
  r.fD = V3(0, 0, 0); r.fC = V3(0, 0, 0);
  if (flags & kEvalDiffuse) r.fD = evaluate_diffuse(nswi, alb, nsc, m, s, t);
  if (flags & kEvalConcentrated) {
    float nan = std::numeric_limits<float>::quiet_NaN();
    float at, ab; V3 tan, bit;
    anisotropy_params(it, ns, alpha, an, at, ab, tan, bit);
    r.fC = evaluate_concentrated(nswi, alb, m, s, t, wo, wi, alpha, at, ab, tan, bit, ns, nsc, false, V3(nan, nan, nan));
  }
  return r;
}
SampleResult MaterialCtx::sample(Rng& r, const Interaction& it, const V3& wo, int wl, float eta_out, int flags,
                                 bool adjoint) const {
  V3 alb = albedo(it);
  float rough = roughness(it);
  float m = metallic(it);
  V3 ns = shading_normal(it, wo, dot(it.ng, wo));
  float eta_mat = ior(wl);
  return principled_sample(r, it, wo, ns, alb, m, mat->specular, rough, mat->anisotropy, mat->transmission, wl, eta_out, eta_mat,
                           flags, adjoint);
}
bool MaterialCtx::has_diffuse_lobe(const Interaction& it) const {
  float m = metallic(it);
  float s = mat->specular, t = mat->transmission;
  return (1.0f - 0.5f * s) * (1.0 - t) * (1.0 - m) > 0.0f;
}
float MaterialCtx::sample_pdf(const Interaction& it, const V3& wo, const V3& wi, float eta_out) const {
  float ngwo = dot(it.ng, wo);
  V3 ns = shading_normal(it, wo, ngwo);
  float nswo = dot(ns, wo);
  float rough = roughness(it);
  float alpha = compute_alpha(rough);
  float m = metallic(it);
  float s = mat->specular, t = mat->transmission, an = mat->anisotropy;
  float eta_mat = mat->ior;
  bool from_out = ngwo >= 0.0f;
  float eo = from_out ? eta_out : eta_mat, et = from_out ? eta_mat : eta_out;
  ProbResult p = compute_probability(m, s, t, nswo, eo, et);
  if (alpha == 0.0f) return p.pD * eval_hemisphere_cos_pdf(ns, wi);
  float at, ab; V3 tan, bit;
  anisotropy_params(it, ns, alpha, an, at, ab, tan, bit);
  float ps = sample_ggx_vndf_global_density(ns, at, ab, tan, bit, wo, wi);
  float pd = eval_hemisphere_cos_pdf(ns, wi);
  return p.pS * ps + p.pD * pd;
}

// ============================================================== camera ====
void Camera::look_at(const V3& p, const V3& target) {
  pos = p;
  fwd = normalize(target - p);
  up = V3(0, 1, 0);
  up = up - dot(up, fwd) * fwd;
  up = normalize(up);
  right = cross(fwd, up);
}

void Camera::compute_ray(Rng& r, float x, float y, float W, float H, V3& o, V3& d) const {
  float fov = float(kPi) * fov_deg / 180.0f;
  float q = std::tan(fov * 0.5f);
  float lx = (x - 0.5f * W) / W * 2.0f;
  float ly = (y - 0.5f * H) / W * 2.0f;
  V3 dir = normalize(fwd + right * (q * lx) - up * (q * ly));
  if (aperture > 0.0f) {
    float dens;
    V2 off = sample_ngon_uniformly(r, blades, blade_rot, dens);
    float t = focal * dot(dir, fwd);
    V3 fp = pos + t * dir;
    V3 org = pos + aperture * off.x * up + aperture * off.y * right;
    o = org; d = normalize(fp - org);
  } else {
    o = pos; d = dir;
  }
}

float Camera::ray_angle(float x, float y, float W, float H) const {
  float fov = float(kPi) * fov_deg / 180.0f;
  float q = std::tan(fov * 0.5f);
  float lx1 = (x + 0.5f - 0.5f * W) / W * 2.0f;
  float ly1 = (y + 0.5f - 0.5f * H) / W * 2.0f;
  float lx2 = (x - 0.5f - 0.5f * W) / W * 2.0f;
  float ly2 = (y - 0.5f - 0.5f * H) / W * 2.0f;
  float ax = std::fabs(std::atan(q * lx1) - std::atan(q * lx2));
  float ay = std::fabs(std::atan(q * ly1) - std::atan(q * ly2));
  return 0.5f * ax + 0.5f * ay;
}

// ========================================================= environment ====
V3 Env::eval(const V3& d) const {
  if (!is_texture) return color;
  float th, ph; sph_from_dir(d, th, ph);
  float u = ph * float(0.5 * kInvPi);
  float v = 1.0f - th * float(kInvPi);
  float c[3]; tex.lookup(u, v, c);
  return V3(c[0], c[1], c[2]);
}

V3 Env::sample(Rng& r, float& density) const {
  SphDir sc;
  do {
    uint32_t idx = dist.sample(r);
    uint32_t W = uint32_t(tex.w), H = uint32_t(tex.h);
    uint32_t x = idx % W, y = idx / W;
    float hf = float(H), wf = float(W);
    float xi0 = r.uniform01f();
    float xi1 = r.uniform01f();
    float left = float(x) / wf;
    float right = (float(x) + 1.0f) / wf;
    float lower = (float(H) - (float(y) + 1.0f)) / hf;
    float upper = float(H - y) / hf;
    float u = (1.0f - xi0) * left + xi0 * right;
    float v = (1.0f - xi1) * lower + xi1 * upper;
    float pxy = weights[size_t(y) * W + x] / value_sum;
    density = wf * hf * pxy;
    float phi = u * 2.0f * float(kPi);
    float theta = (1.0f - v) * float(kPi);
    sc = sph_to_dir(theta, phi);
  } while (sc.sinTheta == 0.0f);
  density /= (2.0f * float(kPi) * float(kPi) * sc.sinTheta);
  return sc.dir;
}

float Env::density(const V3& d) const {
  float th, ph; sph_from_dir(d, th, ph);
  float u = ph * float(0.5 * kInvPi);
  float v = 1.0f - th * float(kInvPi);
  float s = nsin(th);
  size_t W = size_t(tex.w), H = size_t(tex.h);
  size_t x = std::min(size_t(u * float(W)), W - 1);
  size_t y = std::min(size_t((1.0f - v) * float(H)), H - 1);
  float e = float(W) * float(H) * weights[y * W + x] / value_sum;
  return e / std::max(1e-7f, 2.0f * float(kPi * kPi) * s);
}

// =============================================================== scene ====
static V3 json_v3(const Json& j) {
  return V3(float(j.at(size_t(0)).as_number()), float(j.at(size_t(1)).as_number()), float(j.at(size_t(2)).as_number()));
}

static int load_texture(Scene& sc, const std::string& path, int want_ch, bool srgb) {
  ImageF img; std::string err;
  if (!read_image(path, img, err)) throw std::runtime_error(err);
  Texture t; t.w = img.width; t.h = img.height;
  if (want_ch == 1) {
    if (img.channels != 1) throw std::runtime_error("could not read " + path + ", wrong number of channels, expected 1, found " + std::to_string(img.channels));
    t.ch = 1; t.data = img.data;
  } else {
    if (img.channels != 3 && img.channels != 4) throw std::runtime_error("could not read " + path + ", wrong number of channels, expected 3 or 4, found " + std::to_string(img.channels));
    t.ch = 3; t.data.resize(size_t(t.w) * t.h * 3);
    for (size_t i = 0; i < size_t(t.w) * t.h; ++i)
      for (int c = 0; c < 3; ++c) t.data[3 * i + c] = img.data[i * img.channels + c];
  }
  if (srgb) for (float& v : t.data) v = std::pow(std::max(0.0f, std::min(FLT_MAX, v)), 2.2f);
  sc.textures.push_back(std::move(t));
  return int(sc.textures.size() - 1);
}

void Scene::load_job(const std::string& job_path) {
  Json j = read_json_file(job_path);
  const Json* s = j.find("settings");
  if (s) {
    if (s->contains("roulette_start_depth")) settings.roulette_start = int(s->at("roulette_start_depth").as_number());
    if (s->contains("roulette_q")) settings.roulette_q = float(s->at("roulette_q").as_number());
    if (s->contains("width")) settings.width = uint32_t(s->at("width").as_number());
    if (s->contains("height")) settings.height = uint32_t(s->at("height").as_number());
    if (s->contains("num_threads")) settings.num_threads = uint32_t(s->at("num_threads").as_number());
    if (s->contains("max_depth")) settings.max_depth = int(s->at("max_depth").as_number());
    if (s->contains("num_samples")) settings.num_samples = int(s->at("num_samples").as_number());
    if (s->contains("use_mis")) settings.use_mis = s->at("use_mis").as_bool();
  }
  if (const Json* g = j.find("gb300")) {
    if (g->contains("seed")) settings.seed = uint64_t(g->at("seed").as_number());
  }
  load_scene(join_path(dir_of(job_path), j.at("scene").as_string()));
  // A constant non-black background with MIS on and no emissive triangle
  // makes the reference call exit(1) at the first light sample
  // (Scene.cpp:506-511); the oracle refuses such a job up front.
  if (settings.use_mis && light_tris.empty() && !env.is_texture && !env.is_zero())
    throw std::runtime_error("error: no light triangle found");
}

void Scene::load_scene(const std::string& scene_path) {
  std::string folder = dir_of(scene_path);
  Json j = read_json_file(scene_path);
  const Json& cj = j.at("camera");
  V3 p = json_v3(cj.at("position"));
  if (cj.contains("look_at")) camera.look_at(p, json_v3(cj.at("look_at")));
  else camera.look_at(p, p + V3(0, 0, -1));
  if (cj.contains("aperture")) camera.aperture = float(cj.at("aperture").as_number());
  if (cj.contains("focal_distance")) camera.focal = float(cj.at("focal_distance").as_number());
  if (cj.contains("exposure")) camera.exposure = float(cj.at("exposure").as_number());
  if (cj.contains("num_blades")) camera.blades = int(cj.at("num_blades").as_number());
  if (cj.contains("blade_rotation")) camera.blade_rot = float(cj.at("blade_rotation").as_number());
  const Json& w = j.at("world");
  if (w.contains("background_color")) {
    env.is_texture = false; env.color = json_v3(w.at("background_color"));
  } else {
    env.is_texture = true;
    std::string ep = join_path(folder, w.at("environment_texture").as_string());
    ImageF img; std::string err;
    if (!read_image(ep, img, err)) throw std::runtime_error(err);
    if (img.channels != 3 && img.channels != 4) throw std::runtime_error("environment texture needs 3 or 4 channels");
    env.tex.w = img.width; env.tex.h = img.height; env.tex.ch = 3; env.tex.clampU = false; env.tex.clampV = true;
    env.tex.data.resize(size_t(img.width) * img.height * 3);
    for (size_t i = 0; i < size_t(img.width) * img.height; ++i)
      for (int c = 0; c < 3; ++c) env.tex.data[3 * i + c] = img.data[i * img.channels + c];
    float hf = float(img.height);
    env.weights.resize(size_t(img.width) * img.height);
    for (int y = 0; y < img.height; ++y) {
      float theta = ((float(y) + 0.5f) / hf) * float(kPi);
      for (int x = 0; x < img.width; ++x) {
        const float* px = &env.tex.data[(size_t(y) * img.width + x) * 3];
        env.weights[size_t(y) * img.width + x] = norm(V3(px[0], px[1], px[2])) * std::sin(theta);
      }
    }
    env.dist.build(env.weights.data(), env.weights.size());
    float vs = 0.f;
    for (float v : env.weights) vs += v;
    env.value_sum = vs;
  }
  bool vary = false;
  if (w.contains("vary_glass_ior")) vary = w.at("vary_glass_ior").as_bool();
  // extension (not in the reference): "dispersion": {"model": "cauchy", "b", "wavelengths"}
  bool cauchy = false;
  float cauchy_b = 0.0042f, band_um[3] = {0.65f, 0.55f, 0.45f};
  if (w.contains("dispersion")) {
    const Json& dj = w.at("dispersion");
    cauchy = dj.at("model").as_string() == "cauchy";
    if (dj.contains("b")) cauchy_b = float(dj.at("b").as_number());
    if (dj.contains("wavelengths")) for (int k = 0; k < 3; ++k) band_um[k] = float(dj.at("wavelengths").at(size_t(k)).as_number());
  }

  std::string mesh = join_path(folder, j.at("mesh").as_string());
  ObjData obj; std::string err;
  if (!parse_obj(mesh, folder, obj, err)) throw std::runtime_error("TinyObjReader error " + err);
  vertices = obj.vertices; normals = obj.normals; texcoords = obj.texcoords;

  for (const ObjMaterial& om : obj.materials) {   // Scene.cpp:66-118
    Material m;
    m.transmission = 1.0f - om.dissolve;
    m.vary_ior = vary && m.transmission > 0.0f;
    if (!om.bump_texname.empty()) m.normal_tex = load_texture(*this, join_path(folder, om.bump_texname), 3, false);
    if (!om.diffuse_texname.empty()) m.albedo_tex = load_texture(*this, join_path(folder, om.diffuse_texname), 3, true);
    else m.albedo = V3(om.diffuse[0], om.diffuse[1], om.diffuse[2]);
    if (!om.specular_highlight_texname.empty()) m.roughness_tex = load_texture(*this, join_path(folder, om.specular_highlight_texname), 1, false);
    else m.roughness = 1.0f - std::sqrt(om.shininess / 1000.0f);
    if (!om.metallic_texname.empty()) m.metallic_tex = load_texture(*this, join_path(folder, om.metallic_texname), 1, false);
    else m.metallic = om.ambient[0];
    m.specular = om.specular[0];
    m.ior = om.ior;
    set_ior_bands(m, cauchy, cauchy_b, band_um);
    m.anisotropy = om.anisotropy;
    m.emission = V3(om.emission[0], om.emission[1], om.emission[2]);
    m.is_light = om.emission[0] > 0.0f || om.emission[1] > 0.0f || om.emission[2] > 0.0f;
    mats.push_back(m);
  }

  std::vector<float> areas;
  for (size_t s = 0; s < obj.shapes.size(); ++s) {   // Scene.cpp:122-189
    const ObjShape& sh = obj.shapes[s];
    shape_first.push_back(uint32_t(tris.size()));
    size_t nf = sh.num_face_vertices.size();
    for (size_t f = 0; f < nf; ++f) {
      if (sh.num_face_vertices[f] != 3) throw std::runtime_error(" dont support more than 3 points per face ");
      Tri t;
      t.geom = uint32_t(s); t.prim = uint32_t(f);
      for (int k = 0; k < 3; ++k) { t.vi[k] = sh.indices[3 * f + k].v; t.ni[k] = sh.indices[3 * f + k].vn; t.ti[k] = sh.indices[3 * f + k].vt; }
      t.mat = sh.material_ids[f];
      t.sg = sh.smoothing_group_ids[f];
      if (t.mat == -1) throw std::runtime_error(" error face has no material ");
      const ObjMaterial& om = obj.materials[t.mat];
      tris.push_back(t);
      for (int k = 0; k < 3; ++k) for (int c = 0; c < 3; ++c) tri_pos.push_back(vertices[3 * size_t(t.vi[k]) + c]);
      bool light = om.emission[0] > 0.0f || om.emission[1] > 0.0f || om.emission[2] > 0.0f;
      if (light) {
        if (om.diffuse[0] > 0.0f || om.diffuse[1] > 0.0f || om.diffuse[2] > 0.0f || om.specular[0] > 0.0f ||
            om.specular[1] > 0.0f || om.specular[2] > 0.0f)
          throw std::runtime_error(" don't support non black diffuse materials with emission ");
        light_tris.push_back(int32_t(tris.size() - 1));
        const float* q = &tri_pos[tri_pos.size() - 9];
        V3 p0(q[0], q[1], q[2]), p1(q[3], q[4], q[5]), p2(q[6], q[7], q[8]);
        areas.push_back(0.5f * norm(cross(p1 - p0, p2 - p0)));
      }
    }
  }
  light_dist.build(areas.data(), areas.size());
  float ta = 0.f;
  for (float a : areas) ta += a;
  total_light_area = ta;
  bvh.build(tri_pos.data(), tris.size());
}

Interaction Scene::interaction(int32_t ti, const V3& b, const V3& ng) const {
  const Tri& t = tris[ti];
  Interaction it;
  V3 xv[3];
  for (int k = 0; k < 3; ++k) xv[k] = V3(vertices[3 * size_t(t.vi[k])], vertices[3 * size_t(t.vi[k]) + 1], vertices[3 * size_t(t.vi[k]) + 2]);
  it.geomID = t.geom; it.primID = t.prim; it.bary = b;
  it.x = b.x * xv[0] + b.y * xv[1] + b.z * xv[2];
  it.ng = ng;
  it.material = t.mat;
  if (t.sg != 0) {
    V3 nv[3];
    bool all = true;
    for (int k = 0; k < 3; ++k) {
      if (t.ni[k] >= 0) nv[k] = V3(normals[3 * size_t(t.ni[k])], normals[3 * size_t(t.ni[k]) + 1], normals[3 * size_t(t.ni[k]) + 2]);
      else { all = false; break; }
    }
    if (!all) { V3 n = normalize(cross(xv[1] - xv[0], xv[2] - xv[0])); nv[0] = nv[1] = nv[2] = n; }
    it.ns_default = normalize(b.x * nv[0] + b.y * nv[1] + b.z * nv[2]);
    it.h = 0.0f;
    for (int k = 0; k < 3; ++k) {
      float nvng = dot(it.ng, nv[k]);
      float hi = nvng == 0.0f ? 1e6f : (dot(xv[k], nv[k]) - dot(it.x, nv[k])) / nvng;
      it.h += b[k] * b[k] * hi;
    }
  } else {
    it.ns_default = it.ng;
    it.h = 0.0f;
  }
  bool uv_ok = true;
  float uv[3][2];
  for (int k = 0; k < 3; ++k) {
    size_t idx = size_t(int64_t(t.ti[k]));
    if (2 * idx + 1 >= texcoords.size()) { uv_ok = false; break; }
    uv[k][0] = texcoords[2 * idx]; uv[k][1] = texcoords[2 * idx + 1];
  }
  if (uv_ok) {
    it.has_uv = true;
    it.uv[0] = uv[0][0] * b.x + uv[1][0] * b.y + uv[2][0] * b.z;
    it.uv[1] = uv[0][1] * b.x + uv[1][1] * b.y + uv[2][1] * b.z;
  }
  it.tangent = orthonormalized_or_any(it.ng, V3(-it.x.z, 0.0f, it.x.x));
  it.bitangent = cross(it.ng, it.tangent);
  return it;
}

V3 Scene::ray_x(const Interaction& it, bool outside) const {
  float eps = 1e-5f;
  float hmin = std::max(eps, norm(it.x) * eps);
  return it.x + it.ng * (1.01f * (outside ? std::max(0.0f, it.h) + hmin : std::min(0.0f, it.h) - hmin));
}

void Scene::ray_hit(const V3& o, const V3& d, Hit& h, BvhStats* st) const {
  float of[3] = {o.x, o.y, o.z}, df[3] = {d.x, d.y, d.z};
  BvhHit bh = bvh.intersect(of, df, 1e-6f, std::numeric_limits<float>::infinity(), st);
  h = Hit();
  h.wfrom = -d;
  if (bh.prim < 0) return;
  h.hit = true;
  h.tri = bh.prim;
  h.geomID = tris[bh.prim].geom; h.primID = tris[bh.prim].prim;
  h.t = bh.t;
  V3 b(1.0f - bh.u - bh.v, bh.u, bh.v);
  V3 ng = normalize(V3(bh.ng[0], bh.ng[1], bh.ng[2]));
  h.it = interaction(bh.prim, b, ng);
}

V3 Scene::emission(const V3& wo, const Hit& h) const {
  if (dot(h.it.ng, wo) <= 0.0f) return V3(0, 0, 0);
  return mats[h.it.material].emission * float(kInvPi);
}

Interaction Scene::sample_light_position(Rng& r, float& pdfA) const {
  if (light_tris.empty()) { std::fprintf(stderr, "error: no light triangle found \n"); std::exit(1); }
  pdfA = 1.0f / total_light_area;
  uint32_t k = light_dist.sample(r);
  int32_t ti = light_tris[k];
  const float* q = &tri_pos[9 * size_t(ti)];
  V3 p0(q[0], q[1], q[2]), p1(q[3], q[4], q[5]), p2(q[6], q[7], q[8]);
  V3 n = normalize(cross(p1 - p0, p2 - p0));
  V3 b = sample_triangle_uniformly(r);
  return interaction(ti, b, n);
}

void Scene::sample_emission_ray(Rng& r, V3& flux, V3& o, V3& d) const {
  float pPos, pDir;
  Interaction it = sample_light_position(r, pPos);
  V3 dir = sample_hemisphere_cos(r, it.ng, pDir);
  V3 L = mats[it.material].emission * float(kInvPi);      // Scene.cpp:460-470 (no side test)
  flux = L * (std::fabs(dot(it.ng, dir)) / (pPos * pDir));
  o = ray_x(it, true);
  d = dir;
}

void Scene::sample_light_ray(Rng& r, const Interaction& p, float& pdf, V3& o, V3& d, Hit& h, bool& visible, BvhStats* st) const {
  float psurf = !env.is_texture ? 1.0f : (!light_tris.empty() ? 0.5f : 0.0f);
  float xi = r.uniform01f();
  if (xi < psurf) {
    float pdfA;
    Interaction it2 = sample_light_position(r, pdfA);
    V3 diff = it2.x - p.x;
    o = ray_x(p, dot(p.ng, diff) >= 0.0f);
    d = normalize(it2.x - o);
    ray_hit(o, d, h, st);
    visible = h.geomID == it2.geomID && h.primID == it2.primID;
    if (visible) pdf = light_ray_density(p, o, d, h);
  } else {
    d = env.sample(r, pdf);
    o = ray_x(p, dot(p.ng, d) >= 0.0f);
    ray_hit(o, d, h, st);
    visible = is_surface_light(h) || !h.hit;
    if (visible) pdf = light_ray_density(p, o, d, h);
  }
}

float Scene::light_ray_density(const Interaction& p, const V3& o, const V3& d, const Hit& h) const {
  (void)p;
  bool surf = is_surface_light(h);
  bool inf = !h.hit;
  if (!surf && !inf) return 0.0f;
  float psurf = !env.is_texture ? 1.0f : (!light_tris.empty() ? 0.5f : 0.0f);
  float res;
  if (surf) {
    float pdfA = 1.0f / total_light_area;
    float dsq = std::max(1e-5f, norm_sq(o - h.it.x));
    float pw = pdfA * dsq / (1e-7f + std::fabs(dot(h.it.ng, d)));
    res = psurf * pw;
    if (env.is_texture) res += (1.0f - psurf) * env.density(d);
  } else {
    res = env.is_texture ? (1.0f - psurf) * env.density(d) : 0.0f;
  }
  return res;
}

// ======================================================== light ray info ====
void LightRayInfo::update_media(const Scene& sc, const Hit& h, const V3& wto) {
  float nf = dot(h.it.ng, h.wfrom);
  float nt = dot(h.it.ng, wto);
  if (nf >= 0.0f && nt < 0.0f) {
    V3 t = sc.albedo(h.it);
    float ior_in = sc.ctx(h.it).ior(wavelength);
    media.push_back(Medium{int32_t(h.geomID), t, ior_in});
    recompute();
  } else if (nf < 0.0f && nt >= 0.0f) {
    for (size_t i = 0; i < media.size(); ++i)
      if (media[i].geom == int32_t(h.geomID)) { media.erase(media.begin() + i); recompute(); break; }
  }
}
void LightRayInfo::recompute() {
  for (const Medium& m : media) if (m.geom != -1) { transmittance = m.T; return; }
  transmittance = V3(1, 1, 1);
}
int LightRayInfo::sample_wavelength(Rng& r, bool sample, float& prob) {
  if (wavelength == -1 && sample) {
    V3 p = V3(1, 1, 1) / vsum(V3(1, 1, 1));
    float xi = r.uniform01f();
    if (xi < p.x) { wavelength = 0; prob = p.x; }
    else if (xi < p.x + p.y) { wavelength = 1; prob = p.y; }
    else { wavelength = 2; prob = p.z; }
  } else prob = 1.0f;
  return wavelength;
}
float LightRayInfo::outside_ior(const Hit& h) const {
  if (dot(h.wfrom, h.it.ng) < 0.0f) {
    int idx = -1;
    for (size_t i = 0; i < media.size(); ++i) if (media[i].geom == int32_t(h.geomID)) { idx = int(i); break; }
    if (idx == -1) return 1.0f;
    if (media.size() == 1) return 1.0f;
    return idx == 0 ? media[1].ior : media[0].ior;
  }
  if (media.empty()) return 1.0f;
  return media[0].ior;
}

// ============================================================ integrator ====
V3 beers_law(const V3& T, float d) {              // core/include/Hasty/PathTracing.h:46-59
  if (T == V3(1, 1, 1)) return V3(1, 1, 1);
  V3 r;
  for (int i = 0; i < 3; ++i) r[i] = T[i] <= 0.0f ? 0.0f : npow(T[i], 1.0f * d);
  return r;
}

struct MisSample { V3 o, d; LightRayInfo lr; Hit hit; V3 thrD, thrC; float pdf; };

V3 estimate_radiance(const Scene& sc, Rng& r, LightRayInfo& lr, const V3& ro, const V3& rd, V3& normal, V3& albedo,
                     int depth, const Hit* pre, RenderStats& st) {
  if (depth >= sc.settings.max_depth) return V3(0, 0, 0);
  Hit local;
  const Hit& hit = pre ? *pre : local;
  BvhStats bs;
  if (!pre) { sc.ray_hit(ro, rd, local, &bs); st.rays++; }
  if (hit.hit) {
    if (depth == 0) { normal = hit.it.ns_default; albedo = sc.albedo(hit.it); }
    V3 thr = beers_law(lr.transmittance, norm(hit.it.x - ro));
    if (sc.is_surface_light(hit)) return cwise(thr, sc.emission(-rd, hit));
    st.shaded++;
    bool two = sc.has_light() && sc.settings.use_mis;     // MIS.cpp:60-72
    int nstrat = two ? 2 : 1;
    int light_idx = two ? 0 : -1;
    float pdfs[2] = {0, 0};
    float q = depth >= sc.settings.roulette_start ? sc.settings.roulette_q : 0.0f;
    if (r.uniform01f() < q) return V3(0, 0, 0);
    thr = thr / (1.0f - q);
    V3 est(0, 0, 0);
    V3 wo = -rd;
    for (int s = 0; s < nstrat; ++s) {
      MisSample ms; ms.lr = lr;
      if (s == light_idx) {                                // MIS.cpp:32-54
        bool vis;
        sc.sample_light_ray(r, hit.it, ms.pdf, ms.o, ms.d, ms.hit, vis, &bs);
        st.rays++;
        if (!vis || ms.pdf == 0.0f) { ms.thrD = ms.thrC = V3(0, 0, 0); ms.pdf = 0.0f; }
        else {
          EvalResult ev = sc.ctx(hit.it).evaluate(hit.it, wo, ms.d, ms.lr.outside_ior(hit));
          float m = std::fabs(dot(ms.d, hit.it.ng)) / ms.pdf;
          ms.thrD = ev.fD * m; ms.thrC = ev.fC * m;
        }
      } else {                                             // MIS.cpp:6-26, Scene.cpp:328-338
        MaterialCtx mc = sc.ctx(hit.it);
        float prob;
        int wl = ms.lr.sample_wavelength(r, mc.mat->vary_ior, prob);
        float eta_out = ms.lr.outside_ior(hit);
        SampleResult sr = mc.sample(r, hit.it, hit.wfrom, wl, eta_out);
        sr.thrD = sr.thrD / prob; sr.thrC = sr.thrC / prob;
        if (sr.pdf == 0.0f) { ms.thrD = ms.thrC = V3(0, 0, 0); ms.pdf = 0.0f; }
        else {
          ms.o = sc.ray_x(hit.it, sr.outside); ms.d = sr.dir;
          ms.thrD = sr.thrD; ms.thrC = sr.thrC; ms.pdf = sr.pdf;
          sc.ray_hit(ms.o, ms.d, ms.hit, &bs);
          st.rays++;
        }
      }
      pdfs[s] = ms.pdf;
      V3 thr2 = cwise(thr, ms.thrD + ms.thrC);
      if (thr2 == V3(0, 0, 0) || (hit.geomID == ms.hit.geomID && hit.primID == ms.hit.primID)) continue;
      for (int j = 0; j < nstrat; ++j) {
        if (j == s) continue;
        if (j == light_idx) pdfs[j] = sc.light_ray_density(hit.it, ms.o, ms.d, ms.hit);
        else pdfs[j] = sc.ctx(hit.it).sample_pdf(hit.it, hit.wfrom, ms.d, ms.lr.outside_ior(hit));
      }
      float ssum = 0.0f;
      for (int j = 0; j < nstrat; ++j) ssum += pdfs[j] * pdfs[j];
      float w = pdfs[s] * pdfs[s] / ssum;
      thr2 = thr2 * w;
      ms.lr.update_media(sc, hit, ms.d);
      V3 n2, a2;
      V3 li = estimate_radiance(sc, r, ms.lr, ms.o, ms.d, n2, a2, depth + 1, &ms.hit, st);
      est = est + cwise(li, thr2);
    }
    st.nodes += bs.nodes; st.tris += bs.tris;
    return est;
  }
  st.nodes += bs.nodes; st.tris += bs.tris;
  V3 T = beers_law(lr.transmittance, 1e6f);
  V3 L = cwise(T, sc.env.eval(rd));
  normal = V3(0, 0, 0);
  albedo = L;
  return L;
}

V3 render_sample(const Scene& sc, uint32_t x, uint32_t y, uint32_t pass, V3& normal, V3& albedo, RenderStats& st) {
  uint32_t W = sc.settings.width, H = sc.settings.height;
  Rng r(path_key(sc.settings.seed, y * W + x, pass));
  float ox = halton(2, pass), oy = halton(3, pass);
  V3 o, d;
  sc.camera.compute_ray(r, float(x) + ox, float(y) + oy, float(W), float(H), o, d);
  LightRayInfo lr;
  normal = V3(0, 0, 0); albedo = V3(0, 0, 0);
  st.paths++;
  return estimate_radiance(sc, r, lr, o, d, normal, albedo, 0, nullptr, st);
}

}  // namespace hor
