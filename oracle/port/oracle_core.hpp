// Oracle (test infrastructure only -- never linked into the product).
//
// CPU restatement of HastyRenderer's unidirectional path tracer, written to
// follow the reference's arithmetic step by step so that it can be compared
// bit-for-bit with the reference's own code built under oracle/_ref, and
// statistically/per-sample with the CUDA integrator. Each function names the
// reference lines it restates (paths relative to the reference project).
#pragma once
#include <limits>
#include <cstring>
#include <cmath>
#include <cfloat>
#include <cstdint>
#include <memory>
#include <string>
#include <vector>
#include "hor_rng.hpp"
#include "hor_io.hpp"
#include "hor_bvh.hpp"

namespace hor {

constexpr double kPi = 3.1415926535897932384;       // core/src/VMath.cpp:6
constexpr double kInvPi = 1.0 / 3.1415926535897932384;

// ------------------------------------------------------------ vectors ----
// Vec3f semantics of core/include/Hasty/VMath.h:120-330 (component-wise
// division in normalize, float*Vec3f == Vec3f*float, left-to-right dot).
struct V3 {
  float x = 0, y = 0, z = 0;
  V3() = default;
  V3(float a, float b, float c) : x(a), y(b), z(c) {}
  float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
  float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
  static V3 fill(float f) { return V3(f, f, f); }
};
inline V3 operator+(const V3& a, const V3& b) { return V3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V3 operator-(const V3& a, const V3& b) { return V3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 operator-(const V3& a) { return V3(-a.x, -a.y, -a.z); }
inline V3 operator*(const V3& a, float s) { return V3(a.x * s, a.y * s, a.z * s); }
inline V3 operator*(float s, const V3& a) { return a * s; }
inline V3 operator/(const V3& a, float s) { return V3(a.x / s, a.y / s, a.z / s); }
inline bool operator==(const V3& a, const V3& b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
inline bool operator!=(const V3& a, const V3& b) { return !(a == b); }
inline float dot(const V3& a, const V3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(const V3& a, const V3& b) {
  return V3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline V3 cwise(const V3& a, const V3& b) { return V3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline float norm_sq(const V3& a) { return dot(a, a); }
inline float norm(const V3& a) { return std::sqrt(norm_sq(a)); }
inline V3 normalize(const V3& a) { return a / norm(a); }
inline float vsum(const V3& a) { return a.x + a.y + a.z; }
inline float mixf(float a, float b, float l) { return (1.0f - l) * a + l * b; }
inline V3 mixv(const V3& a, const V3& b, float l) {
  return V3((1.0f - l) * a.x + l * b.x, (1.0f - l) * a.y + l * b.y, (1.0f - l) * a.z + l * b.z);
}
inline float sq(float f) { return f * f; }
inline float pow5(float f) { float q = f * f; q = q * q; return f * q; }  // powci<5>, VMath.h:29-46
inline bool finite3(const V3& v) { return std::isfinite(v.x) && std::isfinite(v.y) && std::isfinite(v.z); }

// VMath.h:451-488
inline V3 orthonormalized(const V3& v1, const V3& v2) {
  V3 r = v2 - dot(v2, v1) * v1;
  float len = norm(r);
  return r / len;
}
inline V3 any_orthonormal(const V3& v1) {
  if (std::fabs(v1.x) < 0.7f) return orthonormalized(v1, V3(1, 0, 0));
  return orthonormalized(v1, V3(0, 1, 0));
}
inline V3 orthonormalized_or_any(const V3& v1, const V3& v2) {
  V3 r = v2 - dot(v2, v1) * v1;
  float len = norm(r);
  if (len < 1e-7f) return any_orthonormal(v1);
  return r / len;
}

// RotationBetweenTwoVectors / applyRotation, VMath.h:558-607 (Rodrigues).
struct Rotation {
  float a; V3 b, c, d;
  Rotation(const V3& from, const V3& to) {
    float cosA = dot(from, to);
    float onePlus = 1.0f + cosA;
    if (std::fabs(onePlus) > FLT_EPSILON) {
      V3 k = cross(from, to);
      a = cosA; b = k; c = k; d = k / onePlus;
    } else {
      V3 k = any_orthonormal(from);
      a = -1.0f; b = V3(0, 0, 0); c = k; d = k * 2.0f;
    }
  }
  V3 apply(const V3& x) const { return x * a + cross(b, x) + c * dot(d, x); }
  V3 apply_inverse(const V3& x) const { return x * a - cross(b, x) + c * dot(d, x); }
};

// VMath.h:652-668
inline V3 reflect(const V3& inc, const V3& n) { return inc - 2.0f * dot(n, inc) * n; }
inline V3 reflect_across(const V3& out, const V3& n) { return reflect(-out, n); }

// Test switch (hor_set_ulp_nudge, off by default): moves every result of the
// per-sample sin, cos, atan2, acos and pow calls by one ulp, up or down by a
// hash of the argument's bits. With it on, the oracle measures how often a
// last-ulp change of the math library changes a sample (a branch decision
// flips), which is the kind of difference CUDA's device functions make
// against the host's. Off, these wrappers are the plain calls.
extern bool g_ulp_nudge;
template <class T>
inline T nudge_ulp(T r, T x) {
  if (!g_ulp_nudge) return r;
  uint64_t b = 0;
  std::memcpy(&b, &x, sizeof(T));
  const bool up = ((b * 0x9E3779B97F4A7C15ull) >> 63) != 0;
  return std::nextafter(r, up ? std::numeric_limits<T>::infinity() : -std::numeric_limits<T>::infinity());
}
template <class T> inline T nsin(T x) { return nudge_ulp(T(std::sin(x)), x); }
template <class T> inline T ncos(T x) { return nudge_ulp(T(std::cos(x)), x); }
template <class T> inline T nacos(T x) { return nudge_ulp(T(std::acos(x)), x); }
template <class T> inline T natan2(T y, T x) { return nudge_ulp(T(std::atan2(y, x)), T(y + x)); }
template <class T> inline T npow(T a, T e) { return nudge_ulp(T(std::pow(a, e)), a); }

// SphericalCoordinates, VMath.h:672-700 (y up).
struct SphDir { float cosTheta, sinTheta; V3 dir; };
inline SphDir sph_to_dir(float theta, float phi) {
  SphDir r; r.cosTheta = ncos(theta); r.sinTheta = nsin(theta);
  float sp = nsin(phi), cp = ncos(phi);
  r.dir = V3(r.sinTheta * cp, r.cosTheta, r.sinTheta * sp);
  return r;
}
inline void sph_from_dir(const V3& d, float& theta, float& phi) {
  theta = nacos(d.y);
  phi = natan2(d.z, d.x);
  phi = phi < 0.0f ? phi + float(2.0 * kPi) : phi;
}

// floor_int32 / fmod1p1, VMath.h:18-27
inline int32_t floor_int32(double x) { int i = (int)x; return i - (i > x); }
inline float fmod1p1(float f) { return f - float(floor_int32(f)); }

// ------------------------------------------------------------ sampling ----
struct V2 { float x, y; };
V2 sample_disk_uniformly(Rng& r, float& pdf);                                  // Sample.cpp:5-11
V2 sample_ngon_uniformly(Rng& r, int blades, float rotation, float& pdf);       // Sample.cpp:12-42
V3 sample_sphere_uniformly(Rng& r, float& pdf);                                // Sample.cpp:43-56
V3 sample_hemisphere_uniformly(Rng& r, const V3& n, float& pdf);               // Sample.cpp:59-75
V3 sample_hemisphere_cos(Rng& r, const V3& n, float& pdf);                     // Sample.cpp:77-108
float eval_hemisphere_cos_pdf(const V3& n, const V3& d);                       // Sample.cpp:109-117
V3 sample_cosine_lobe(Rng& r, const V3& lobe, float e, float& pdf);            // Sample.cpp:122-151
float eval_cosine_lobe_pdf(const V3& lobe, float e, const V3& d);              // Sample.cpp:153-158
V3 sample_triangle_uniformly(Rng& r);                                          // Sample.cpp:160-180

// ---------------------------------------------------------------- BSDF ----
bool refraction_direction(const V3& wi, const V3& n, float eta_i, float eta_t, V3& wt);   // BRDF.cpp:11-30
bool refraction_cos_t(float cos_i, float eta_i, float eta_t, float& cos_t);                // BRDF.cpp:31-49
V3 refraction_direction_from_angles(const V3& wi, const V3& n, float ratio, float ci, float ct);  // BRDF.cpp:51-61
float fresnel_dielectric(float ci, float ct, float eta_i, float eta_t);                    // BRDF.cpp:74-81
float dggx_iso(float nh, float alpha);                                                     // BRDF.cpp:130-135
V3 sample_dggx(Rng& r, const V3& n, float alpha, const V3& d1, float& pdf);               // BRDF.cpp:84-121
float sample_dggx_density(const V3& n, float alpha, const V3& d1, const V3& d2);          // BRDF.cpp:122-129
float dggx(float nh, float th, float bh, float at, float ab);                              // BRDF.cpp:149-153
float smith_ggx(float nv, float tv, float bv, float at, float ab);                         // BRDF.cpp:155-159
V3 sample_ggx_vndf(const V3& wo, float ax, float ay, float xi1, float xi2);               // BRDF.cpp:163-185
V3 sample_ggx_vndf_global(Rng& r, const V3& n, float at, float ab, const V3& t, const V3& b, const V3& d1, float& pdf);  // BRDF.cpp:186-213
float sample_ggx_vndf_global_density(const V3& n, float at, float ab, const V3& t, const V3& b, const V3& d1, const V3& d2);  // BRDF.cpp:214-226

struct Interaction {            // SurfaceInteraction, core/include/Hasty/Scene.h:20-33
  uint32_t geomID = 0, primID = 0;
  float h = 0;
  V3 x, ng, ns_default, tangent, bitangent;
  int32_t material = -1;
  bool has_uv = false;
  float uv[2] = {0, 0};
  V3 bary;
};

struct Texture {                // Texture<T>, core/include/Hasty/Texture.h:119-139
  int w = 0, h = 0, ch = 0;
  std::vector<float> data;
  bool clampU = false, clampV = false;
  void lookup(float u, float v, float* out) const;
};

struct Material {               // PrincipledBRDF members, BRDF.h:161-171 + MTL emission
  V3 albedo; int albedo_tex = -1;
  float roughness = 0; int roughness_tex = -1;
  float metallic = 0; int metallic_tex = -1;
  float specular = 0, ior = 1, anisotropy = 0, transmission = 0;
  int normal_tex = -1;
  bool vary_ior = false;
  V3 emission;
  bool is_light = false;
  float ior_band[3] = {1, 1, 1};   // band IORs (reference ratios, or the Cauchy extension)
};

// Band IORs of a material: the reference's ratios, or Cauchy's ior + b / lambda^2.
void set_ior_bands(Material& m, bool cauchy, float b, const float* band_um);

struct SampleResult { bool outside; V3 dir, thrD, thrC; float pdf; };     // BRDF.h:58-70
struct EvalResult { V3 fD, fC, ns; };                                      // BRDF.h:46-56
struct ProbResult { bool none; float pD, pS, pR; bool refr; float FD, cosT; };  // BRDF.h:102-111

// ShaderEvalFlag (BRDF.h): which lobes a sample or an evaluation covers.
enum : int { kEvalDiffuse = 1, kEvalConcentrated = 2, kEvalAll = 3 };

float compute_alpha(float roughness);                                                          // BRDF.cpp:253-263
ProbResult compute_probability(float m, float s, float t, float cos_o, float eta_o, float eta_r,
                               int flags = kEvalAll);                                          // BRDF.cpp:264-307
void anisotropy_params(const Interaction& it, const V3& ns, float alpha, float aniso, float& at, float& ab, V3& t, V3& b);  // :308-316
V3 evaluate_diffuse(float nsWi, const V3& albedo, float nscale, float m, float s, float t);   // :319-326
V3 evaluate_concentrated(float nsWi, const V3& albedo, float m, float s, float t, const V3& wo, const V3& wi,
                         float alpha, float at, float ab, const V3& tan, const V3& bit, const V3& ns,
                         float nscale, bool force, const V3& FD);                              // :328-394
SampleResult principled_sample(Rng& r, const Interaction& it, const V3& wo, const V3& ns, const V3& albedo,
                               float m, float s, float rough, float aniso, float t, int wavelength,
                               float eta_out, float eta_mat, int flags = kEvalAll,
                               bool adjoint = false);                                          // :397-579

struct MaterialCtx {            // evaluation of a PrincipledBRDF at a hit (texture lookups)
  const Material* mat;
  const std::vector<Texture>* tex;
  V3 albedo(const Interaction& it) const;
  float roughness(const Interaction& it) const;
  float metallic(const Interaction& it) const;
  float ior(int wavelength) const;                                          // BRDF.cpp:589-603
  V3 shading_normal(const Interaction& it, const V3& wo, float ngwo) const;  // BRDF.cpp:604-628
  EvalResult evaluate(const Interaction& it, const V3& wo, const V3& wi, float eta_out,
                      int flags = kEvalAll) const;                                          // :630-679
  SampleResult sample(Rng& r, const Interaction& it, const V3& wo, int wavelength, float eta_out,
                      int flags = kEvalAll, bool adjoint = false) const;                    // :681-700
  bool has_diffuse_lobe(const Interaction& it) const;                                       // :743-750
  float sample_pdf(const Interaction& it, const V3& wo, const V3& wi, float eta_out) const;  // :702-742
};

// ----------------------------------------------------------- scene ----
struct Camera {                 // core/include/Hasty/Camera.h:36-46, Camera.cpp:9-38
  V3 pos = V3(0, 0, 0), fwd = V3(0, 0, -1), right = V3(1, 0, 0), up = V3(0, 1, 0);
  float fov_deg = 45.0f, aperture = 0, focal = 1, exposure = 0;
  int blades = 8; float blade_rot = 0;
  void look_at(const V3& p, const V3& target);
  void compute_ray(Rng& r, float px, float py, float W, float H, V3& o, V3& d) const;  // Camera.cpp:41-81
  float ray_angle(float px, float py, float W, float H) const;                          // Camera.cpp:83-98
};

struct Settings {               // RenderSettings defaults, RenderJob.h:15-30
  int roulette_start = 1; float roulette_q = 0.3f;
  uint32_t width = 720, height = 720, num_threads = 4;
  int max_depth = 30, num_samples = 32; bool use_mis = true;
  uint64_t seed = 0;
};

struct Env {                    // EnvironmentTexture + ImageDistribution, Environment.h:47-171
  bool is_texture = false;
  V3 color;
  Texture tex;
  std::vector<float> weights;   // notNormalizedPdf
  DiscreteDist dist;
  float value_sum = 0;
  bool is_zero() const { return !is_texture && color == V3(0, 0, 0); }
  V3 eval(const V3& d) const;
  V3 sample(Rng& r, float& density) const;
  float density(const V3& d) const;
};

struct Tri { uint32_t geom, prim; int32_t vi[3], ni[3], ti[3]; int32_t mat; uint32_t sg; };

struct Hit {                    // RayHit (Scene.h:35-46) for the oracle
  bool hit = false;
  uint32_t geomID = 0xFFFFFFFFu, primID = 0xFFFFFFFFu;
  int32_t tri = -1;
  float t = 0;
  V3 wfrom;
  Interaction it;
};

struct Scene {
  Camera camera;
  Settings settings;
  Env env;
  std::vector<float> vertices, normals, texcoords;
  std::vector<Tri> tris;
  std::vector<float> tri_pos;   // 9 floats per triangle
  std::vector<uint32_t> shape_first;
  std::vector<Material> mats;
  std::vector<Texture> textures;
  std::vector<int32_t> light_tris;
  DiscreteDist light_dist;
  float total_light_area = 0;
  Bvh2 bvh;

  void load_job(const std::string& job_path);
  void load_scene(const std::string& scene_path);
  int32_t tri_index(uint32_t geom, uint32_t prim) const { return int32_t(shape_first[geom] + prim); }
  Interaction interaction(int32_t tri, const V3& bary, const V3& ng) const;   // Scene.cpp:202-255
  V3 ray_x(const Interaction& it, bool outside) const;                        // Scene.cpp:257-270
  void ray_hit(const V3& o, const V3& d, Hit& h, BvhStats* st) const;         // Scene.cpp:281-303
  bool has_light() const { return !light_tris.empty() || !env.is_zero(); }
  bool is_surface_light(const Hit& h) const { return h.hit && mats[h.it.material].is_light; }
  V3 emission(const V3& wo, const Hit& h) const;                              // Scene.cpp:471-477
  V3 albedo(const Interaction& it) const { return ctx(it).albedo(it); }
  MaterialCtx ctx(const Interaction& it) const { return MaterialCtx{&mats[it.material], &textures}; }
  Interaction sample_light_position(Rng& r, float& pdfA) const;               // Scene.cpp:506-526
  void sample_emission_ray(Rng& r, V3& flux, V3& o, V3& d) const;              // sampleLightRay, Scene.cpp:527-537
  bool has_surface_light() const { return !light_tris.empty(); }
  void sample_light_ray(Rng& r, const Interaction& p, float& pdf, V3& o, V3& d, Hit& h, bool& visible, BvhStats* st) const;  // :538-586
  float light_ray_density(const Interaction& p, const V3& o, const V3& d, const Hit& h) const;  // :587-616
};

struct Medium { int32_t geom; V3 T; float ior; };
struct LightRayInfo {           // core/src/LightRayInfo.cpp, LightRayInfo.h:30-55
  int wavelength = -1;
  std::vector<Medium> media;
  V3 transmittance = V3(1, 1, 1);
  void update_media(const Scene& sc, const Hit& h, const V3& wto);
  void recompute();
  int sample_wavelength(Rng& r, bool sample, float& prob);
  float outside_ior(const Hit& h) const;
};

V3 beers_law(const V3& T, float d);              // core/include/Hasty/PathTracing.h:46-59

struct RenderStats { uint64_t rays = 0, nan = 0, nodes = 0, tris = 0, shaded = 0, paths = 0; };

// estimateRadiance, core/src/PathTracing.cpp:21-95
V3 estimate_radiance(const Scene& sc, Rng& r, LightRayInfo& lr, const V3& ro, const V3& rd, V3& normal, V3& albedo,
                     int depth, const Hit* pre, RenderStats& st);

// One camera sample of pixel (x, y) in pass `pass`, RNG keyed per path.
V3 render_sample(const Scene& sc, uint32_t x, uint32_t y, uint32_t pass, V3& normal, V3& albedo, RenderStats& st);

}  // namespace hor
