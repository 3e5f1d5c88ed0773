// Device-side shading math of the path tracer: vectors, the PCG32 path
// streams, sampling routines, the Principled BSDF, textures, environment,
// camera and light sampling. Each routine follows the reference function it
// names (paths relative to the reference project); the integrator kernels in
// integrator.cu call them per path.
//
// integrator.cu is compiled without FMA contraction (--fmad=false) so that
// products and sums round as the reference's scalar C++ does; transcendental
// functions are CUDA's (sinf, cosf, acosf, atan2f, powf, fmodf, sqrtf).
#pragma once
#include <cstdint>
#include <cfloat>
#include "bounds.cuh"
#include "hasty_types.h"

// Which large shading routines are compiled out of line (one shared copy,
// called) instead of inlined at every call site; bits of HASTY_OUTLINE_MASK:
//   1 bsdf_sample, 2 bsdf_eval + bsdf_pdf, 4 make_inter, 8 environment and
//   light densities and sampling, 16 shade_ctx. Only code placement changes;
//   every result is the same.
#ifndef HASTY_OUTLINE_MASK
#define HASTY_OUTLINE_MASK 0
#endif
#if (HASTY_OUTLINE_MASK & 1)
#define HFN_SAMPLE __device__ __noinline__
#else
#define HFN_SAMPLE __device__ __forceinline__
#endif
#if (HASTY_OUTLINE_MASK & 2)
#define HFN_EVAL __device__ __noinline__
#else
#define HFN_EVAL __device__ __forceinline__
#endif
#if (HASTY_OUTLINE_MASK & 4)
#define HFN_INTER __device__ __noinline__
#else
#define HFN_INTER __device__ __forceinline__
#endif
#if (HASTY_OUTLINE_MASK & 8)
#define HFN_ENV __device__ __noinline__
#else
#define HFN_ENV __device__ __forceinline__
#endif
#if (HASTY_OUTLINE_MASK & 16)
#define HFN_CTX __device__ __noinline__
#else
#define HFN_CTX __device__ __forceinline__
#endif

namespace hasty {
namespace dev {

constexpr double kPi = 3.1415926535897932384;
constexpr double kInvPi = 1.0 / 3.1415926535897932384;
#define HPI_F float(3.1415926535897932384)
#define HINVPI_F float(1.0 / 3.1415926535897932384)
#define HTWOPI_F float(2.0 * 3.1415926535897932384)

// ---------------------------------------------------------------- vec3 --
struct V3 {
  float x, y, z;
  __device__ V3() : x(0.f), y(0.f), z(0.f) {}
  __device__ V3(float a, float b, float c) : x(a), y(b), z(c) {}
  __device__ float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
  __device__ void set(int i, float v) { if (i == 0) x = v; else if (i == 1) y = v; else z = v; }
};
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return V3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return V3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ V3 operator-(V3 a) { return V3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ V3 operator*(V3 a, float s) { return V3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ V3 operator*(float s, V3 a) { return a * s; }
__device__ __forceinline__ V3 operator/(V3 a, float s) { return V3(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ bool eq(V3 a, V3 b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
__device__ __forceinline__ bool is_zero(V3 a) { return a.x == 0.f && a.y == 0.f && a.z == 0.f; }
__device__ __forceinline__ float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ V3 cross(V3 a, V3 b) { return V3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
__device__ __forceinline__ V3 cwise(V3 a, V3 b) { return V3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ float norm_sq(V3 a) { return dot(a, a); }
__device__ __forceinline__ float norm(V3 a) { return sqrtf(norm_sq(a)); }
__device__ __forceinline__ V3 normalize(V3 a) { return a / norm(a); }
__device__ __forceinline__ float mixf(float a, float b, float l) { return (1.0f - l) * a + l * b; }
__device__ __forceinline__ V3 mixv(V3 a, V3 b, float l) {
  return V3((1.0f - l) * a.x + l * b.x, (1.0f - l) * a.y + l * b.y, (1.0f - l) * a.z + l * b.z);
}
__device__ __forceinline__ float sq(float f) { return f * f; }
__device__ __forceinline__ float pow5(float f) { float q = f * f; q = q * q; return f * q; }
__device__ __forceinline__ V3 ld3(const float* p) { return V3(p[0], p[1], p[2]); }
__device__ __forceinline__ bool has_nan(V3 a) { return a.x != a.x || a.y != a.y || a.z != a.z; }

// VMath.h:451-488
__device__ __forceinline__ V3 orthonormalized(V3 v1, V3 v2) { V3 r = v2 - dot(v2, v1) * v1; return r / norm(r); }
__device__ __forceinline__ V3 any_orthonormal(V3 v1) {
  return fabsf(v1.x) < 0.7f ? orthonormalized(v1, V3(1.f, 0.f, 0.f)) : orthonormalized(v1, V3(0.f, 1.f, 0.f));
}
__device__ __forceinline__ V3 orthonormalized_or_any(V3 v1, V3 v2) {
  V3 r = v2 - dot(v2, v1) * v1;
  float len = norm(r);
  return len < 1e-7f ? any_orthonormal(v1) : r / len;
}

// Rodrigues rotation taking `from` to `to`, VMath.h:558-607.
struct Rot {
  float a; V3 b, c, d;
  __device__ Rot(V3 from, V3 to) {
    float ca = dot(from, to);
    float op = 1.0f + ca;
    if (fabsf(op) > FLT_EPSILON) { V3 k = cross(from, to); a = ca; b = k; c = k; d = k / op; }
    else { V3 k = any_orthonormal(from); a = -1.0f; b = V3(); c = k; d = k * 2.0f; }
  }
  __device__ V3 apply(V3 x) const { return x * a + cross(b, x) + c * dot(d, x); }
};

__device__ __forceinline__ V3 reflect_across(V3 out, V3 n) { V3 inc = -out; return inc - 2.0f * dot(n, inc) * n; }

__device__ __forceinline__ int floor_int32(double x) { int i = (int)x; return i - (i > x); }
__device__ __forceinline__ float fmod1p1(float f) { return f - float(floor_int32(f)); }
__device__ __forceinline__ float clampf(float v, float lo, float hi) { return v < lo ? lo : (v > hi ? hi : v); }

// ----------------------------------------------------------------- RNG --
__device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
  uint64_t z = x + 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__device__ __forceinline__ uint64_t path_key(uint64_t seed, uint32_t pixel, uint32_t pass) {
  return splitmix64(splitmix64(seed) ^ ((uint64_t(pass) << 32) | uint64_t(pixel)));
}
constexpr uint64_t kPcgMult = 6364136223846793005ull;

// PCG32 stream of one camera path; the increment is re-derived from the
// path key so that only the 64-bit state is stored between kernels.
struct Rng {
  uint64_t state, inc;
  __device__ static uint64_t inc_of(uint64_t key) { return (splitmix64(key ^ 0xA5A5A5A5A5A5A5A5ull) << 1) | 1ull; }
  __device__ void seed(uint64_t key) {
    inc = inc_of(key);
    state = 0;
    state = state * kPcgMult + inc;
    state += splitmix64(key);
    state = state * kPcgMult + inc;
  }
  __device__ uint32_t next() {
    uint64_t old = state;
    state = old * kPcgMult + inc;
    uint32_t xs = uint32_t(((old >> 18) ^ old) >> 27);
    uint32_t rot = uint32_t(old >> 59);
    return (xs >> rot) | (xs << ((32u - rot) & 31u));
  }
  // RNG::uniform01f, core/include/Hasty/Random.h:131-137
  __device__ float u01() { return float(next() & 0x007FFFFFu) * 1.1920928955078125e-07f; }
};

// A stream that serves a given list of values in order (known-answer tests).
struct ReplayRng {
  const uint32_t* v; uint32_t n, pos;
  __device__ uint32_t next() { uint32_t x = v[pos % n]; ++pos; return x; }
  __device__ float u01() { return float(next() & 0x007FFFFFu) * 1.1920928955078125e-07f; }
};

// std::discrete_distribution draw as libstdc++ performs it: one
// generate_canonical<double,53> (two 32-bit draws, low word first; the sum
// u1 + u2*2^32 rounded once to double, then scaled by 2^-64, which is what
// converting the 64-bit integer and multiplying gives), then lower_bound in
// the cumulative table. `guide` (optional, K+1 entries, K a power of two)
// holds for bucket k the first index whose cumulative value is >= k/K, so the
// lower bound of u lies in [guide[k], guide[k+1]] with k = floor(u*K) exact.
template <class R> __device__ __forceinline__ uint32_t sample_cdf(const double* cdf, uint32_t n, R& r,
                                                                  const uint32_t* guide = nullptr, uint32_t log2k = 0) {
  if (n < 2 || cdf == nullptr) return 0u;
  uint64_t lo32 = r.next();
  uint64_t hi32 = r.next();
  double u = __ull2double_rn((hi32 << 32) | lo32) * 5.421010862427522170037264004349708557e-20;   // 2^-64
  if (u >= 1.0) u = 0.99999999999999988898;   // nextafter(1, 0)
  uint32_t lo = 0, hi = n;
  if (guide) {
    uint32_t k = uint32_t(u * double(1u << log2k));
    lo = guide[k];
    hi = guide[k + 1] + 1u;
    hi = hi < n ? hi : n;
  }
  while (lo < hi) { uint32_t mid = (lo + hi) >> 1; if (cdf[mid] < u) lo = mid + 1; else hi = mid; }
  return lo < n ? lo : n - 1;
}

// Halton value k of base b (core/include/Hasty/Random.h:14-63).
__device__ __forceinline__ float halton(uint32_t base, uint32_t k) {
  uint32_t i = k + 1, n = 0, d = 1;
  while (i) { n = n * base + i % base; i /= base; d *= base; }
  return float(n) / float(d);
}

// Upper bound on rejection-loop trials; the reference loops unbounded. Hitting
// it is counted (stats) and the last trial is used.
constexpr int kMaxTrials = 64;

// ------------------------------------------------------------ sampling --
// Sample.cpp:5-11
template <class R> __device__ __forceinline__ void disk_uniform(R& r, float& px, float& py) {
  float alpha = r.u01() * HTWOPI_F;
  float rad = sqrtf(r.u01());
  px = rad * cosf(alpha); py = rad * sinf(alpha);
}
// Sample.cpp:12-42 (aperture-blade polygon by rejection)
template <class R> __device__ __forceinline__ void ngon_uniform(R& r, const CameraDev& cam, float& sx, float& sy, int& capped) {
  float d = -cam.ngon_nx;
  for (int t = 0; t < kMaxTrials; ++t) {
    disk_uniform(r, sx, sy);
    float rad = sqrtf(sx * sx + sy * sy);
    float ang = atan2f(sy, sx);
    ang -= cam.blade_rot;
    ang += HTWOPI_F * (1.0f + FLT_EPSILON);
    ang = fmodf(ang, cam.ngon_per);
    float qx = rad * cosf(ang), qy = rad * sinf(ang);
    if (!((cam.ngon_nx * qx + cam.ngon_ny * qy + d) > 0.0f)) return;
  }
  capped = 1;
}
// Sample.cpp:77-108
template <class R> __device__ __forceinline__ V3 hemisphere_cos(R& r, V3 n, float& pdf, int& capped) {
  V3 dir; float c = 0.f;
  Rot rot(V3(0.f, 0.f, 1.f), n);
  for (int t = 0; t < kMaxTrials; ++t) {
    float xi1 = r.u01();
    float xi2 = r.u01();
    float phi = 2.0f * HPI_F * xi2;
    c = sqrtf(xi1);
    float s = sqrtf(1.0f - xi1);
    V3 rv(s * cosf(phi), s * sinf(phi), c);
    dir = normalize(rot.apply(rv));
    c = dot(dir, n);
    if (!(c <= 0.0f)) break;
    if (t == kMaxTrials - 1) capped = 1;
  }
  pdf = HINVPI_F * c;
  return dir;
}
__device__ __forceinline__ float hemisphere_cos_pdf(V3 n, V3 d) { float c = dot(n, d); return c < 0.0f ? 0.0f : HINVPI_F * c; }
// Sample.cpp:160-180
template <class R> __device__ __forceinline__ V3 triangle_uniform(R& r) {
  float s = r.u01();
  float t = sqrtf(r.u01());
  float b1 = 1.0f - t, b3 = t * s;
  float b2 = fmaxf(0.0f, 1.0f - b1 - b3);
  return V3(b1, b2, b3);
}

// ---------------------------------------------------------------- BSDF --
// BRDF.cpp:31-49
__device__ __forceinline__ bool refraction_cos_t(float ci, float ei, float et, float& ct) {
  float rel = ei / et;
  float si2 = fmaxf(0.f, 1.f - ci * ci);
  float st2 = (rel * rel) * si2;
  if (st2 >= 1.0f) return false;
  ct = sqrtf(1.0f - st2);
  return true;
}
// BRDF.cpp:74-81
__device__ __forceinline__ float fresnel_dielectric(float ci, float ct, float ei, float et) {
  float rp = (et * ci - ei * ct) / (et * ci + ei * ct);
  float ro = (ei * ci - et * ct) / (ei * ci + et * ct);
  return 0.5f * (rp * rp + ro * ro);
}
// BRDF.cpp:149-159
__device__ __forceinline__ float dggx(float nh, float th, float bh, float at, float ab) {
  return HINVPI_F / (at * ab * sq(sq(th / at) + sq(bh / ab) + sq(nh)));
}
__device__ __forceinline__ float smith_ggx(float nv, float tv, float bv, float at, float ab) {
  float lambda = 0.5f * (sqrtf(1.0f + (sq(at * tv) + sq(ab * bv)) / sq(nv)) - 1.0f);
  return 1.0f / (1.0f + lambda);
}
// Heitz visible-normal sampling, BRDF.cpp:163-185
__device__ __forceinline__ V3 ggx_vndf(V3 wo, float ax, float ay, float xi1, float xi2) {
  V3 vh = normalize(V3(ax * wo.x, ay * wo.y, wo.z));
  V3 t1 = cross(vh, V3(0.f, 0.f, 1.f));
  t1 = norm_sq(t1) < 1e-12f ? V3(1.f, 0.f, 0.f) : normalize(t1);
  V3 t2 = cross(t1, vh);
  float rr = sqrtf(xi1);
  float a = 1.0f / (1.0f + vh.z);
  float phi = HPI_F * ((xi2 < a) ? (xi2 / a) : (1.0f + (xi2 - a) / (1.0f - a)));
  float p1 = rr * cosf(phi);
  float p2 = rr * sinf(phi) * (xi2 < a ? 1.0f : vh.z);
  float p3 = sqrtf(fmaxf(0.0f, 1.0f - p1 * p1 - p2 * p2));
  V3 nh = p1 * t1 + p2 * t2 + p3 * vh;
  return normalize(V3(ax * nh.x, ay * nh.y, fmaxf(0.0f, nh.z)));
}
// BRDF.cpp:186-213; two uniforms per trial, the second-listed argument drawn
// first (the reference's compiler evaluates arguments right to left).
template <class R> __device__ __forceinline__ V3 ggx_vndf_global(R& r, V3 n, float at, float ab, V3 t, V3 b, V3 d1, float& pdf, int& capped) {
  if (dot(d1, n) <= 0.0f) { pdf = 0.0f; return -n; }
  V3 ng;
  V3 ve(dot(t, d1), dot(b, d1), dot(n, d1));
  for (int k = 0; k < kMaxTrials; ++k) {
    float xi2 = r.u01();
    float xi1 = r.u01();
    V3 ne = ggx_vndf(ve, at, ab, xi1, xi2);
    ng = normalize(t * ne.x + b * ne.y + n * ne.z);
    if (!(dot(ng, d1) <= 0.0f)) break;
    if (k == kMaxTrials - 1) capped = 1;
  }
  V3 d2 = normalize(reflect_across(d1, ng));
  float g1 = smith_ggx(dot(n, d1), dot(t, d1), dot(b, d1), at, ab);
  float d = dggx(dot(n, ng), dot(t, ng), dot(b, ng), at, ab);
  float ph = g1 * dot(d1, ng) * d / dot(d1, n);
  pdf = ph / (1e-7f + 4.0f * fabsf(dot(d1, ng)));
  return d2;
}
// BRDF.cpp:214-226
__device__ __forceinline__ float ggx_vndf_density(V3 n, float at, float ab, V3 t, V3 b, V3 d1, V3 d2) {
  if (dot(d1, n) <= 0.0f) return 0.0f;
  V3 ng = normalize(d1 + d2);
  float g1 = smith_ggx(dot(n, d1), dot(t, d1), dot(b, d1), at, ab);
  float d = dggx(dot(n, ng), dot(t, ng), dot(b, ng), at, ab);
  float ph = g1 * fmaxf(0.0f, dot(d1, ng)) * d / dot(d1, n);
  return ph / (1e-7f + 4.0f * fabsf(dot(d1, ng)));
}
__device__ __forceinline__ float normal_scale(V3 wi, V3 ns, V3 ng) { return fabsf(dot(wi, ns)) / (1e-7f + fabsf(dot(wi, ng))); }
// BRDF.cpp:253-263
__device__ __forceinline__ float compute_alpha(float r) { float a = r * r; return (a < 1e-2f && a != 0.0f) ? 1e-2f : a; }

struct Prob { bool none, refr; float pD, pS, pR, FD, cosT; };
// ShaderEvalFlag (BRDF.h): the lobes a sample covers.
enum : int { kLobeDiffuse = 1, kLobeConcentrated = 2, kLobeAll = 3 };
// BRDF.cpp:264-307
__device__ __forceinline__ Prob compute_probability(float m, float s, float t, float cos_o, float eo, float er,
                                                    int lobes = kLobeAll) {
  Prob p; p.cosT = 0.0f;
  p.refr = refraction_cos_t(cos_o, eo, er, p.cosT);
  p.FD = p.refr ? fresnel_dielectric(cos_o, p.cosT, eo, er) : 1.0f;
  float mD = (1.0f - t) * (1.0f - m) * (1.0f - 0.5f * s);
  float mS = mixf(mixf(0.5f * s, p.FD, t), 1.0f, m);
  // t = +0 with FD <= 1 and m <= 1: the double product is a non-negative
  // value times +0 times a non-negative value, i.e. +0, so the FP64 pipe
  // (a small fraction of the FP32 rate on this GPU) is skipped for it
  float mR = (__float_as_uint(t) == 0u && p.FD <= 1.0f && m <= 1.0f)
                 ? 0.0f
                 : float((1.0 - double(p.FD)) * double(t) * (1.0 - double(m)));
  if (!(lobes & kLobeDiffuse)) mD = 0.0f;
  if (!(lobes & kLobeConcentrated)) { mS = 0.0f; mR = 0.0f; }
  float sum = mD + mS + mR;
  p.none = sum == 0.0f;
  if (p.none) { p.pD = p.pS = p.pR = 0.0f; }
  else { p.pD = mD / sum; p.pS = mS / sum; p.pR = mR / sum; }
  return p;
}

// Surface point of a hit (Scene.cpp:202-255, SurfaceInteraction Scene.h:20-33).
struct Inter {
  V3 x, ng, ns, tan, bit;
  float h, u, v;
  int tri, mat;
  uint32_t geom;
  bool has_uv;
};

// BRDF.cpp:308-316
__device__ __forceinline__ void anisotropy_params(const Inter& it, V3 ns, float alpha, float aniso, float& at, float& ab, V3& t, V3& b) {
  float aspect = sqrtf(1.0f - 0.9f * aniso);
  at = alpha / aspect; ab = alpha * aspect;
  Rot rot(it.ng, ns);
  t = rot.apply(it.tan); b = rot.apply(it.bit);
}
// BRDF.cpp:319-326
__device__ __forceinline__ V3 eval_diffuse(float nswi, V3 albedo, float nscale, float m, float s, float t) {
  if (nswi < 0.0f) return V3();
  float k = HINVPI_F * nscale * (1.0f - 0.5f * s);
  if (t == 0.0f && m == 0.0f) return albedo * k;   // the double product is k exactly (1 - (+/-0) = 1)
  double kd = double(k) * (1.0 - double(t)) * (1.0 - double(m));
  return albedo * float(kd);
}
// BRDF.cpp:328-394 (rough dielectrics are refused at load time)
__device__ __forceinline__ V3 eval_concentrated(float nswi, V3 albedo, float m, float s, float t, V3 wo, V3 wi, float alpha,
                                                float at, float ab, V3 tan, V3 bit, V3 ns, float nscale, bool force, float FD) {
  if (nswi < 0.0f) return V3();
  V3 h = normalize(wo + wi);
  float lh = fabsf(dot(wi, h));
  float c5 = pow5(1.0f - lh);
  float nh = dot(ns, h);
  float nv = fabsf(dot(ns, wo));
  float nl = fabsf(dot(ns, wi));
  float G = smith_ggx(nv, dot(tan, wo), dot(bit, wo), at, ab) * smith_ggx(nl, dot(tan, wi), dot(bit, wi), at, ab);
  float D = (alpha == 0.0f) ? (force ? 4.0f * nl : 0.0f) : dggx(nh, dot(tan, h), dot(bit, h), at, ab);
  V3 spec_trans = (t > 0.0f && force) ? V3(FD, FD, FD) : V3();
  V3 spec_metal = albedo * (1.0f - c5) + V3(1.f, 1.f, 1.f) * c5;
  float sd = 0.5f * s;
  return mixv(mixv(V3(sd, sd, sd), spec_trans, t), spec_metal, m) * (D * G * nscale / fabsf(1e-7f + 4.0f * nv * nl));
}

// ------------------------------------------------------------ textures --
__device__ __forceinline__ void tex_lookup(const SceneDev& sc, int ti, float u0, float v0, float* out) {
  if (!HASTY_IN_BOUNDS(ti >= 0 && ti < sc.n_textures, BB_TEXTURE)) ti = 0;
  const TextureDev td = sc.textures[ti];
  float u = td.clamp_u ? clampf(u0, 0.0f, 1.0f - FLT_EPSILON) : fmod1p1(u0);
  float omv = td.clamp_v ? clampf(1.0f - v0, 0.0f, 1.0f - FLT_EPSILON) : fmod1p1(1.0f - v0);
  int col = int(u * float(td.w)), row = int(omv * float(td.h));
  col = col >= td.w ? td.w - 1 : (col < 0 ? 0 : col);
  row = row >= td.h ? td.h - 1 : (row < 0 ? 0 : row);
  const int64_t texel = int64_t(row) * td.w + col;
  if (td.fmt == 1) {
    const float* lut = sc.tex_pool + td.lut;
    if (td.ch == 1) {
      out[0] = lut[sc.tex_pool8[td.offset + texel]];
    } else {
      uint32_t w = *reinterpret_cast<const uint32_t*>(sc.tex_pool8 + td.offset + 4 * texel);
      out[0] = lut[w & 0xFFu]; out[1] = lut[(w >> 8) & 0xFFu]; out[2] = lut[(w >> 16) & 0xFFu];
    }
    return;
  }
  const float* p = sc.tex_pool + td.offset + texel * td.ch;
  for (int c = 0; c < td.ch; ++c) out[c] = p[c];
}
__device__ __forceinline__ V3 mat_albedo(const SceneDev& sc, const MaterialDev& m, const Inter& it) {
  if (m.albedo_tex < 0) return ld3(m.albedo);
  if (!it.has_uv) return V3(1.0f, 0.0f, 0.7f);     // Texture.h:98-101
  float c[3]; tex_lookup(sc, m.albedo_tex, it.u, it.v, c);
  return V3(c[0], c[1], c[2]);
}
__device__ __forceinline__ float mat_scalar(const SceneDev& sc, float val, int tex, const Inter& it) {
  if (tex < 0) return val;
  if (!it.has_uv) return -1.0f;
  float c; tex_lookup(sc, tex, it.u, it.v, &c);
  return c;
}
// BRDF.cpp:589-603
__device__ __forceinline__ float mat_ior(const MaterialDev& m, int wl) {
  if (!m.vary_ior) return m.ior;
  // precomputed on the host (MaterialDev::ior_band); selected with constant
  // indices so that a material copy can stay in registers
  if (wl == 0) return m.ior_band[0];
  if (wl == 1) return m.ior_band[1];
  if (wl == 2) return m.ior_band[2];
  return __int_as_float(0x7fc00000);
}
// BRDF.cpp:604-628
__device__ __forceinline__ V3 shading_normal(const SceneDev& sc, const MaterialDev& m, const Inter& it, V3 wo, float ngwo) {
  float side = ngwo < 0.0f ? -1.0f : 1.0f;
  V3 ns;
  if (m.normal_tex >= 0) {
    V3 col(1.0f, 0.0f, 0.7f);
    if (it.has_uv) { float c[3]; tex_lookup(sc, m.normal_tex, it.u, it.v, c); col = V3(c[0], c[1], c[2]); }
    V3 tn = 2.0f * col - V3(1.f, 1.f, 1.f);
    ns = normalize(it.tan * tn.x + it.bit * tn.y + it.ng * tn.z);
  } else {
    ns = it.ns;
  }
  float side_s = dot(ns, wo) < 0.0f ? -1.0f : 1.0f;
  if (side != side_s) ns = it.ng;
  return ns * side;
}

// Per-vertex shading frame shared by evaluate / pdf / sample: the shading
// normal for wo (getShadingNormal), texture lookups, alpha and the rotated
// anisotropic frame (computeAnisotropyParameters). Each quantity is computed
// exactly as the reference computes it inside each of those calls.
struct ShadeCtx { V3 ns, alb, tan, bit; float rough, met, alpha, at, ab, ngwo, nswo; };
HFN_CTX ShadeCtx shade_ctx(const SceneDev& sc, const MaterialDev& m, const Inter& it, V3 wo) {
  ShadeCtx c;
  c.ngwo = dot(it.ng, wo);
  c.ns = shading_normal(sc, m, it, wo, c.ngwo);
  c.nswo = dot(c.ns, wo);
  c.alb = mat_albedo(sc, m, it);
  c.rough = mat_scalar(sc, m.roughness, m.roughness_tex, it);
  c.met = mat_scalar(sc, m.metallic, m.metallic_tex, it);
  c.alpha = compute_alpha(c.rough);
  anisotropy_params(it, c.ns, c.alpha, m.anisotropy, c.at, c.ab, c.tan, c.bit);
  return c;
}

struct BsdfEval { V3 fD, fC; };
// PrincipledBRDF::evaluate, BRDF.cpp:630-679
HFN_EVAL BsdfEval bsdf_eval(const ShadeCtx& c, const MaterialDev& m, const Inter& it, V3 wo, V3 wi) {
  float nswi = dot(c.ns, wi);
  float nsc = normal_scale(wi, c.ns, it.ng);
  BsdfEval e;
  e.fD = eval_diffuse(nswi, c.alb, nsc, c.met, m.specular, m.transmission);
  e.fC = eval_concentrated(nswi, c.alb, c.met, m.specular, m.transmission, wo, wi, c.alpha, c.at, c.ab, c.tan, c.bit, c.ns,
                           nsc, false, 0.0f);
  return e;
}

// PrincipledBRDF::evaluateSamplePDF, BRDF.cpp:702-742 (nominal IOR)
HFN_EVAL float bsdf_pdf(const ShadeCtx& c, const MaterialDev& m, V3 wo, V3 wi, float eta_out) {
  bool from_out = c.ngwo >= 0.0f;
  float eo = from_out ? eta_out : m.ior, et = from_out ? m.ior : eta_out;
  Prob p = compute_probability(c.met, m.specular, m.transmission, c.nswo, eo, et);
  if (c.alpha == 0.0f) return p.pD * hemisphere_cos_pdf(c.ns, wi);
  float ps = ggx_vndf_density(c.ns, c.at, c.ab, c.tan, c.bit, wo, wi);
  float pd = hemisphere_cos_pdf(c.ns, wi);
  return p.pS * ps + p.pD * pd;
}

struct BsdfSample { bool outside; V3 dir, thrD, thrC; float pdf; };
// PrincipledBRDF::sample (member + static), BRDF.cpp:397-579, 681-700;
// `lobes` restricts the strategies (ShaderEvalFlag), `adjoint` drops the
// (eta_o / eta_t)^2 radiance scaling of refraction (importance transport).
template <class R>
HFN_SAMPLE BsdfSample bsdf_sample(const ShadeCtx& c, const MaterialDev& m, const Inter& it, V3 wo, int wl, float eta_out,
                                  R& r, int& capped, int lobes = kLobeAll, bool adjoint = false) {
  BsdfSample res;
  const V3 ns = c.ns, alb = c.alb, tan = c.tan, bit = c.bit;
  const float met = c.met, alpha = c.alpha, at = c.at, ab = c.ab, nswo = c.nswo;
  float eta_mat = mat_ior(m, wl);
  float s = m.specular, t = m.transmission;
  res.outside = c.ngwo >= 0.0f;
  float eo = res.outside ? eta_out : eta_mat;
  float er = res.outside ? eta_mat : eta_out;
  Prob p = compute_probability(met, s, t, nswo, eo, er, lobes);
  if (p.none) { res.dir = V3(1.f, 0.f, 0.f); res.pdf = 0.0f; return res; }
  V3 fD, fC;
  float xi = r.u01();
  int strat = xi < p.pR ? 3 : (xi < (p.pR + p.pS) ? 2 : 1);
  if (strat == 2) {
    if (alpha == 0.0f) {
      res.dir = reflect_across(wo, ns);
      res.pdf = 1e12f;
      float nswi = dot(ns, res.dir);
      float nsc = normal_scale(res.dir, ns, it.ng);
      fC = (1e12f / p.pS) * eval_concentrated(nswi, alb, met, s, t, wo, res.dir, alpha, at, ab, tan, bit, ns, nsc, true, p.FD);
    } else {
      float pdf_spec;
      res.dir = ggx_vndf_global(r, ns, at, ab, tan, bit, wo, pdf_spec, capped);
      float pdf_diff = hemisphere_cos_pdf(ns, res.dir);
      res.pdf = p.pS * pdf_spec + p.pD * pdf_diff;
      float nswi = dot(ns, res.dir);
      float nsc = normal_scale(res.dir, ns, it.ng);
      fD = eval_diffuse(nswi, alb, nsc, met, s, t);
      fC = eval_concentrated(nswi, alb, met, s, t, wo, res.dir, alpha, at, ab, tan, bit, ns, nsc, false, p.FD);
    }
  } else if (strat == 1) {
    float pdf_diff;
    res.dir = hemisphere_cos(r, ns, pdf_diff, capped);
    float nswi = dot(ns, res.dir);
    float nsc = normal_scale(res.dir, ns, it.ng);
    if (alpha == 0.0f) {
      res.pdf = p.pD * pdf_diff;
      fD = eval_diffuse(nswi, alb, nsc, met, s, t);
    } else {
      float pdf_spec = ggx_vndf_density(ns, at, ab, tan, bit, wo, res.dir);
      res.pdf = p.pS * pdf_spec + (1.0f - p.pS) * pdf_diff;
      fD = eval_diffuse(nswi, alb, nsc, met, s, t);
      fC = eval_concentrated(nswi, alb, met, s, t, wo, res.dir, alpha, at, ab, tan, bit, ns, nsc, false, p.FD);
    }
  } else {
    res.outside = !res.outside;
    res.pdf = 1e12f;
    if (!p.refr) {
      res.dir = V3(1.f, 0.f, 0.f);
    } else {
      float ratio = eo / er;
      res.dir = normalize((-ratio) * wo + (ratio * nswo - p.cosT) * ns);
      float fc = res.pdf / p.pR * (adjoint ? 1.0f : sq(ratio)) * (1.0f - p.FD) / fabsf(dot(res.dir, it.ng));
      V3 mask = wl < 0 ? V3(1.f, 1.f, 1.f) : V3(wl == 0 ? 1.f : 0.f, wl == 1 ? 1.f : 0.f, wl == 2 ? 1.f : 0.f);
      fC = fc * mask;
    }
  }
  float mm = fabsf(dot(res.dir, it.ng)) / res.pdf;
  res.thrD = fD * mm;
  res.thrC = fC * mm;
  return res;
}

// ---------------------------------------------------------- interaction --
// Geometric normal of a triangle as the ray/triangle test produces it
// (unnormalised cross((v2-v0),(v0-v1)) = (v1-v0)x(v2-v0)).
__device__ __forceinline__ V3 tri_ng_raw(const float* p) {
  V3 e1(p[0] - p[3], p[1] - p[4], p[2] - p[5]);
  V3 e2(p[6] - p[0], p[7] - p[1], p[8] - p[2]);
  return cross(e2, e1);
}

// Scene::getInteraction, Scene.cpp:202-255
HFN_INTER Inter make_inter(const SceneDev& sc, int tri, V3 b, V3 ng) {
  Inter it;
  const TriAttr a = sc.tri_attr[tri];
  const float* p = sc.tri_pos + 9 * int64_t(tri);
  V3 x0 = ld3(p), x1 = ld3(p + 3), x2 = ld3(p + 6);
  it.tri = tri; it.geom = a.geom; it.mat = a.mat;
  if (!HASTY_IN_BOUNDS(a.mat >= 0 && a.mat < sc.n_mats, BB_MATERIAL)) it.mat = 0;
  it.x = b.x * x0 + b.y * x1 + b.z * x2;
  it.ng = ng;
  it.h = 0.0f;
  if (a.smooth) {
    V3 nv0, nv1, nv2;
    if (a.ni[0] >= 0 && a.ni[1] >= 0 && a.ni[2] >= 0) {
      nv0 = ld3(sc.normals + 3 * int64_t(a.ni[0])); nv1 = ld3(sc.normals + 3 * int64_t(a.ni[1])); nv2 = ld3(sc.normals + 3 * int64_t(a.ni[2]));
    } else {
      nv0 = nv1 = nv2 = normalize(cross(x1 - x0, x2 - x0));
    }
    it.ns = normalize(b.x * nv0 + b.y * nv1 + b.z * nv2);
    V3 xv[3] = {x0, x1, x2}, nv[3] = {nv0, nv1, nv2};
    for (int k = 0; k < 3; ++k) {
      float nvng = dot(it.ng, nv[k]);
      float hi = nvng == 0.0f ? 1e6f : (dot(xv[k], nv[k]) - dot(it.x, nv[k])) / nvng;
      it.h += b[k] * b[k] * hi;
    }
  } else {
    it.ns = it.ng;
  }
  it.has_uv = false; it.u = 0.f; it.v = 0.f;
  bool ok = true;
  float uv[3][2];
  for (int k = 0; k < 3; ++k) {
    int64_t ti = a.ti[k];
    if (ti < 0 || 2 * ti + 1 >= sc.n_texcoords) { ok = false; break; }
    uv[k][0] = sc.texcoords[2 * ti]; uv[k][1] = sc.texcoords[2 * ti + 1];
  }
  if (ok) {
    it.has_uv = true;
    it.u = uv[0][0] * b.x + uv[1][0] * b.y + uv[2][0] * b.z;
    it.v = uv[0][1] * b.x + uv[1][1] * b.y + uv[2][1] * b.z;
  }
  it.tan = orthonormalized_or_any(it.ng, V3(-it.x.z, 0.0f, it.x.x));
  it.bit = cross(it.ng, it.tan);
  return it;
}

// Hit record (t, u, v, triangle) -> interaction (Scene.cpp:294-302).
__device__ __forceinline__ Inter inter_from_hit(const SceneDev& sc, int tri, float u, float v) {
  if (!HASTY_IN_BOUNDS(tri >= 0 && tri < sc.n_tris, BB_TRI)) tri = 0;
  V3 b(1.0f - u - v, u, v);
  V3 ng = normalize(tri_ng_raw(sc.tri_pos + 9 * int64_t(tri)));
  return make_inter(sc, tri, b, ng);
}

// Only the position of a hit (what the light-pdf needs).
__device__ __forceinline__ V3 hit_point(const SceneDev& sc, int tri, float u, float v) {
  if (!HASTY_IN_BOUNDS(tri >= 0 && tri < sc.n_tris, BB_TRI)) tri = 0;
  const float* p = sc.tri_pos + 9 * int64_t(tri);
  V3 b(1.0f - u - v, u, v);
  return b.x * ld3(p) + b.y * ld3(p + 3) + b.z * ld3(p + 6);
}

// Scene::constructRayX, Scene.cpp:257-270
__device__ __forceinline__ V3 ray_x(const Inter& it, bool outside) {
  float eps = 1e-5f;
  float hmin = fmaxf(eps, norm(it.x) * eps);
  return it.x + it.ng * (1.01f * (outside ? fmaxf(0.0f, it.h) + hmin : fminf(0.0f, it.h) - hmin));
}

// --------------------------------------------------------- environment --
__device__ __forceinline__ void sph_from_dir(V3 d, float& th, float& ph) {
  th = acosf(d.y);
  ph = atan2f(d.z, d.x);
  ph = ph < 0.0f ? ph + HTWOPI_F : ph;
}
// EnvironmentTexture::evalEmission / BackgroundColor, Environment.h:26-29,135-140
HFN_ENV V3 env_eval(const SceneDev& sc, V3 d) {
  const EnvDev& e = sc.env;
  if (!e.is_texture) return ld3(e.color);
  float th, ph; sph_from_dir(d, th, ph);
  float u = ph * float(0.5 * kInvPi);
  float v = 1.0f - th * HINVPI_F;
  float uu = fmod1p1(u);
  float omv = clampf(1.0f - v, 0.0f, 1.0f - FLT_EPSILON);
  int col = int(uu * float(e.w)), row = int(omv * float(e.h));
  col = col >= e.w ? e.w - 1 : col; row = row >= e.h ? e.h - 1 : row;
  return ld3(e.texels + 3 * (int64_t(row) * e.w + col));
}
// EnvironmentTexture::evalSamplingDensity, Environment.h:159-166
HFN_ENV float env_density(const SceneDev& sc, V3 d) {
  const EnvDev& e = sc.env;
  float th, ph; sph_from_dir(d, th, ph);
  float u = ph * float(0.5 * kInvPi);
  float v = 1.0f - th * HINVPI_F;
  float s = sinf(th);
  uint32_t x = uint32_t(u * float(e.w)), y = uint32_t((1.0f - v) * float(e.h));
  x = x < uint32_t(e.w - 1) ? x : uint32_t(e.w - 1);
  y = y < uint32_t(e.h - 1) ? y : uint32_t(e.h - 1);
  float dens = float(e.w) * float(e.h) * e.weights[int64_t(y) * e.w + x] / e.value_sum;
  return dens / fmaxf(1e-7f, 2.0f * float(kPi * kPi) * s);
}
// EnvironmentTexture::sample + ImageDistribution::sample, Environment.h:60-79,142-153
template <class R> HFN_ENV V3 env_sample(const SceneDev& sc, R& r, float& density, int& capped) {
  const EnvDev& e = sc.env;
  uint32_t n = uint32_t(e.w) * uint32_t(e.h);
  V3 dir; float sin_t = 0.f;
  for (int k = 0; k < kMaxTrials; ++k) {
    uint32_t idx = sample_cdf(e.cdf, n, r, e.guide, e.guide_log2);
    uint32_t W = uint32_t(e.w), H = uint32_t(e.h);
    uint32_t x = idx % W, y = idx / W;
    float hf = float(H), wf = float(W);
    float xi0 = r.u01();
    float xi1 = r.u01();
    float left = float(x) / wf, right = (float(x) + 1.0f) / wf;
    float lower = (float(H) - (float(y) + 1.0f)) / hf, upper = float(H - y) / hf;
    float u = (1.0f - xi0) * left + xi0 * right;
    float v = (1.0f - xi1) * lower + xi1 * upper;
    float pxy = e.weights[int64_t(y) * W + x] / e.value_sum;
    density = wf * hf * pxy;
    float phi = u * 2.0f * HPI_F;
    float theta = (1.0f - v) * HPI_F;
    sin_t = sinf(theta);
    float ct = cosf(theta), sp = sinf(phi), cp = cosf(phi);
    dir = V3(sin_t * cp, ct, sin_t * sp);
    if (sin_t != 0.0f) break;
    if (k == kMaxTrials - 1) capped = 1;
  }
  density /= (2.0f * HPI_F * HPI_F * sin_t);
  return dir;
}

// Scene::evalLightRayFromStartPointDensity, Scene.cpp:587-616. `tri` < 0 is
// a miss; `x2`/`ng2` are the hit's position and unit geometric normal.
HFN_ENV float light_density(const SceneDev& sc, V3 o, V3 d, int tri, V3 x2, V3 ng2) {
  bool surf = tri >= 0 && sc.mats[sc.tri_attr[tri].mat].is_light;
  bool inf = tri < 0;
  if (!surf && !inf) return 0.0f;
  float ps = sc.p_surface;
  if (surf) {
    float dsq = fmaxf(1e-5f, norm_sq(o - x2));
    float pw = sc.light_pdf_area * dsq / (1e-7f + fabsf(dot(ng2, d)));
    float res = ps * pw;
    if (sc.env_is_sampled) res += (1.0f - ps) * env_density(sc, d);
    return res;
  }
  return sc.env_is_sampled ? (1.0f - ps) * env_density(sc, d) : 0.0f;
}

// Scene::getEmissionRadiance, Scene.cpp:471-477
__device__ __forceinline__ V3 emission(const SceneDev& sc, int mat, V3 ng, V3 wo) {
  if (dot(ng, wo) <= 0.0f) return V3();
  return ld3(sc.mats[mat].emission) * HINVPI_F;
}

// beersLaw, core/include/Hasty/PathTracing.h:46-59
__device__ __forceinline__ V3 beers(V3 T, float d) {
  if (T.x == 1.0f && T.y == 1.0f && T.z == 1.0f) return V3(1.f, 1.f, 1.f);
  return V3(T.x <= 0.0f ? 0.0f : powf(T.x, 1.0f * d), T.y <= 0.0f ? 0.0f : powf(T.y, 1.0f * d), T.z <= 0.0f ? 0.0f : powf(T.z, 1.0f * d));
}

// Camera::computeRay, Camera.cpp:41-81
template <class R> __device__ __forceinline__ void camera_ray(const CameraDev& c, R& r, float x, float y, float W, float H, V3& o, V3& d, int& capped) {
  float lx = (x - 0.5f * W) / W * 2.0f;
  float ly = (y - 0.5f * H) / W * 2.0f;
  V3 fwd = ld3(c.fwd), right = ld3(c.right), up = ld3(c.up), pos = ld3(c.pos);
  V3 dir = normalize(fwd + right * (c.q * lx) - up * (c.q * ly));
  if (c.aperture > 0.0f) {
    float sx, sy;
    ngon_uniform(r, c, sx, sy, capped);
    float t = c.focal * dot(dir, fwd);
    V3 fp = pos + t * dir;
    V3 org = pos + (c.aperture * sx) * up + (c.aperture * sy) * right;
    o = org; d = normalize(fp - org);
  } else {
    o = pos; d = dir;
  }
}

}  // namespace dev
}  // namespace hasty
