// Closest-hit traversal of the compressed 8-wide BVH and the binary BVH
// (per-ray step machines, exact ray/triangle test), host + device. Shared by
// the closest-hit kernels (trace.cu) and the photon mapper (photon.cu); every
// including translation unit gets its own copy (anonymous namespace). All
// rounding is explicit (mulr/addr/subr/divr, fmaf), so the results do not
// depend on the compiler's FMA contraction setting.
//
// The ray/triangle test is Moeller-Trumbore in Embree's sign conventions and
// rounds every product and sum separately (no FMA contraction), so t, u, v
// and the chosen triangle are the ones the CPU oracle computes. The far
// limit is applied to the divided distance and ties at equal t go to the
// smaller triangle id, so the answer does not depend on traversal order.
// Binary-BVH box tests round each step once and are padded by
// 1 +/- 2*gamma(3), so no box that holds the closest hit is culled by
// rounding (Ize 2013); the wide BVH's one-FMA child planes carry an absolute
// error bound instead (plane_terms). The far limit at the current closest
// hit is padded by 1 + 2*gamma(3) in both.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstring>

#include "bounds.cuh"

namespace hasty {
namespace {

#define HDI __host__ __device__ __forceinline__

constexpr unsigned kFullMask = 0xFFFFFFFFu;

struct Hit { float t, u, v; int tri; };

HDI float mulr(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fmul_rn(a, b);
#else
  return a * b;        // host objects are built with -ffp-contract=off
#endif
}
HDI float addr(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fadd_rn(a, b);
#else
  return a + b;
#endif
}
HDI float subr(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fsub_rn(a, b);
#else
  return a - b;
#endif
}
HDI float divr(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fdiv_rn(a, b);
#else
  return a / b;
#endif
}
HDI uint32_t f2u(float f) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(f);
#else
  uint32_t u; std::memcpy(&u, &f, 4); return u;
#endif
}
HDI float u2f(uint32_t u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float f; std::memcpy(&f, &u, 4); return f;
#endif
}
HDI uint32_t popc(uint32_t x) {
#ifdef __CUDA_ARCH__
  return __popc(x);
#else
  return uint32_t(__builtin_popcount(x));
#endif
}
HDI uint32_t highest_bit(uint32_t x) {   // x != 0
#ifdef __CUDA_ARCH__
  return 31u - __clz(x);
#else
  return 31u - uint32_t(__builtin_clz(x));
#endif
}
HDI uint32_t lowest_bit(uint32_t x) {    // x != 0
#ifdef __CUDA_ARCH__
  return uint32_t(__ffs(x)) - 1u;
#else
  return uint32_t(__builtin_ctz(x));
#endif
}
HDI float4 ld(const float4* p) {
#ifdef __CUDA_ARCH__
  return __ldg(p);
#else
  return *p;
#endif
}
HDI float dotr(float ax, float ay, float az, float bx, float by, float bz) {
  return addr(addr(mulr(ax, bx), mulr(ay, by)), mulr(az, bz));
}

HDI void tri_test(float ox, float oy, float oz, float dx, float dy, float dz, float4 v0, float4 e1, float4 e2, Hit& best) {
  float nx = subr(mulr(e2.y, e1.z), mulr(e2.z, e1.y));
  float ny = subr(mulr(e2.z, e1.x), mulr(e2.x, e1.z));
  float nz = subr(mulr(e2.x, e1.y), mulr(e2.y, e1.x));
  float cx = subr(v0.x, ox), cy = subr(v0.y, oy), cz = subr(v0.z, oz);
  float rx = subr(mulr(cy, dz), mulr(cz, dy));
  float ry = subr(mulr(cz, dx), mulr(cx, dz));
  float rz = subr(mulr(cx, dy), mulr(cy, dx));
  float den = dotr(nx, ny, nz, dx, dy, dz);
  float ad = fabsf(den);
  float sg = den < 0.f ? -1.f : 1.f;
  float U = mulr(dotr(rx, ry, rz, e2.x, e2.y, e2.z), sg);
  float V = mulr(dotr(rx, ry, rz, e1.x, e1.y, e1.z), sg);
  if (!(den != 0.f && U >= 0.f && V >= 0.f && addr(U, V) <= ad)) return;
  float T = mulr(dotr(nx, ny, nz, cx, cy, cz), sg);
  if (!(mulr(ad, 1e-6f) < T)) return;
  float t = divr(T, ad);
  int id = int(f2u(v0.w));
  if (t < best.t || (t == best.t && (best.tri < 0 || id < best.tri))) {
    best.t = t; best.u = divr(U, ad); best.v = divr(V, ad); best.tri = id;
  }
}

HDI float slab(float b, float o, float id) { return mulr(subr(b, o), id); }

constexpr float kPadHi = 1.0000008f;   // 1 + 2*gamma(3), rounded up
constexpr float kPadLo = 0.9999992f;
constexpr float kInf = __builtin_huge_valf();

struct RayInv { float ix, iy, iz; };
HDI RayInv inverse_dir(float dx, float dy, float dz) {
  const float eps = 1e-20f;
  RayInv r;
  r.ix = 1.0f / (fabsf(dx) > eps ? dx : copysignf(eps, dx));
  r.iy = 1.0f / (fabsf(dy) > eps ? dy : copysignf(eps, dy));
  r.iz = 1.0f / (fabsf(dz) > eps ? dz : copysignf(eps, dz));
  return r;
}

// ---------------------------------------------------------- binary BVH ----
constexpr int kStack = 64;

// Traversal state of one ray. init() sets it up; each step() walks inner
// nodes to the next leaf, tests the leaf's triangles and pops the next
// subtree; it returns true once the ray is finished (result in `best`).
// Whole-ray traversal is init() + step() until true; the persistent GPU
// kernels interleave steps of many rays, with identical results per ray.
// The traversal stack is kept outside the struct (passed to step()) so the
// scalar state can stay in registers.
struct TravBinary {
  using Entry = int;
  static constexpr int kDepth = kStack;
  float ox, oy, oz, dx, dy, dz;
  RayInv iv;
  bool neg_x, neg_y, neg_z;
  Hit best;
  int link, sp;
  bool any;   // stop at the first triangle hit (visibility only); set after init
  bool overflow;   // a subtree was skipped because the stack was full
#ifdef HASTY_DEBUG_BOUNDS
  int32_t lim_nodes = 0x7FFFFFFF, lim_tris = 0x7FFFFFFF;   // bounds-checked build: array sizes
#endif

  HDI void init(float ox_, float oy_, float oz_, float dx_, float dy_, float dz_) {
    ox = ox_; oy = oy_; oz = oz_; dx = dx_; dy = dy_; dz = dz_;
    any = false;
    overflow = false;
    best.t = kInf; best.u = best.v = 0.f; best.tri = -1;
    iv = inverse_dir(dx, dy, dz);
    neg_x = iv.ix < 0.f; neg_y = iv.iy < 0.f; neg_z = iv.iz < 0.f;
    sp = 0;
    link = 0;   // root (always an inner node)
  }

  HDI bool step(const float4* nodes, const float4* tris, int* stack) {
    while (link >= 0) {
#ifdef HASTY_DEBUG_BOUNDS
      if (!HASTY_IN_BOUNDS(link < lim_nodes, BB_NODE)) return true;
#endif
      float4 n0 = ld(&nodes[4 * link + 0]);
      float4 n1 = ld(&nodes[4 * link + 1]);
      float4 n2 = ld(&nodes[4 * link + 2]);
      float4 n3 = ld(&nodes[4 * link + 3]);
      float tlim = best.t * kPadHi;
      // near/far planes by the direction sign: (b - o) * id is monotonic in b,
      // so this picks exactly what per-axis min/max would
      float t0min = fmaxf(fmaxf(slab(neg_x ? n0.y : n0.x, ox, iv.ix), slab(neg_y ? n0.w : n0.z, oy, iv.iy)),
                          fmaxf(slab(neg_z ? n2.y : n2.x, oz, iv.iz), 0.0f)) * kPadLo;
      float t0max = fminf(fminf(fminf(slab(neg_x ? n0.x : n0.y, ox, iv.ix), slab(neg_y ? n0.z : n0.w, oy, iv.iy)),
                                slab(neg_z ? n2.x : n2.y, oz, iv.iz)) * kPadHi, tlim);
      float t1min = fmaxf(fmaxf(slab(neg_x ? n1.y : n1.x, ox, iv.ix), slab(neg_y ? n1.w : n1.z, oy, iv.iy)),
                          fmaxf(slab(neg_z ? n2.w : n2.z, oz, iv.iz), 0.0f)) * kPadLo;
      float t1max = fminf(fminf(fminf(slab(neg_x ? n1.x : n1.y, ox, iv.ix), slab(neg_y ? n1.z : n1.w, oy, iv.iy)),
                                slab(neg_z ? n2.z : n2.w, oz, iv.iz)) * kPadHi, tlim);
      bool h0 = t0min <= t0max, h1 = t1min <= t1max;
      int l0 = int(f2u(n3.x)), l1 = int(f2u(n3.y));
      if (h0 && h1) {
        int far_l = l1;
        link = l0;
        if (t1min < t0min) { link = l1; far_l = l0; }
        if (sp < kStack) stack[sp++] = far_l; else overflow = true;
      } else if (h0) {
        link = l0;
      } else if (h1) {
        link = l1;
      } else {
        if (sp == 0) return true;
        link = stack[--sp];
      }
    }
    // leaf: link = ~(first << 3 | count)
    int code = ~link;
    int first = code >> 3, cnt = code & 7;
    for (int k = 0; k < cnt; ++k) {
      int ti = first + k;
#ifdef HASTY_DEBUG_BOUNDS
      if (!HASTY_IN_BOUNDS(ti >= 0 && ti < lim_tris, BB_LEAF_TRI)) return true;
#endif
      tri_test(ox, oy, oz, dx, dy, dz, ld(&tris[3 * ti]), ld(&tris[3 * ti + 1]), ld(&tris[3 * ti + 2]), best);
    }
    if (sp == 0 || (any && best.tri >= 0)) return true;
    link = stack[--sp];
    return false;
  }
};

HDI Hit trace_binary(const float4* nodes, const float4* tris, float ox, float oy, float oz, float dx, float dy, float dz) {
  TravBinary tr;
  int stack[kStack];
  tr.init(ox, oy, oz, dx, dy, dz);
  while (!tr.step(nodes, tris, stack)) {}
  return tr.best;
}

// ------------------------------------------------- compressed 8-wide BVH ----
// Node groups of Ylitie, Karras and Laine 2017: (base index, mask) where bits
// 24..31 are children still to visit, each at bit 24 + (slot ^ octant) so the
// highest bit is the nearest child, and bits 0..7 hold the parent's
// inner-child mask; for triangle groups bits 0..23 are triangles to test.
// Child boxes are decoded as the builder verified them (fma of the 8-bit
// coordinate and the power-of-two step) and tested with the padded slabs.
constexpr int kWideStack = 32;

HDI uint32_t byte_of(uint32_t w, uint32_t k) { return (w >> (8 * k)) & 0xFFu; }

// 2^23 + byte k of w as a float, exactly: one byte permute places the byte
// in the mantissa of 2^23 (the offset is folded into the planes' b terms).
HDI float byte_biased(uint32_t w, uint32_t k) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(__byte_perm(w, 0x4B000000u, k | 0x7540u));
#else
  return 8388608.0f + float(byte_of(w, k));
#endif
}

// Same contract as TravBinary: a step tests the pending triangle group and
// opens one node.
// Per-node, per-axis terms of the child slab test t = fma(q, a, b). A child
// plane is x = fma(q, s, p0) rounded once (the float plane the layout writer
// makes conservative); the slab parameter is T = (x - o) / d. Here a = s * inv
// is exact (s is a power of two, inv = fl(1/d)) and b = (p0 - o) * inv, so
//   fma(q, a, b) = T (1 + th), |th| <= gamma(2),  plus  R,
//   |R| <= u |inv| (|p0| + 255 s + 2 |p0 - o|) (1 + 4u),  u = 2^-24,
// R coming from x's own rounding (which this form skips) and from b's two
// roundings; and |T| <= (|p0 - o| + 255 s) |inv| (1 + u). With the rounding
// of b -/+ eps, the total error is below u |inv| (|p0| + 765 s + 5 |p0 - o|)
// to first order; eps = 2^-22 |inv| (|p0| + 1024 s + 6 |p0 - o|) + 1e-37
// covers it at least twice over (the constant covers products in the
// subnormal range). Near planes use b - eps and far planes b + eps, so each
// near value is at most, and each far value at least, the exact T: the box
// test needs no further padding and culls no box the ray enters.
// (Coordinates and grid steps are assumed below 2^120, far beyond any scene.)
struct PlaneTerms { float a, b_near, b_far; };
HDI PlaneTerms plane_terms(float p0, float o, float inv, float s) {
  PlaneTerms t;
  const float d = subr(p0, o);
  const float b = mulr(d, inv);
  const float mag = fmaf(6.0f, fabsf(d), fmaf(1024.0f, s, fabsf(p0)));
  const float eps = fmaf(mulr(mag, fabsf(inv)), 2.384185791015625e-07f, 1e-37f);   // 2^-22
  t.a = mulr(s, inv);
  // The child loop evaluates fma(2^23 + q, a, b') with b' = b -/+ eps - 2^23 a
  // (2^23 a is exact; the FMA forms (2^23 + q) a exactly). The one extra
  // rounding, of b' itself, is at most u (2^23 |a| + |b| + eps) = s |inv| / 2
  // + u (|b| + eps): half a grid step, added to eps with a relative margin
  // of 1e-6; the u |b| part is inside eps's factor-two margin.
  const float half = mulr(mulr(0.5000005f, s), fabsf(inv));
  const float e = addr(eps, half);
  const float a23 = mulr(-8388608.0f, t.a);
  t.b_near = addr(subr(b, e), a23);
  t.b_far = addr(addr(b, e), a23);
  return t;
}

struct TravWide {
  using Entry = uint2;
  static constexpr int kDepth = kWideStack;
  float ox, oy, oz, dx, dy, dz;
  RayInv iv;
  bool neg_x, neg_y, neg_z;
  uint32_t oct, oct4;
  Hit best;
  uint2 ng, tg;
  int sp;
  // Visibility only: stop at the first triangle hit (best is then a hit,
  // not necessarily the closest). Set after init.
  bool any;
  bool overflow;   // a node group was skipped because the stack was full
#ifdef HASTY_DEBUG_BOUNDS
  int32_t lim_nodes = 0x7FFFFFFF, lim_tris = 0x7FFFFFFF;   // bounds-checked build: array sizes
#endif

  HDI void init(float ox_, float oy_, float oz_, float dx_, float dy_, float dz_) {
    ox = ox_; oy = oy_; oz = oz_; dx = dx_; dy = dy_; dz = dz_;
    any = false;
    overflow = false;
    best.t = kInf; best.u = best.v = 0.f; best.tri = -1;
    iv = inverse_dir(dx, dy, dz);
    neg_x = iv.ix < 0.f; neg_y = iv.iy < 0.f; neg_z = iv.iz < 0.f;
    oct = (neg_x ? 4u : 0u) | (neg_y ? 2u : 0u) | (neg_z ? 1u : 0u);
    oct4 = oct * 0x01010101u;
    sp = 0;
    ng = make_uint2(0u, 0x80000000u);
    tg = make_uint2(0u, 0u);
  }

  HDI bool step(const float4* nodes, const float4* tris, uint2* stack) {
    while (tg.y) {
      uint32_t b = lowest_bit(tg.y);
      tg.y &= tg.y - 1u;
      int ti = int(tg.x + b);
#ifdef HASTY_DEBUG_BOUNDS
      if (!HASTY_IN_BOUNDS(ti >= 0 && ti < lim_tris, BB_LEAF_TRI)) return true;
#endif
      tri_test(ox, oy, oz, dx, dy, dz, ld(&tris[3 * ti]), ld(&tris[3 * ti + 1]), ld(&tris[3 * ti + 2]), best);
    }
    if (any && best.tri >= 0) return true;
    if (ng.y <= 0x00FFFFFFu) {
      if (sp == 0) return true;
      ng = stack[--sp];
    }
    uint32_t bit = highest_bit(ng.y);
    uint32_t slot = (bit - 24u) ^ oct;
    uint32_t imask = ng.y & 0xFFu;
    uint32_t node = ng.x + popc(imask & ~(0xFFFFFFFFu << slot));
    ng.y &= ~(1u << bit);
    if (ng.y > 0x00FFFFFFu) {
      if (sp < kWideStack) stack[sp++] = ng; else overflow = true;
    }

#ifdef HASTY_DEBUG_BOUNDS
    if (!HASTY_IN_BOUNDS(node < uint32_t(lim_nodes), BB_NODE)) return true;
#endif
    float4 f0 = ld(&nodes[5 * node + 0]);
    float4 f1 = ld(&nodes[5 * node + 1]);
    float4 f2 = ld(&nodes[5 * node + 2]);
    float4 f3 = ld(&nodes[5 * node + 3]);
    float4 f4 = ld(&nodes[5 * node + 4]);
    uint32_t eword = f2u(f0.w);
    int ex = int(int8_t(eword & 0xFFu)), ey = int(int8_t((eword >> 8) & 0xFFu)), ez = int(int8_t((eword >> 16) & 0xFFu));
    uint32_t node_imask = eword >> 24;
    float sx = u2f(uint32_t(ex + 127) << 23), sy = u2f(uint32_t(ey + 127) << 23), sz = u2f(uint32_t(ez + 127) << 23);
    // Child plane t = q * A + B per axis (one FMA per plane), A = 2^e * inv
    // (exact), B = (p0 - o) * inv moved by eps to the conservative side.
    const PlaneTerms px = plane_terms(f0.x, ox, iv.ix, sx);
    const PlaneTerms py = plane_terms(f0.y, oy, iv.iy, sy);
    const PlaneTerms pz = plane_terms(f0.z, oz, iv.iz, sz);
    uint32_t child_base = f2u(f1.x), tri_base = f2u(f1.y);
    uint32_t meta_w[2] = {f2u(f1.z), f2u(f1.w)};
    // near and far planes per axis, chosen once by the ray's direction sign
    const uint32_t nx[2] = {neg_x ? f2u(f3.z) : f2u(f2.x), neg_x ? f2u(f3.w) : f2u(f2.y)};
    const uint32_t fx[2] = {neg_x ? f2u(f2.x) : f2u(f3.z), neg_x ? f2u(f2.y) : f2u(f3.w)};
    const uint32_t ny[2] = {neg_y ? f2u(f4.x) : f2u(f2.z), neg_y ? f2u(f4.y) : f2u(f2.w)};
    const uint32_t fy[2] = {neg_y ? f2u(f2.z) : f2u(f4.x), neg_y ? f2u(f2.w) : f2u(f4.y)};
    const uint32_t nz[2] = {neg_z ? f2u(f4.z) : f2u(f3.x), neg_z ? f2u(f4.w) : f2u(f3.y)};
    const uint32_t fz[2] = {neg_z ? f2u(f3.x) : f2u(f4.z), neg_z ? f2u(f3.y) : f2u(f4.w)};
    float tlim = best.t * kPadHi;
    uint32_t hitmask = 0;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      uint32_t meta4 = meta_w[h];
      uint32_t inner4 = (meta4 & (meta4 << 1)) & 0x10101010u;     // 24..31 marks an inner child
      uint32_t inner_mask4 = (inner4 >> 4) * 0xFFu;
      uint32_t bit_index4 = (meta4 ^ (oct4 & inner_mask4)) & 0x1F1F1F1Fu;
      uint32_t child_bits4 = (meta4 >> 5) & 0x07070707u;
#pragma unroll
      for (uint32_t k = 0; k < 4; ++k) {
        float tnx = fmaf(byte_biased(nx[h], k), px.a, px.b_near);
        float tfx = fmaf(byte_biased(fx[h], k), px.a, px.b_far);
        float tny = fmaf(byte_biased(ny[h], k), py.a, py.b_near);
        float tfy = fmaf(byte_biased(fy[h], k), py.a, py.b_far);
        float tnz = fmaf(byte_biased(nz[h], k), pz.a, pz.b_near);
        float tfz = fmaf(byte_biased(fz[h], k), pz.a, pz.b_far);
        float tmin = fmaxf(fmaxf(tnx, tny), fmaxf(tnz, 0.0f));
        float tmax = fminf(fminf(tfx, tfy), fminf(tfz, tlim));
        if (tmin <= tmax) hitmask |= byte_of(child_bits4, k) << byte_of(bit_index4, k);
      }
    }
    ng = make_uint2(child_base, (hitmask & 0xFF000000u) | node_imask);
    tg = make_uint2(tri_base, hitmask & 0x00FFFFFFu);
    return false;
  }
};

// Array sizes for the bounds-checked build's traversal checks (no-op otherwise).
#ifdef HASTY_DEBUG_BOUNDS
#define HASTY_TRAV_LIMITS(tr, n_nodes, n_tris) ((tr).lim_nodes = (n_nodes), (tr).lim_tris = (n_tris))
#else
#define HASTY_TRAV_LIMITS(tr, n_nodes, n_tris) ((void)0)
#endif

HDI Hit trace_wide(const float4* nodes, const float4* tris, float ox, float oy, float oz, float dx, float dy, float dz) {
  TravWide tr;
  uint2 stack[kWideStack];
  tr.init(ox, oy, oz, dx, dy, dz);
  while (!tr.step(nodes, tris, stack)) {}
  return tr.best;
}

template <int KIND>
HDI Hit trace_any(const float4* nodes, const float4* tris, float ox, float oy, float oz, float dx, float dy, float dz) {
  if (KIND == 1) return trace_wide(nodes, tris, ox, oy, oz, dx, dy, dz);
  return trace_binary(nodes, tris, ox, oy, oz, dx, dy, dz);
}

}  // namespace
}  // namespace hasty
