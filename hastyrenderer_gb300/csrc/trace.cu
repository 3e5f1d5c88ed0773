// Closest-hit ray queries over the binary BVH (the role of Embree's
// rtcIntersect1 in core/src/Scene.cpp:281-303: tnear 1e-6, tfar +inf,
// u/v = weights of the 2nd/3rd vertex). One thread per queued ray, stack of
// 64 node links in registers/local memory, nearer child first.
//
// The ray/triangle test is Moeller-Trumbore in Embree's sign conventions and
// rounds every product and sum separately (no FMA contraction), so t, u, v
// and the chosen triangle are the ones the CPU checker computes. Ties at
// equal t go to the smaller triangle id. Box tests may contract; their exit
// distance is padded by a few ulps so that no box holding the closest hit is
// culled by rounding.
#include <cuda_runtime.h>
#include "hasty_types.h"
#include "wavefront.h"

namespace hasty {
namespace {

struct Hit { float t, u, v; int tri; };

__device__ __forceinline__ float mulr(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float addr(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float subr(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float dotr(float ax, float ay, float az, float bx, float by, float bz) {
  return addr(addr(mulr(ax, bx), mulr(ay, by)), mulr(az, bz));
}

__device__ __forceinline__ void tri_test(float ox, float oy, float oz, float dx, float dy, float dz,
                                         float4 v0, float4 e1, float4 e2, Hit& best) {
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
  // compare divided distances: the closest hit then does not depend on the
  // order in which triangles are tested
  float t = __fdiv_rn(T, ad);
  int id = __float_as_int(v0.w);
  if (t < best.t || (t == best.t && (best.tri < 0 || id < best.tri))) {
    best.t = t; best.u = __fdiv_rn(U, ad); best.v = __fdiv_rn(V, ad); best.tri = id;
  }
}

constexpr int kStack = 64;

// Slab distance (b - o) / d with each step rounded once: relative error of a
// few ulps whatever the magnitudes, so padding the interval keeps the test
// conservative (robust traversal in the sense of Ize 2013).
__device__ __forceinline__ float slab(float b, float o, float id) { return __fmul_rn(__fsub_rn(b, o), id); }

constexpr float kPadHi = 1.0000008f;   // 1 + 2*gamma(3), rounded up
constexpr float kPadLo = 0.9999992f;

__device__ __forceinline__ Hit trace_binary(const SceneDev& sc, float ox, float oy, float oz, float dx, float dy, float dz) {
  Hit best; best.t = __int_as_float(0x7f800000); best.u = best.v = 0.f; best.tri = -1;
  const float eps = 1e-20f;
  float idx = 1.0f / (fabsf(dx) > eps ? dx : copysignf(eps, dx));
  float idy = 1.0f / (fabsf(dy) > eps ? dy : copysignf(eps, dy));
  float idz = 1.0f / (fabsf(dz) > eps ? dz : copysignf(eps, dz));
  int stack[kStack];
  int sp = 0;
  int link = 0;   // root (always an inner node)
  const float4* nodes = sc.nodes;
  const float4* tris = sc.isect_tris;
  while (true) {
    while (link >= 0) {
      float4 n0 = __ldg(&nodes[4 * link + 0]);
      float4 n1 = __ldg(&nodes[4 * link + 1]);
      float4 n2 = __ldg(&nodes[4 * link + 2]);
      float4 n3 = __ldg(&nodes[4 * link + 3]);
      float tlim = best.t * kPadHi;
      float a0 = slab(n0.x, ox, idx), a1 = slab(n0.y, ox, idx);
      float b0 = slab(n0.z, oy, idy), b1 = slab(n0.w, oy, idy);
      float c0 = slab(n2.x, oz, idz), c1 = slab(n2.y, oz, idz);
      float t0min = fmaxf(fmaxf(fminf(a0, a1), fminf(b0, b1)), fmaxf(fminf(c0, c1), 0.0f)) * kPadLo;
      float t0max = fminf(fminf(fmaxf(a0, a1), fmaxf(b0, b1)), fmaxf(c0, c1)) * kPadHi;
      t0max = fminf(t0max, tlim);
      float d0 = slab(n1.x, ox, idx), d1 = slab(n1.y, ox, idx);
      float e0 = slab(n1.z, oy, idy), e1v = slab(n1.w, oy, idy);
      float f0 = slab(n2.z, oz, idz), f1 = slab(n2.w, oz, idz);
      float t1min = fmaxf(fmaxf(fminf(d0, d1), fminf(e0, e1v)), fmaxf(fminf(f0, f1), 0.0f)) * kPadLo;
      float t1max = fminf(fminf(fmaxf(d0, d1), fmaxf(e0, e1v)), fmaxf(f0, f1)) * kPadHi;
      t1max = fminf(t1max, tlim);
      bool h0 = t0min <= t0max, h1 = t1min <= t1max;
      int l0 = __float_as_int(n3.x), l1 = __float_as_int(n3.y);
      if (h0 && h1) {
        int far_l = l1;
        link = l0;
        if (t1min < t0min) { link = l1; far_l = l0; }
        if (sp < kStack) stack[sp++] = far_l;
      } else if (h0) {
        link = l0;
      } else if (h1) {
        link = l1;
      } else {
        if (sp == 0) return best;
        link = stack[--sp];
      }
    }
    // leaf: link = ~(first << 3 | count)
    int code = ~link;
    int first = code >> 3, cnt = code & 7;
    for (int k = 0; k < cnt; ++k) {
      int ti = first + k;
      float4 v0 = __ldg(&tris[3 * ti + 0]);
      float4 e1 = __ldg(&tris[3 * ti + 1]);
      float4 e2 = __ldg(&tris[3 * ti + 2]);
      tri_test(ox, oy, oz, dx, dy, dz, v0, e1, e2, best);
    }
    if (sp == 0) return best;
    link = stack[--sp];
  }
}

__global__ void __launch_bounds__(128) k_trace(SceneDev sc, PathsDev P, int q) {
  uint32_t n = P.counts[2 + q];
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0 && n) atomicAdd(&P.stats[ST_RAYS], (unsigned long long)n);
  if (i >= n) return;
  int rid = P.rq[q][i];
  float4 o = P.ray_o[rid], d = P.ray_d[rid];
  Hit h = trace_binary(sc, o.x, o.y, o.z, d.x, d.y, d.z);
  P.hit[rid] = make_float4(h.t, h.u, h.v, __int_as_float(h.tri));
}

__global__ void k_trace_rays(SceneDev sc, const float* rays, int n, float4* hits) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float* r = rays + 6 * int64_t(i);
  Hit h = trace_binary(sc, r[0], r[1], r[2], r[3], r[4], r[5]);
  hits[i] = make_float4(h.t, h.u, h.v, __int_as_float(h.tri));
}

}  // namespace

void launch_trace(const SceneDev& sc, const PathsDev& p, int q, int max_rays, cudaStream_t st) {
  int blocks = (max_rays + 127) / 128;
  k_trace<<<blocks > 0 ? blocks : 1, 128, 0, st>>>(sc, p, q);
}

void launch_trace_rays(const SceneDev& sc, const float* rays, int n, float4* hits, cudaStream_t st) {
  if (n <= 0) return;
  k_trace_rays<<<(n + 127) / 128, 128, 0, st>>>(sc, rays, n, hits);
}

}  // namespace hasty
