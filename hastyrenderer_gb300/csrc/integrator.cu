// Wavefront form of the reference's recursive estimator
// (estimateRadiance, core/src/PathTracing.cpp:21-95; strategies in
// core/src/MIS.cpp). Per bounce, `k_resolve` finishes the previous vertex's
// two MIS samples once their rays have been traced (light sample: visibility,
// light pdf, power-heuristic weight, emitted radiance; BSDF sample: weight and
// the next vertex) and plays Russian roulette; `k_sample` shades the
// surviving vertices (light sample, BSDF sample, medium stack, dispersion
// band) and queues the rays they need.
// Random numbers are drawn in the reference's order, one PCG32 stream per
// (job seed, pixel, pass).
#include <cuda_runtime.h>
#include <algorithm>
#include "device_common.cuh"
#include "traverse.cuh"
#include "wavefront.h"

namespace hasty {
namespace {
using namespace dev;

constexpr unsigned kFull = 0xFFFFFFFFu;

__device__ __forceinline__ float4 f4(V3 v, float w) { return make_float4(v.x, v.y, v.z, w); }
__device__ __forceinline__ V3 xyz(float4 v) { return V3(v.x, v.y, v.z); }

// Exclusive offset of this lane's `cnt` items in a per-warp block reserved
// with one atomic (ballot/shuffle compaction). All 32 lanes must call it.
__device__ __forceinline__ uint32_t warp_reserve(uint32_t* counter, uint32_t cnt) {
  uint32_t lane = threadIdx.x & 31u;
  uint32_t x = cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) { uint32_t y = __shfl_up_sync(kFull, x, o); if (lane >= uint32_t(o)) x += y; }
  uint32_t total = __shfl_sync(kFull, x, 31);
  uint32_t base = 0;
  if (lane == 31 && total) base = atomicAdd(counter, total);
  base = __shfl_sync(kFull, base, 31);
  return base + x - cnt;
}

// Medium stack of one path (LightRayInfo, core/src/LightRayInfo.cpp:8-126),
// read and updated in place in the path state: only the depth n is held in
// a register, so paths outside any medium never touch it. Entries 0..3 are
// the path's own (P.med / P.med_geom); deeper entries live in the path's
// overflow block, taken from the batch's pool on the first push past 4
// (rare: nested glass). kMediaMax entries in all; a push beyond that, or
// with the pool exhausted, is dropped and counted.
struct Media {
  int n;
  const PathsDev& P;
  int s;
  float4* med;
  int32_t* geom;
  __device__ Media(const PathsDev& P_, int s_, int count)
      : n(count), P(P_), s(s_), med(P_.med + kMaxMedia * int64_t(s_)), geom(P_.med_geom + kMaxMedia * int64_t(s_)) {}
  __device__ int64_t pool_index(int k) const {
    int64_t b = P.med_block[s];
    if (!HASTY_IN_BOUNDS(b >= 0 && b < P.med_pool_blocks && k - kMaxMedia < kMediaBlock, BB_MEDIA)) b = 0;
    return b * kMediaBlock + (k - kMaxMedia);
  }
  __device__ float4 entry(int k) const { return k < kMaxMedia ? med[k] : P.med_pool[pool_index(k)]; }
  __device__ int32_t geom_at(int k) const { return k < kMaxMedia ? geom[k] : P.med_pool_geom[pool_index(k)]; }
  __device__ void set(int k, float4 e, int32_t g) {
    if (k < kMaxMedia) { med[k] = e; geom[k] = g; return; }
    const int64_t i = pool_index(k);
    P.med_pool[i] = e;
    P.med_pool_geom[i] = g;
  }
  // first entry of medium g, -1 when absent
  __device__ int find(int g) const {
    for (int i = 0; i < n; ++i) if (geom_at(i) == g) return i;
    return -1;
  }
  __device__ V3 T(int k) const { return xyz(entry(k)); }
  __device__ V3 transmittance() const { return n > 0 ? T(0) : V3(1.f, 1.f, 1.f); }
  __device__ float outside_ior(const Inter& it, V3 wfrom) const {
    if (dot(wfrom, it.ng) < 0.0f) {
      int idx = find(int(it.geom));
      if (idx == -1 || n == 1) return 1.0f;
      return idx == 0 ? med[1].w : med[0].w;
    }
    return n == 0 ? 1.0f : med[0].w;
  }
  // Whether a push can be stored: below kMaxMedia always; deeper with an
  // overflow block (the batch's pool must have some), taken now if the path
  // has none.
  __device__ bool room_for_push() {
    if (n < kMaxMedia) return true;
    if (n >= kMediaMax || P.med_pool_blocks <= 0) return false;
    if (n == kMaxMedia && P.med_block[s] < 0) {
      const uint32_t b = atomicAdd(&P.counts[kMediaPoolCounter], 1u);
      if (b >= uint32_t(P.med_pool_blocks)) return false;
      P.med_block[s] = int32_t(b);
    }
    return true;
  }
  // Transmittance() of the stack that update(sc, m, it, wfrom, wto, wl)
  // would leave, without changing it (the light sample's stack is only
  // needed for that); overflow as update's return value.
  __device__ V3 transmittance_after(const SceneDev& sc, const MaterialDev& m, const Inter& it, V3 wfrom, V3 wto,
                                    int& overflow) const {
    float nf = dot(it.ng, wfrom), nt = dot(it.ng, wto);
    if (nf >= 0.0f && nt < 0.0f) {
      if (n >= kMediaMax || (n >= kMaxMedia && P.med_pool_blocks <= 0)) { overflow = 1; return T(0); }
      return n == 0 ? mat_albedo(sc, m, it) : T(0);
    }
    if (nf < 0.0f && nt >= 0.0f) {
      int idx = find(int(it.geom));
      if (idx > 0) return T(0);
      if (idx == 0) return n > 1 ? T(1) : V3(1.f, 1.f, 1.f);
    }
    return transmittance();
  }
  // Push or pop for a direction change at `it` (in place); returns 1 when a
  // push was dropped.
  __device__ int update(const SceneDev& sc, const MaterialDev& m, const Inter& it, V3 wfrom, V3 wto, int wl) {
    float nf = dot(it.ng, wfrom), nt = dot(it.ng, wto);
    if (nf >= 0.0f && nt < 0.0f) {
      if (!room_for_push()) return 1;
      set(n, f4(mat_albedo(sc, m, it), mat_ior(m, wl)), int(it.geom));
      ++n;
    } else if (nf < 0.0f && nt >= 0.0f) {
      int idx = find(int(it.geom));
      if (idx >= 0) {
        for (int j = idx; j < n - 1; ++j) set(j, entry(j + 1), geom_at(j + 1));
        --n;
      }
    }
    return 0;
  }
};

// Where a kernel finds a path's job. OneJob: a batch of passes of one job
// (scene and batch as kernel parameters). ChunkTable (packed batches): the
// chunk named by the path's flags.
struct OneJob {
  SceneDev sc;
  BatchDesc b;
};
__device__ __forceinline__ int n_paths_of(const OneJob& j) { return j.b.n_paths; }
__device__ __forceinline__ int n_paths_of(const ChunkTable& t) { return t.n_paths; }
__device__ __forceinline__ uint32_t flags_of(const OneJob&, const PathsDev&, int) { return 0u; }
__device__ __forceinline__ uint32_t flags_of(const ChunkTable&, const PathsDev& P, int s) {
  return __float_as_uint(P.rad[s].w);
}
__device__ __forceinline__ const SceneDev& scene_of(const OneJob& j, uint32_t) { return j.sc; }
__device__ __forceinline__ const SceneDev& scene_of(const ChunkTable& t, uint32_t flags) {
  return t.c[flags >> PF_CHUNK_SHIFT].sc;
}
// Pass and pixel of slot s in its batch.
struct SlotPos { uint64_t seed; uint32_t px, pass; int chunk; };
__device__ __forceinline__ SlotPos slot_pos(const OneJob& j, int s, uint32_t) {
  const int npix = j.sc.width * j.sc.height;
  const int k = s / npix;
  return {j.b.seed, uint32_t(s - k * npix), j.b.pass_base + uint32_t(k), 0};
}
__device__ __forceinline__ SlotPos chunk_pos(const ChunkTable& t, int s, int c) {
  const ChunkDev& ch = t.c[c];
  const int local = s - ch.first_slot;
  const int k = local / ch.npix;
  return {ch.seed, uint32_t(local - k * ch.npix), ch.pass_base + uint32_t(k), c};
}
__device__ __forceinline__ SlotPos slot_pos(const ChunkTable& t, int s, uint32_t flags) {
  return chunk_pos(t, s, int(flags >> PF_CHUNK_SHIFT));
}
// Chunk of slot s at ray generation (chunks are in slot order).
__device__ __forceinline__ int chunk_of_slot(const ChunkTable& t, int s) {
  int lo = 0, hi = t.n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (t.c[mid].first_slot <= s) lo = mid; else hi = mid - 1;
  }
  return lo;
}
__device__ __forceinline__ SlotPos raygen_pos(const OneJob& j, int s) { return slot_pos(j, s, 0u); }
__device__ __forceinline__ SlotPos raygen_pos(const ChunkTable& t, int s) { return chunk_pos(t, s, chunk_of_slot(t, s)); }
__device__ __forceinline__ int max_depth_of(const OneJob& j) { return j.sc.max_depth; }
__device__ __forceinline__ int max_depth_of(const ChunkTable&) { return 1; }   // batches of positive depths only

// Camera sample sp of job scene sc into path slot s: the camera ray (queued
// as the slot's BSDF ray), throughput 1, AOVs cleared. Returns whether the
// path traces at all (max_depth > 0).
__device__ __forceinline__ bool start_path(const SceneDev& sc, const PathsDev& P, int s, const SlotPos& sp,
                                           int& capped, bool keep_media_block = false) {
  const uint32_t chunk_bits = uint32_t(sp.chunk) << PF_CHUNK_SHIFT;
  const uint32_t px = sp.px, pass = sp.pass;
  int x = int(px % uint32_t(sc.width)), y = int(px / uint32_t(sc.width));
  Rng r; r.seed(path_key(sp.seed, px, pass));
  float ox = halton(2, pass), oy = halton(3, pass);
  V3 o, d;
  camera_ray(sc.cam, r, float(x) + ox, float(y) + oy, float(sc.width), float(sc.height), o, d, capped);
  P.rng[s] = r.state;
  P.thr[s] = make_float4(1.f, 1.f, 1.f, 0.f);
  P.rad[s] = make_float4(0.f, 0.f, 0.f, __uint_as_float(PF_CAMERA | PF_PEND_B | chunk_bits));
  if (!keep_media_block) P.med_block[s] = -1;
  if (sc.max_depth <= 0) {
    // a traced path writes its outputs itself (normal and albedo when its
    // camera ray is resolved, colour when it ends, at the latest at the last
    // bounce); an untraced one leaves zeros
    P.out_color[s] = make_float4(0.f, 0.f, 0.f, 0.f);
    P.out_normal[s] = make_float4(0.f, 0.f, 0.f, 0.f);
    P.out_albedo[s] = make_float4(0.f, 0.f, 0.f, 0.f);
    return false;
  }
  P.ray_o[2 * s] = f4(o, __uint_as_float(uint32_t(sp.chunk)));
  P.ray_d[2 * s] = f4(d, 0.f);
  return true;
}

template <class Src>
__global__ void __launch_bounds__(256) k_raygen(const __grid_constant__ Src src, PathsDev P) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  const int n_paths = n_paths_of(src);
  if (s == 0) {
    uint32_t n = max_depth_of(src) > 0 ? uint32_t(n_paths) : 0u;
    P.counts[0] = n; P.counts[1] = 0; P.counts[2] = n; P.counts[3] = 0;
    P.counts[kMediaPoolCounter] = 0;
    P.counts[kFetchCounter] = 0;   // for the first closest-hit launch
    P.counts[kSampleCount] = 0;
    atomicAdd(&P.stats[ST_PATHS], (unsigned long long)n_paths);
  }
  if (s >= n_paths) return;
  const SlotPos sp = raygen_pos(src, s);
  int capped = 0;
  const bool traced = start_path(scene_of(src, uint32_t(sp.chunk) << PF_CHUNK_SHIFT), P, s, sp, capped);
  if (capped) atomicAdd(&P.stats[ST_TRIAL_CAP], 1ull);
  if (!traced) return;
  P.pq[0][s] = s;
  P.rq[0][s] = 2 * s;
}

// One bounce of one path (slot s) is split in two kernels so that each runs
// a smaller, more uniform body and the sampling kernel only sees paths that
// continue:
//  * resolve_path: resolve the previous vertex's light sample and the BSDF
//    sample's hit (self-intersection, MIS weight, depth limit, miss, emitter,
//    Russian roulette); a path that survives leaves its transmittance-and-
//    roulette factor (its hit stays in place) for
//  * sample_path: the light strategy's sample and the BSDF sample of the
//    vertex, queued as the slot's two rays.
// The arithmetic is the single-kernel bounce's, in the same order.
struct ResolveRes { bool sample; int shaded; int cls; V3 L; };

// Shading class of a material for grouping the sample queue: the lobes its
// sampling and evaluation take (diffuse only; diffuse + GGX; dielectric).
__device__ __forceinline__ int shade_class(const MaterialDev& m) {
  if (m.transmission != 0.0f || m.vary_ior) return 2;
  if (m.metallic == 0.0f && m.metallic_tex < 0 && m.specular == 0.0f) return 0;
  return 1;
}
struct SampleRes { bool keep, emitB, emitL; int overflow, capped; V3 L; };

__device__ __forceinline__ ResolveRes resolve_path(const SceneDev& sc, const PathsDev& P, int s, uint64_t key) {
  ResolveRes res;
  res.sample = false;
  res.shaded = 0;
  float4 rad = P.rad[s];
  uint32_t flags = __float_as_uint(rad.w);
  V3 L = xyz(rad);
  bool done = false;

  // ---- resolve the pending light sample (MIS.cpp:32-54 + PathTracing.cpp:62-81)
  if (flags & PF_PEND_L) {
    float4 h = P.hit[2 * s + 1];
    float4 nc = P.nee_c[s], nt = P.nee_t[s];
    int ltri = __float_as_int(nt.w), htri = __float_as_int(h.w);
    if (!HASTY_IN_BOUNDS(htri < sc.n_tris, BB_TRI)) htri = -1;
    bool vis = ltri >= 0 ? (htri == ltri) : (htri < 0 || sc.mats[sc.tri_attr[htri].mat].is_light);
    if (vis) {
      V3 o = xyz(P.ray_o[2 * s + 1]), d = xyz(P.ray_d[2 * s + 1]);
      V3 x2, ng2;
      if (htri >= 0) { x2 = hit_point(sc, htri, h.y, h.z); ng2 = normalize(tri_ng_raw(sc.tri_pos + 9 * int64_t(htri))); }
      float pdfL = light_density(sc, o, d, htri, x2, ng2);
      if (pdfL != 0.0f) {
        float pB = nc.w;
        float w = (pdfL * pdfL) / ((0.0f + pdfL * pdfL) + pB * pB);
        V3 Li = htri >= 0 ? cwise(beers(xyz(nt), norm(x2 - o)), emission(sc, sc.tri_attr[htri].mat, ng2, -d))
                          : cwise(beers(xyz(nt), 1e6f), env_eval(sc, d));
        L = L + cwise(Li, (xyz(nc) / pdfL) * w);
      }
    }
  }

  // ---- resolve the pending BSDF sample and shade the vertex it reached
  if (!(flags & PF_PEND_B)) {
    done = true;
  } else {
    float4 h = P.hit[2 * s];
    int htri = __float_as_int(h.w);
    if (!HASTY_IN_BOUNDS(htri < sc.n_tris, BB_TRI)) htri = -1;
    V3 o = xyz(P.ray_o[2 * s]), d = xyz(P.ray_d[2 * s]);
    float4 thr4 = P.thr[s];
    V3 thr = xyz(thr4);
    int depth = 0;
    Inter it;
    bool have_it = false;
    if (!(flags & PF_CAMERA)) {
      float4 pb = P.pend_b[s];
      if (htri == __float_as_int(pb.w)) {          // isSelfIntersection, PathTracing.h:41-45
        done = true;
      } else {
        float wB = 1.0f;
        if (sc.two_strategies) {
          V3 x2, ng2;
          if (htri >= 0) { it = inter_from_hit(sc, htri, h.y, h.z); have_it = true; x2 = it.x; ng2 = it.ng; }
          float pdfL = light_density(sc, o, d, htri, x2, ng2);
          float pB = thr4.w;
          wB = (pB * pB) / ((0.0f + pdfL * pdfL) + pB * pB);
        }
        thr = cwise(thr, xyz(pb) * wB);
        depth = int(flags & PF_DEPTH_MASK) + 1;
      }
    }
    if (!done && depth >= sc.max_depth) done = true;
    if (!done) {
      // transmittance of the medium stack: its first entry (Media::transmittance)
      V3 Tp = (flags & PF_NMED_MASK) ? xyz(P.med[4 * int64_t(s)]) : V3(1.f, 1.f, 1.f);
      if (htri < 0) {                              // miss: PathTracing.cpp:86-94
        V3 Le = cwise(beers(Tp, 1e6f), env_eval(sc, d));
        L = L + cwise(thr, Le);
        if (depth == 0) { P.out_normal[s] = make_float4(0.f, 0.f, 0.f, 0.f); P.out_albedo[s] = f4(Le, 0.f); }
        done = true;
      } else {
        if (!have_it) it = inter_from_hit(sc, htri, h.y, h.z);
        const MaterialDev& m = sc.mats[it.mat];
        if (depth == 0) { P.out_normal[s] = f4(it.ns, 0.f); P.out_albedo[s] = f4(mat_albedo(sc, m, it), 0.f); }
        V3 tl = beers(Tp, norm(it.x - o));
        if (m.is_light) {                          // PathTracing.cpp:38-41
          L = L + cwise(thr, cwise(tl, emission(sc, it.mat, it.ng, -d)));
          done = true;
        } else {
          res.shaded = 1;
          Rng r; r.inc = Rng::inc_of(key); r.state = P.rng[s];
          float qrr = depth >= sc.rr_start ? sc.rr_q : 0.0f;      // PathTracing.cpp:49-56
          if (r.u01() < qrr) {
            done = true;
          } else {
            tl = tl / (1.0f - qrr);
            P.rng[s] = r.state;
            P.thr[s] = f4(thr, thr4.w);
            // the sample kernel rebuilds the interaction from the hit (as
            // here: inter_from_hit of the same triangle and u, v) and takes
            // the transmittance-and-roulette factor from pend_b, which this
            // bounce has consumed
            P.pend_b[s] = f4(tl, 0.f);
            flags = (flags & (PF_WL_MASK | PF_NMED_MASK | PF_CHUNK_MASK)) | uint32_t(depth);
            res.sample = true;
            res.cls = shade_class(m);
          }
        }
      }
    }
  }
  if (res.sample) P.rad[s] = f4(L, __uint_as_float(flags));
  res.L = L;
  return res;
}

__device__ __forceinline__ SampleRes sample_path(const SceneDev& sc, const PathsDev& P, int s, uint64_t key) {
  SampleRes res;
  res.keep = res.emitB = res.emitL = false;
  res.overflow = res.capped = 0;
  int& overflow = res.overflow;
  int& capped = res.capped;
  bool& emitB = res.emitB;
  bool& emitL = res.emitL;
  float4 rad = P.rad[s];
  uint32_t flags = __float_as_uint(rad.w);
  V3 L = xyz(rad);
  const int depth = int(flags & PF_DEPTH_MASK);
  const float4 hb = P.hit[2 * s];
  const Inter it = inter_from_hit(sc, __float_as_int(hb.w), hb.y, hb.z);
  const V3 tl = xyz(P.pend_b[s]);
  const MaterialDev& m = sc.mats[it.mat];
  const V3 thr = xyz(P.thr[s]);
  const V3 d = xyz(P.ray_d[2 * s]);
  const float ray_w = __uint_as_float(flags >> PF_CHUNK_SHIFT);   // chunk of a packed batch (0 otherwise)
  Media M(P, s, int((flags & PF_NMED_MASK) >> PF_NMED_SHIFT));
  Rng r; r.inc = Rng::inc_of(key); r.state = P.rng[s];
  V3 wo = -d;
  const ShadeCtx cx = shade_ctx(sc, m, it, wo);
  int wl = int((flags & PF_WL_MASK) >> PF_WL_SHIFT) - 1;
  float eta_out = M.outside_ior(it, wo);
  bool next_ok = depth + 1 < sc.max_depth;
  // light strategy (Scene.cpp:538-586)
  if (sc.two_strategies) {
    float xi = r.u01();
    V3 oL, dL; int ltri = -1;
    if (xi < sc.p_surface) {
      uint32_t kk = sample_cdf(sc.light_cdf, uint32_t(sc.n_light_tris), r, sc.light_guide, sc.light_guide_log2);
      if (!HASTY_IN_BOUNDS(kk < uint32_t(sc.n_light_tris), BB_LIGHT)) kk = 0;
      ltri = sc.light_tris[kk];
      if (!HASTY_IN_BOUNDS(ltri >= 0 && ltri < sc.n_tris, BB_TRI)) ltri = 0;
      V3 bb = triangle_uniform(r);
      const float* lp = sc.tri_pos + 9 * int64_t(ltri);
      V3 xl = bb.x * ld3(lp) + bb.y * ld3(lp + 3) + bb.z * ld3(lp + 6);
      oL = ray_x(it, dot(it.ng, xl - it.x) >= 0.0f);
      dL = normalize(xl - oL);
    } else {
      float dens;
      dL = env_sample(sc, r, dens, capped);
      oL = ray_x(it, dot(it.ng, dL) >= 0.0f);
    }
    if (next_ok) {
      BsdfEval ev = bsdf_eval(cx, m, it, wo, dL);
      V3 c3 = cwise(tl, ev.fD + ev.fC) * fabsf(dot(dL, it.ng));
      if (!is_zero(c3)) {
        float pBL = bsdf_pdf(cx, m, wo, dL, eta_out);
        int ovL = 0;
        const V3 TL = M.transmittance_after(sc, m, it, wo, dL, ovL);
        overflow |= ovL;
        P.nee_c[s] = f4(cwise(thr, c3), pBL);
        P.nee_t[s] = f4(TL, __int_as_float(ltri));
        P.ray_o[2 * s + 1] = f4(oL, ray_w);
        P.ray_d[2 * s + 1] = f4(dL, 0.f);
        emitL = true;
      }
    }
  }
  // BSDF strategy (MIS.cpp:6-26, Scene.cpp:328-338)
  float prob = 1.0f;
  if (wl == -1 && m.vary_ior) {              // LightRayInfo.cpp:52-79
    float p3 = 1.0f / 3.0f;
    float xi = r.u01();
    if (xi < p3) wl = 0; else if (xi < p3 + p3) wl = 1; else wl = 2;
    prob = p3;
  }
  BsdfSample bs = bsdf_sample(cx, m, it, wo, wl, eta_out, r, capped);
  if (bs.pdf != 0.0f) {
    V3 t2 = cwise(tl, bs.thrD / prob + bs.thrC / prob);
    if (!is_zero(t2) && next_ok) {
      overflow |= M.update(sc, m, it, wo, bs.dir, wl);
      P.thr[s] = f4(thr, bs.pdf);
      P.pend_b[s] = f4(t2, __int_as_float(it.tri));
      P.ray_o[2 * s] = f4(ray_x(it, bs.outside), ray_w);
      P.ray_d[2 * s] = f4(bs.dir, 0.f);
      emitB = true;
    }
  }
  P.rng[s] = r.state;
  uint32_t nf = uint32_t(depth) | (uint32_t(wl + 1) << PF_WL_SHIFT) | (uint32_t(M.n) << PF_NMED_SHIFT) |
                (emitB ? PF_PEND_B : 0u) | (emitL ? PF_PEND_L : 0u) | (flags & PF_CHUNK_MASK);
  res.keep = emitB || emitL;
  if (res.keep) P.rad[s] = f4(L, __uint_as_float(nf));
  res.L = L;
  return res;
}

// Block shapes of the resolve and sample kernels (single-job and engine):
// both are latency-bound (dependent loads of hit, triangle, material,
// texture), so occupancy pays more than registers: 64 registers, 1024
// threads per SM (8 blocks of 128 measured ahead of 4, 6 and 12 at 128
// threads); the block sizes are set at kResolveThreads and kSampleThreads.


// Paths of queue q: resolve; finished ones leave their radiance in
// out_color, survivors are appended to the sample queue.
// The block's survivors are appended to the sample queue grouped by shading
// class (block order kept within a class), so that the sample kernel's warps
// mostly run one class's code.
// 256-thread blocks (4 per SM, 64 registers): the class grouping of the
// sample queue spans 256 paths. 1080p sphere field, M samples/s: 128: 899,
// 256: 903 (shading 8.32 -> 8.00 ms per step), 512: 888 (the larger blocks
// interleave worse with the other render lane's tracing).
constexpr int kResolveThreads = 256;
template <class Src, int RT = kResolveThreads>
__global__ void __launch_bounds__(RT, 1024 / RT) k_resolve(const __grid_constant__ Src src, PathsDev P, int q) {
  constexpr int kWarps = RT / 32;
  __shared__ uint32_t s_cnt[kWarps][3];
  __shared__ uint32_t s_base;
  const uint32_t n_in = P.counts[q];
  if (blockIdx.x == 0 && threadIdx.x == 0) P.counts[kFetchCounter] = 0;   // for the next closest-hit launch
  if (blockIdx.x * blockDim.x >= n_in) return;    // whole block past the queue
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  bool valid = i < n_in;
  int s = valid ? P.pq[q][i] : 0;
  if (valid && !HASTY_IN_BOUNDS(s >= 0 && s < P.capacity, BB_QUEUE)) { valid = false; s = 0; }
  ResolveRes res;
  res.sample = false;
  res.shaded = 0;
  res.cls = 0;
  if (valid) {
    const uint32_t fl = flags_of(src, P, s);
    const SlotPos sp = slot_pos(src, s, fl);
    res = resolve_path(scene_of(src, fl), P, s, path_key(sp.seed, sp.px, sp.pass));
    if (!res.sample) P.out_color[s] = f4(res.L, 0.f);
  }
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  unsigned mine = 0;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const unsigned bc = __ballot_sync(kFull, res.sample && res.cls == c);
    if (lane == 0) s_cnt[warp][c] = uint32_t(__popc(bc));
    if (res.sample && res.cls == c) mine = bc;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t tot = 0;
    for (int w = 0; w < kWarps; ++w) tot += s_cnt[w][0] + s_cnt[w][1] + s_cnt[w][2];
    s_base = tot ? atomicAdd(&P.counts[kSampleCount], tot) : 0u;
  }
  __syncthreads();
  if (res.sample) {
    uint32_t off = s_base + uint32_t(__popc(mine & ((1u << lane) - 1u)));
    for (int c = 0; c < res.cls; ++c)
      for (int w = 0; w < kWarps; ++w) off += s_cnt[w][c];
    for (uint32_t w = 0; w < warp; ++w) off += s_cnt[w][res.cls];
    P.sq[off] = s;
  }
  const unsigned sb = __ballot_sync(kFull, res.shaded != 0);
  if (lane == 0 && sb) atomicAdd(&P.stats[ST_SHADED], (unsigned long long)__popc(sb));
}

// Paths of the sample queue: sample the vertex; paths with rays go to queue
// q^1 and their rays to ray queue q^1, the rest leave their radiance.
// 512-thread blocks (2 per SM, 64 registers). 1080p sphere field, M
// samples/s (shading ms per step): 128: 903 (8.00), 256: 942 (7.41),
// 512: 946 (7.17), 1024: 904-929 (7.25).
constexpr int kSampleThreads = 512;
template <class Src, int ST = kSampleThreads>
__global__ void __launch_bounds__(ST, 1024 / ST) k_sample(const __grid_constant__ Src src, PathsDev P, int q) {
  const uint32_t n_in = P.counts[kSampleCount];
  uint32_t* pq_cnt = &P.counts[q ^ 1];
  uint32_t* rq_cnt = &P.counts[2 + (q ^ 1)];
  int32_t* pq_out = P.pq[q ^ 1];
  int32_t* rq_out = P.rq[q ^ 1];
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if ((i & ~31u) >= n_in) return;
  bool valid = i < n_in;
  int s = valid ? P.sq[i] : 0;
  if (valid && !HASTY_IN_BOUNDS(s >= 0 && s < P.capacity, BB_QUEUE)) { valid = false; s = 0; }
  SampleRes res;
  res.keep = res.emitB = res.emitL = false;
  res.overflow = res.capped = 0;
  if (valid) {
    const uint32_t fl = flags_of(src, P, s);
    const SlotPos sp = slot_pos(src, s, fl);
    res = sample_path(scene_of(src, fl), P, s, path_key(sp.seed, sp.px, sp.pass));
    if (!res.keep) P.out_color[s] = f4(res.L, 0.f);
  }
  // warp-ballot compaction of the surviving paths and their rays
  uint32_t nrays = (res.emitB ? 1u : 0u) + (res.emitL ? 1u : 0u);
  uint32_t roff = warp_reserve(rq_cnt, nrays);
  if (res.emitB) rq_out[roff++] = 2 * s;
  if (res.emitL) rq_out[roff] = 2 * s + 1;
  unsigned kb = __ballot_sync(kFull, res.keep);
  uint32_t lane = threadIdx.x & 31u;
  uint32_t pbase = 0;
  if (lane == 0 && kb) pbase = atomicAdd(pq_cnt, uint32_t(__popc(kb)));
  pbase = __shfl_sync(kFull, pbase, 0);
  if (res.keep) pq_out[pbase + __popc(kb & ((1u << lane) - 1u))] = s;
  unsigned ob = __ballot_sync(kFull, res.overflow != 0);
  unsigned cb = __ballot_sync(kFull, res.capped != 0);
  if (lane == 0) {
    if (ob) atomicAdd(&P.stats[ST_MEDIA_OVERFLOW], (unsigned long long)__popc(ob));
    if (cb) atomicAdd(&P.stats[ST_TRIAL_CAP], (unsigned long long)__popc(cb));
  }
}

// ---- Path kernel for cache-resident scenes ---------------------------------
// One persistent thread carries one camera sample through all of its bounces
// (closest hits, resolve, sample) and takes the next sample of the batch when
// its path ends (one atomic per warp hands out samples in order). Its path
// state lives in a pool of one slot per resident thread (a few tens of MB,
// which stays in L2) instead of a batch-sized pool that every bounce streams
// through HBM; each finished sample goes to the batch's output arrays at its
// sample index, as the wavefront leaves it. The bounce is resolve_path and
// sample_path, the wavefront's own code, and random numbers are keyed by the
// sample, so every sample's value is the wavefront's bit for bit. For scenes
// whose BVH and triangles stay in L1/L2, where the wavefront's per-bounce
// path-state traffic, not the closest-hit search, bounds the rate.

template <int KIND> struct PathTrav { using T = TravBinary; };
template <> struct PathTrav<1> { using T = TravWide; };

template <int KIND>
__device__ __forceinline__ float4 closest_hit(const SceneDev& sc, float4 o, float4 d, bool first_hit,
                                              unsigned long long& overflows) {
  typename PathTrav<KIND>::T tr;
  typename PathTrav<KIND>::T::Entry stack[PathTrav<KIND>::T::kDepth];
  tr.init(o.x, o.y, o.z, d.x, d.y, d.z);
  tr.any = first_hit;
  HASTY_TRAV_LIMITS(tr, sc.n_nodes, sc.n_tris);
  while (!tr.step(sc.nodes, sc.isect_tris, stack)) {}
  overflows += tr.overflow ? 1u : 0u;
  return make_float4(tr.best.t, tr.best.u, tr.best.v, __int_as_float(tr.best.tri));
}

// The threads of a block run the loop together until all of them are done,
// in three stages separated by block barriers: closest hits of the pending
// rays, resolve, sample. All warps of a block are then in the same stage's
// code at once, as in the wavefront's separate kernels, rather than spread
// over the whole kernel (whose code does not fit the instruction cache).
// Lanes without a path take new samples (one atomic per warp) at the top of
// an iteration.
constexpr int kPathBlockThreads = 256;
#ifndef HASTY_PATH_MIN_BLOCKS
#define HASTY_PATH_MIN_BLOCKS 2
#endif
template <class Src, int KIND>
__global__ void __launch_bounds__(kPathBlockThreads, HASTY_PATH_MIN_BLOCKS) k_paths(const __grid_constant__ Src src, PathsDev P,
                                                                PathsDev O) {
  __shared__ int s_more;
  const int s = blockIdx.x * blockDim.x + threadIdx.x;   // this thread's path slot
  const uint32_t n = uint32_t(n_paths_of(src));
  const uint32_t lane = threadIdx.x & 31u;
  const unsigned below = (1u << lane) - 1u;
  if (s == 0) atomicAdd(&P.stats[ST_PATHS], (unsigned long long)n);
  P.med_block[s] = -1;     // the slot's medium overflow block, kept for all its paths of this launch
  unsigned long long n_rays = 0, n_shaded = 0, n_over = 0, n_cap = 0, n_stack = 0;
  int g = -1;              // sample index of the path in the slot (-1: none)
  bool drained = false;    // warp-uniform: every sample of the batch has been handed out
  uint64_t key = 0;
  for (;;) {
    // ---- new samples for lanes without a path
    const unsigned need = __ballot_sync(kFull, g < 0);
    if (need && !drained) {
      uint32_t base = 0;
      if (lane == 0) base = atomicAdd(&P.counts[kFetchCounter], uint32_t(__popc(need)));
      base = __shfl_sync(kFull, base, 0);
      if (base + uint32_t(__popc(need)) >= n) drained = true;
      if (g < 0) {
        const uint32_t gi = base + uint32_t(__popc(need & below));
        if (gi < n) {
          g = int(gi);
          const SlotPos sp = raygen_pos(src, g);
          key = path_key(sp.seed, sp.px, sp.pass);
          int capped = 0;
          const bool traced =
              start_path(scene_of(src, uint32_t(sp.chunk) << PF_CHUNK_SHIFT), P, s, sp, capped, true);
          n_cap += unsigned(capped);
          if (!traced) {
            const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
            O.out_color[g] = z; O.out_normal[g] = z; O.out_albedo[g] = z;
            g = -1;
          }
        }
      }
    }
    if (threadIdx.x == 0) s_more = 0;
    __syncthreads();
    if (g >= 0 || !drained) s_more = 1;
    __syncthreads();
    if (!s_more) break;
    // ---- closest hits
    if (g >= 0) {
      const uint32_t fl = __float_as_uint(P.rad[s].w);
      const SceneDev& sc = scene_of(src, fl);
      for (int r = 0; r < 2; ++r) {
        if (!(fl & (r ? PF_PEND_L : PF_PEND_B))) continue;
        // light rays of environment-only lighting: visible iff nothing is hit
        P.hit[2 * s + r] =
            closest_hit<KIND>(sc, P.ray_o[2 * s + r], P.ray_d[2 * s + r], r == 1 && sc.n_light_tris == 0, n_stack);
        ++n_rays;
      }
    }
    __syncthreads();
    // ---- resolve
    bool live = false;
    V3 L(0.f, 0.f, 0.f);
    if (g >= 0) {
      const uint32_t fl = __float_as_uint(P.rad[s].w);
      const ResolveRes rr = resolve_path(scene_of(src, fl), P, s, key);
      n_shaded += unsigned(rr.shaded);
      live = rr.sample;
      L = rr.L;
    }
    __syncthreads();
    // ---- sample
    if (live) {
      const uint32_t fl = __float_as_uint(P.rad[s].w);
      const SampleRes sr = sample_path(scene_of(src, fl), P, s, key);
      n_over += unsigned(sr.overflow);
      n_cap += unsigned(sr.capped);
      live = sr.keep;
      L = sr.L;
    }
    if (g >= 0 && !live) {
      O.out_color[g] = f4(L, 0.f);
      O.out_normal[g] = P.out_normal[s];
      O.out_albedo[g] = P.out_albedo[s];
      g = -1;
    }
    __syncthreads();
  }
  for (int o = 16; o > 0; o >>= 1) {
    n_rays += __shfl_down_sync(kFull, n_rays, o);
    n_shaded += __shfl_down_sync(kFull, n_shaded, o);
    n_over += __shfl_down_sync(kFull, n_over, o);
    n_cap += __shfl_down_sync(kFull, n_cap, o);
    n_stack += __shfl_down_sync(kFull, n_stack, o);
  }
  if (lane == 0) {
    if (n_stack) atomicAdd(&P.stats[ST_STACK_OVERFLOW], n_stack);
    if (n_rays) atomicAdd(&P.stats[ST_RAYS], n_rays);
    if (n_shaded) atomicAdd(&P.stats[ST_SHADED], n_shaded);
    if (n_over) atomicAdd(&P.stats[ST_MEDIA_OVERFLOW], n_over);
    if (n_cap) atomicAdd(&P.stats[ST_TRIAL_CAP], n_cap);
  }
}

// Adds passes [0, n_passes) of the slots from `first` (pass k of pixel px in
// slot first + k * npix + px) into the FP64 accumulators, one pass after the
// other: acc = ((acc + v_0) + v_1) + ..., so the sums do not depend on how
// the passes were grouped into batches (single job, packed batches, serving).
// A sample whose radiance has a NaN is dropped with its AOVs
// (core/src/PathTracing.cpp:132-142).
#ifndef HASTY_ACC_UNROLL
#define HASTY_ACC_UNROLL 4
#endif
constexpr int kAccUnroll = HASTY_ACC_UNROLL;
__global__ void k_accumulate(PathsDev P, int first, int n_passes, int npix, double* acc_c, double* acc_n,
                             double* acc_a) {
  int px = blockIdx.x * blockDim.x + threadIdx.x;
  if (px >= npix) return;
  double c[3], n[3], a[3];
  for (int q = 0; q < 3; ++q) { c[q] = acc_c[3 * px + q]; n[q] = acc_n[3 * px + q]; a[q] = acc_a[3 * px + q]; }
  unsigned nan = 0;
  auto add = [&](float4 cc, float4 nn, float4 aa) {
    if (cc.x != cc.x || cc.y != cc.y || cc.z != cc.z) { ++nan; return; }
    c[0] += cc.x; c[1] += cc.y; c[2] += cc.z;
    n[0] += nn.x; n[1] += nn.y; n[2] += nn.z;
    a[0] += aa.x; a[1] += aa.y; a[2] += aa.z;
  };
  // kAccUnroll passes' loads are issued before their adds (which stay in
  // pass order), so a thread has that many passes' reads in flight
  int k = 0;
  for (; k + kAccUnroll <= n_passes; k += kAccUnroll) {
    float4 cc[kAccUnroll], nn[kAccUnroll], aa[kAccUnroll];
#pragma unroll
    for (int u = 0; u < kAccUnroll; ++u) {
      const int64_t s = first + int64_t(k + u) * npix + px;
      cc[u] = P.out_color[s]; nn[u] = P.out_normal[s]; aa[u] = P.out_albedo[s];
    }
#pragma unroll
    for (int u = 0; u < kAccUnroll; ++u) add(cc[u], nn[u], aa[u]);
  }
  for (; k < n_passes; ++k) {
    const int64_t s = first + int64_t(k) * npix + px;
    add(P.out_color[s], P.out_normal[s], P.out_albedo[s]);
  }
  for (int q = 0; q < 3; ++q) { acc_c[3 * px + q] = c[q]; acc_n[3 * px + q] = n[q]; acc_a[3 * px + q] = a[q]; }
  if (nan) atomicAdd(&P.stats[ST_NAN], (unsigned long long)nan);
}

// computeEstimate (apps/ViewerUtils.cpp:95-121): sum / (1e-7 + N), then the
// exposure scale 2^exposure for the colour AOV (PathTracingViewer.cpp:160).
__global__ void k_estimate(const double* acc, int n, float den, float scale, float* out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] = (float(acc[i]) / den) * scale;
}

}  // namespace

void launch_raygen(const SceneDev& sc, const PathsDev& p, const BatchDesc& b, cudaStream_t st) {
  int blocks = (b.n_paths + 255) / 256;
  k_raygen<OneJob><<<blocks > 0 ? blocks : 1, 256, 0, st>>>(OneJob{sc, b}, p);
}

void launch_raygen_packed(const ChunkTable& t, const PathsDev& p, cudaStream_t st) {
  int blocks = (t.n_paths + 255) / 256;
  k_raygen<ChunkTable><<<blocks > 0 ? blocks : 1, 256, 0, st>>>(t, p);
}

// The sample-queue counter is cleared by the closest-hit launch before.
void launch_shade(const SceneDev& sc, const PathsDev& p, const BatchDesc& b, int q, int max_paths, cudaStream_t st) {
  const OneJob src{sc, b};
  k_resolve<OneJob><<<(max_paths + kResolveThreads - 1) / kResolveThreads, kResolveThreads, 0, st>>>(src, p, q);
  k_sample<OneJob><<<(max_paths + kSampleThreads - 1) / kSampleThreads, kSampleThreads, 0, st>>>(src, p, q);
}

void launch_shade_packed(const ChunkTable& t, const PathsDev& p, int q, int max_paths, cudaStream_t st,
                         int resolve_threads, int sample_threads) {
  // block shapes chosen per batch (the autotuner's candidates); 1024 threads per SM each
  if (resolve_threads == 128) k_resolve<ChunkTable, 128><<<(max_paths + 127) / 128, 128, 0, st>>>(t, p, q);
  else k_resolve<ChunkTable, 256><<<(max_paths + 255) / 256, 256, 0, st>>>(t, p, q);
  if (sample_threads == 256) k_sample<ChunkTable, 256><<<(max_paths + 255) / 256, 256, 0, st>>>(t, p, q);
  else k_sample<ChunkTable, 512><<<(max_paths + 511) / 512, 512, 0, st>>>(t, p, q);
}

namespace {
template <class K>
int path_grid_of(K kernel) {
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kPathBlockThreads, 0);
  return std::max(1, sms) * std::max(1, per_sm);
}
int path_grid() {
  static int g = 0;
  if (!g) g = std::max(path_grid_of(k_paths<OneJob, 1>), path_grid_of(k_paths<ChunkTable, 1>));
  return g;
}
template <class Src>
void launch_paths_src(const Src& src, int n_paths, int bvh_kind, const PathsDev& slots, const PathsDev& out,
                      cudaStream_t st) {
  const int grid = std::min(path_grid(), std::max(1, (n_paths + kPathBlockThreads - 1) / kPathBlockThreads));
  // fetch counter, sample-queue length (unused here) and medium-pool counter
  static_assert(kMediaPoolCounter == kFetchCounter + 2, "counters cleared together");
  cudaMemsetAsync(&slots.counts[kFetchCounter], 0, 3 * sizeof(uint32_t), st);
  if (bvh_kind == 1) k_paths<Src, 1><<<grid, kPathBlockThreads, 0, st>>>(src, slots, out);
  else k_paths<Src, 0><<<grid, kPathBlockThreads, 0, st>>>(src, slots, out);
}
}  // namespace

int64_t path_slots() { return int64_t(path_grid()) * kPathBlockThreads; }

void launch_paths(const SceneDev& sc, const BatchDesc& b, const PathsDev& slots, const PathsDev& out, cudaStream_t st) {
  launch_paths_src(OneJob{sc, b}, b.n_paths, sc.bvh_kind, slots, out, st);
}

void launch_paths_packed(const ChunkTable& t, int bvh_kind, const PathsDev& slots, const PathsDev& out, cudaStream_t st) {
  launch_paths_src(t, t.n_paths, bvh_kind, slots, out, st);
}

void launch_accumulate(const SceneDev& sc, const PathsDev& p, const BatchDesc& b, double* ac, double* an, double* aa, cudaStream_t st) {
  launch_accumulate_range(p, 0, sc.width * sc.height, b.n_passes, ac, an, aa, st);
}

void launch_accumulate_range(const PathsDev& p, int first, int npix, int n_passes, double* ac, double* an, double* aa,
                             cudaStream_t st) {
  k_accumulate<<<(npix + 255) / 256, 256, 0, st>>>(p, first, n_passes, npix, ac, an, aa);
}

void launch_estimate(const double* acc, int n, float den, float scale, float* out, cudaStream_t st) {
  k_estimate<<<(n + 255) / 256, 256, 0, st>>>(acc, n, den, scale, out);
}

}  // namespace hasty

// ----------------------------------------------------------------------------
// Known-answer evaluation of the device BSDF (parity tests): case c reads 33
// floats (x, Ng, Ns, tangent, bitangent, albedo, metallic, specular, roughness,
// anisotropy, transmission, IOR, vary-IOR flag, wo, wi, wavelength, outside
// IOR) and draws from replay[c*n_replay ...].
namespace hasty {
namespace {
using namespace dev;
__global__ void k_debug_bsdf(int which, const float* in, int n, const uint32_t* replay, int n_replay, float* out) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const float* p = in + 33 * int64_t(c);
  float* o = out + 12 * int64_t(c);
  SceneDev sc{};
  Inter it;
  it.x = ld3(p); it.ng = ld3(p + 3); it.ns = ld3(p + 6); it.tan = ld3(p + 9); it.bit = ld3(p + 12);
  it.h = 0.f; it.u = it.v = 0.f; it.tri = 0; it.mat = 0; it.geom = 0; it.has_uv = false;
  MaterialDev m{};
  m.albedo[0] = p[15]; m.albedo[1] = p[16]; m.albedo[2] = p[17];
  m.albedo_tex = m.roughness_tex = m.metallic_tex = m.normal_tex = -1;
  m.metallic = p[18]; m.specular = p[19]; m.roughness = p[20]; m.anisotropy = p[21];
  m.transmission = p[22]; m.ior = p[23]; m.vary_ior = p[24] != 0.0f;
  m.ior_band[0] = m.ior * (1.43f / 1.45f);
  m.ior_band[1] = m.ior * (1.45f / 1.45f);
  m.ior_band[2] = m.ior * (1.47f / 1.45f);
  V3 wo = ld3(p + 25), wi = ld3(p + 28);
  int wl = int(p[31]);
  float eta = p[32];
  for (int k = 0; k < 12; ++k) o[k] = 0.f;
  if (which == 0) {
    ReplayRng r{replay + int64_t(c) * n_replay, uint32_t(n_replay), 0u};
    int capped = 0;
    BsdfSample s = bsdf_sample(shade_ctx(sc, m, it, wo), m, it, wo, wl, eta, r, capped);
    o[0] = s.outside ? 1.f : 0.f;
    o[1] = s.dir.x; o[2] = s.dir.y; o[3] = s.dir.z;
    o[4] = s.thrD.x; o[5] = s.thrD.y; o[6] = s.thrD.z;
    o[7] = s.thrC.x; o[8] = s.thrC.y; o[9] = s.thrC.z;
    o[10] = s.pdf; o[11] = float(r.pos);
  } else if (which == 1) {
    BsdfEval e = bsdf_eval(shade_ctx(sc, m, it, wo), m, it, wo, wi);
    V3 ns = shading_normal(sc, m, it, wo, dot(it.ng, wo));
    o[0] = e.fD.x; o[1] = e.fD.y; o[2] = e.fD.z; o[3] = e.fC.x; o[4] = e.fC.y; o[5] = e.fC.z;
    o[6] = ns.x; o[7] = ns.y; o[8] = ns.z;
  } else {
    o[0] = bsdf_pdf(shade_ctx(sc, m, it, wo), m, wo, wi, eta);
  }
}
}  // namespace

void launch_debug_bsdf(int which, const float* in, int n, const uint32_t* replay, int n_replay, float* out, cudaStream_t st) {
  k_debug_bsdf<<<(n + 127) / 128, 128, 0, st>>>(which, in, n, replay, n_replay, out);
}
}  // namespace hasty

// ============================================================================
// Multi-job engine kernels (see MultiDev in wavefront.h). One iteration:
// k_multi_plan (1 thread) decides how many new camera samples to issue into
// free slots, k_multi_regen starts them, the closest-hit kernel traces every
// queued ray, k_resolve_multi and k_sample_multi advance every queued path by
// one bounce (the same resolve_path / sample_path as the single-job kernels)
// and record per slot whether the path lives on and which rays it queued
// (finished samples go to their job's sums), three compaction kernels rebuild
// the path queue, the ray queue and the free-group list from those flags in
// ascending slot order, and k_multi_cond flips the queue parity and sets the
// enclosing CUDA-graph while-loop's condition. Keeping every list in slot
// order keeps the structure-of-arrays path state accessed in dense runs
// however often slots are recycled. New samples only go into groups of
// kGroup slots whose paths have all ended: the 32 samples of a group are
// adjacent pixels of one pass that start together, so a warp's paths stay at
// one depth and write and read whole runs of path state, as in a plain batch,
// while the pool as a whole never drains (no per-batch tail).
namespace hasty {
namespace {
using namespace dev;

enum : uint8_t { SF_ALIVE = 1, SF_RAY_B = 2, SF_RAY_L = 4 };
constexpr int kCompactThreads = 256;
constexpr int kCompactSteps = 8;
constexpr int kCompactTile = kCompactThreads * kCompactSteps;   // slots per compaction block

// Logical index of the last segment in [lo, hi] whose first sample is <= g
// (segments are contiguous and in increasing order of `begin`).
__device__ __forceinline__ uint32_t segment_index(const MultiDev& m, unsigned long long g, uint32_t lo, uint32_t hi) {
  while (lo < hi) {
    uint32_t mid = lo + ((hi - lo + 1u) >> 1);
    if (m.segs[mid & m.seg_mask].begin <= g) lo = mid; else hi = mid - 1u;
  }
  return lo;
}

__global__ void k_multi_init(PathsDev P, MultiDev m, int cap) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < cap) {
    if (i % kGroup == 0) m.free_slots[i / kGroup] = i;   // ascending
    m.flags[i] = 0;
  }
  if (i == 0) {
    *m.free_count = uint32_t(cap);                     // cap is a multiple of kGroup
    for (int k = 0; k < 4; ++k) P.counts[k] = 0;
    for (int k = 0; k < kCtlWords; ++k) m.ctl[k] = 0;
  }
}

__global__ void k_multi_plan(PathsDev P, MultiDev m) {
  uint32_t q = m.ctl[0];
  uint32_t live = P.counts[q];
  uint32_t n_new = 0;
  unsigned long long next = *m.next_sample, total = *m.total_samples;
  if (live < m.regen_below && next < total) {
    unsigned long long left = total - next;
    uint32_t fc = *m.free_count;
    n_new = left < fc ? uint32_t(left) : fc;
  }
  if (n_new > 0) {   // segments this regeneration draws from: narrows every thread's search
    uint32_t lo = segment_index(m, next, m.seg_window[0], m.seg_window[1] - 1u);
    m.ctl[8] = lo;
    m.ctl[9] = segment_index(m, next + n_new - 1u, lo, m.seg_window[1] - 1u);
  }
  P.counts[kSampleCount] = 0;
  m.ctl[1] = n_new;
  m.ctl[3] = P.counts[q];
  m.ctl[4] = P.counts[2 + q];
  *m.regen_base = next;
  P.counts[q] += n_new;
  P.counts[2 + q] += n_new;
  *m.next_sample = next + n_new;
}

__global__ void __launch_bounds__(256) k_multi_regen(PathsDev P, MultiDev m, const JobDev* __restrict__ jobs) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t n_new = m.ctl[1];
  if (i >= n_new) return;
  uint32_t q = m.ctl[0];
  int s = m.free_slots[i / kGroup] + int(i % kGroup);   // the lowest free groups, in ascending order
  unsigned long long g = *m.regen_base + i;
  const SegDev& seg = m.segs[segment_index(m, g, m.ctl[8], m.ctl[9]) & m.seg_mask];
  const int j = seg.job;
  const uint32_t pass = seg.pass;
  const uint32_t px = uint32_t(g - seg.begin);
  const JobDev& job = jobs[j];
  const SceneDev& sc = job.sc;
  m.slot_meta[s] = make_uint4(uint32_t(j), px, pass, pass % job.lanes);
  int x = int(px % uint32_t(sc.width)), y = int(px / uint32_t(sc.width));
  Rng r; r.seed(path_key(job.seed, px, pass));
  float ox = halton(2, pass), oy = halton(3, pass);
  V3 o, d; int capped = 0;
  camera_ray(sc.cam, r, float(x) + ox, float(y) + oy, float(sc.width), float(sc.height), o, d, capped);
  if (capped) atomicAdd(&P.stats[ST_TRIAL_CAP], 1ull);
  P.rng[s] = r.state;
  P.thr[s] = make_float4(1.f, 1.f, 1.f, 0.f);
  P.rad[s] = make_float4(0.f, 0.f, 0.f, __uint_as_float(PF_CAMERA | PF_PEND_B));
  P.out_normal[s] = make_float4(0.f, 0.f, 0.f, 0.f);
  P.out_albedo[s] = make_float4(0.f, 0.f, 0.f, 0.f);
  P.med_block[s] = -1;
  P.ray_o[2 * s] = f4(o, 0.f);
  P.ray_d[2 * s] = f4(d, 0.f);
  P.pq[q][m.ctl[3] + i] = s;
  P.rq[q][m.ctl[4] + i] = 2 * s;
  if (i == 0) atomicAdd(&P.stats[ST_PATHS], (unsigned long long)n_new);
}

// Fixed-point addition of one finished sample (NaN radiance drops the sample
// and its AOVs, core/src/PathTracing.cpp:132-142). Values beyond +/-2^30 are
// clamped and counted. Component k of the pixel is acc[k * stride]: a warp's
// adjacent pixels then add into adjacent words.
__device__ __forceinline__ void add_fixed(unsigned long long* acc, int64_t stride, V3 L, float4 n, float4 a,
                                          unsigned long long* stats) {
  float v[9] = {L.x, L.y, L.z, n.x, n.y, n.z, a.x, a.y, a.z};
  bool sat = false;
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    float x = v[k];
    if (fabsf(x) > 1073741824.0f) { x = copysignf(1073741824.0f, x); sat = true; }
    long long qv = __float2ll_rn(x * 4294967296.0f);
    if (qv) atomicAdd(&acc[k * stride], (unsigned long long)qv);
  }
  if (sat) atomicAdd(&stats[MS_SATURATED], 1ull);
}

// A finished sample of job j: fixed-point sums of its pixel (NaN radiance is
// dropped and counted), then the per-job finished counters, one atomic per
// distinct job in the warp.
__device__ __forceinline__ void finish_multi(const PathsDev& P, const MultiDev& m, const JobDev* __restrict__ jobs,
                                             bool finished, int j, int s, uint4 meta, V3 L) {
  if (finished) {
    const JobDev& job = jobs[j];
    if (has_nan(L)) atomicAdd(&P.stats[ST_NAN], 1ull);
    else add_fixed(job.acc + int64_t(meta.w) * 9 * job.npix + meta.y, job.npix, L, P.out_normal[s], P.out_albedo[s],
                   P.stats);
    m.flags[s] = 0;
  }
  const uint32_t lane = threadIdx.x & 31u;
  unsigned same = __match_any_sync(kFull, finished ? j : -1);
  if (finished && (__ffs(same) - 1) == int(lane)) atomicAdd(jobs[j].done, (unsigned long long)__popc(same));
}

// The job table is passed as a restrict pointer of its own: no store of the
// kernel writes it, so its scene fields are loaded once rather than again after
// every path-state store.
__global__ void __launch_bounds__(kResolveThreads, 4) k_resolve_multi(PathsDev P, MultiDev m, const JobDev* __restrict__ jobs) {
  const uint32_t q = m.ctl[0];
  const uint32_t n_in = P.counts[q];
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if ((i & ~31u) >= n_in) return;
  const bool valid = i < n_in;
  int s = valid ? P.pq[q][i] : 0;
  const uint4 meta = valid ? m.slot_meta[s] : make_uint4(0u, 0u, 0u, 0u);
  const int j = int(meta.x);
  ResolveRes res;
  res.sample = false;
  res.shaded = 0;
  if (valid) res = resolve_path(jobs[j].sc, P, s, path_key(jobs[j].seed, meta.y, meta.z));
  finish_multi(P, m, jobs, valid && !res.sample, j, s, meta, res.L);
  const uint32_t lane = threadIdx.x & 31u;
  unsigned kb = __ballot_sync(kFull, res.sample);
  uint32_t base = 0;
  if (lane == 0 && kb) base = atomicAdd(&P.counts[kSampleCount], uint32_t(__popc(kb)));
  base = __shfl_sync(kFull, base, 0);
  if (res.sample) P.sq[base + __popc(kb & ((1u << lane) - 1u))] = s;
  unsigned sb = __ballot_sync(kFull, res.shaded != 0);
  if (lane == 0 && sb) atomicAdd(&P.stats[ST_SHADED], (unsigned long long)__popc(sb));
}

__global__ void __launch_bounds__(kSampleThreads, 2) k_sample_multi(PathsDev P, MultiDev m, const JobDev* __restrict__ jobs) {
  const uint32_t n_in = P.counts[kSampleCount];
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if ((i & ~31u) >= n_in) return;
  const bool valid = i < n_in;
  int s = valid ? P.sq[i] : 0;
  const uint4 meta = valid ? m.slot_meta[s] : make_uint4(0u, 0u, 0u, 0u);
  const int j = int(meta.x);
  SampleRes res;
  res.keep = res.emitB = res.emitL = false;
  res.overflow = res.capped = 0;
  if (valid) {
    res = sample_path(jobs[j].sc, P, s, path_key(jobs[j].seed, meta.y, meta.z));
    if (res.keep) m.flags[s] = uint8_t(SF_ALIVE | (res.emitB ? SF_RAY_B : 0) | (res.emitL ? SF_RAY_L : 0));
  }
  finish_multi(P, m, jobs, valid && !res.keep, j, s, meta, res.L);
  const uint32_t lane = threadIdx.x & 31u;
  unsigned ob = __ballot_sync(kFull, res.overflow != 0);
  unsigned cb = __ballot_sync(kFull, res.capped != 0);
  if (lane == 0) {
    if (ob) atomicAdd(&P.stats[ST_MEDIA_OVERFLOW], (unsigned long long)__popc(ob));
    if (cb) atomicAdd(&P.stats[ST_TRIAL_CAP], (unsigned long long)__popc(cb));
  }
}

// ---- ordered compaction of the slot flags ---------------------------------
// Block b covers slots [b*kCompactTile, (b+1)*kCompactTile), step k of
// thread t is slot b*kCompactTile + k*kCompactThreads + t, so slot order is
// (block, step, thread) order, and each warp's step is one group of kGroup
// slots. Counts per block: live paths, queued rays, free groups.
struct SlotFlags {
  bool in, alive, rb, rl;
};

__device__ __forceinline__ SlotFlags slot_flags(const MultiDev& m, int64_t s, int cap) {
  SlotFlags f;
  f.in = s < cap;
  uint8_t v = f.in ? m.flags[s] : uint8_t(0);
  f.alive = (v & SF_ALIVE) != 0;
  f.rb = (v & SF_RAY_B) != 0;
  f.rl = (v & SF_RAY_L) != 0;
  return f;
}

__global__ void __launch_bounds__(kCompactThreads) k_compact_count(MultiDev m, int cap) {
  __shared__ uint32_t s_sum[3][kCompactThreads / 32];
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  uint32_t na = 0, nr = 0, nf = 0;
  for (int k = 0; k < kCompactSteps; ++k) {
    SlotFlags f = slot_flags(m, int64_t(blockIdx.x) * kCompactTile + k * kCompactThreads + t, cap);
    na += f.alive ? 1u : 0u;
    const bool gfree = __ballot_sync(kFull, f.alive) == 0u && __shfl_sync(kFull, f.in ? 1 : 0, 0) != 0;
    nf += (gfree && lane == 0) ? 1u : 0u;
    nr += (f.rb ? 1u : 0u) + (f.rl ? 1u : 0u);
  }
  for (int o = 16; o > 0; o >>= 1) {
    na += __shfl_down_sync(kFull, na, o);
    nr += __shfl_down_sync(kFull, nr, o);
    nf += __shfl_down_sync(kFull, nf, o);
  }
  if (lane == 0) { s_sum[0][warp] = na; s_sum[1][warp] = nr; s_sum[2][warp] = nf; }
  __syncthreads();
  if (t < 3) {
    uint32_t v = 0;
    for (int w = 0; w < kCompactThreads / 32; ++w) v += s_sum[t][w];
    m.block_sums[3 * int64_t(blockIdx.x) + t] = v;
  }
}

// One block: exclusive scan of the per-block counts (in place) and the
// totals: next path-queue length, next ray-queue length, free slots (whole
// free groups).
__global__ void __launch_bounds__(1024) k_compact_scan(PathsDev P, MultiDev m, int n_blocks) {
  __shared__ uint32_t s_warp[3][32];
  __shared__ uint32_t s_carry[3];
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  if (t < 3) s_carry[t] = 0;
  __syncthreads();
  for (int base = 0; base < n_blocks; base += 1024) {
    const int i = base + t;
    uint32_t v[3], incl[3];
    for (int c = 0; c < 3; ++c) {
      v[c] = i < n_blocks ? m.block_sums[3 * int64_t(i) + c] : 0u;
      uint32_t x = v[c];
      for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(kFull, x, o);
        if (lane >= o) x += y;
      }
      incl[c] = x;
      if (lane == 31) s_warp[c][warp] = x;
    }
    __syncthreads();
    if (warp == 0) {
      for (int c = 0; c < 3; ++c) {
        uint32_t x = s_warp[c][lane];
        for (int o = 1; o < 32; o <<= 1) {
          uint32_t y = __shfl_up_sync(kFull, x, o);
          if (lane >= o) x += y;
        }
        s_warp[c][lane] = x;        // inclusive over warps
      }
    }
    __syncthreads();
    if (i < n_blocks) {
      for (int c = 0; c < 3; ++c)
        m.block_sums[3 * int64_t(i) + c] = s_carry[c] + (warp ? s_warp[c][warp - 1] : 0u) + incl[c] - v[c];
    }
    __syncthreads();
    if (t < 3) s_carry[t] += s_warp[t][31];
    __syncthreads();
  }
  if (t == 0) {
    const uint32_t q = m.ctl[0];
    P.counts[q ^ 1] = s_carry[0];
    P.counts[2 + (q ^ 1)] = s_carry[1];
    *m.free_count = s_carry[2] * uint32_t(kGroup);
  }
}

__global__ void __launch_bounds__(kCompactThreads) k_compact_scatter(PathsDev P, MultiDev m, int cap) {
  __shared__ uint32_t s_w[3][kCompactThreads / 32];
  __shared__ uint32_t s_run[3];
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const uint32_t q = m.ctl[0];
  int32_t* pq_out = P.pq[q ^ 1];
  int32_t* rq_out = P.rq[q ^ 1];
  if (t < 3) s_run[t] = m.block_sums[3 * int64_t(blockIdx.x) + t];
  __syncthreads();
  const unsigned below = (1u << lane) - 1u;
  for (int k = 0; k < kCompactSteps; ++k) {
    const int64_t s = int64_t(blockIdx.x) * kCompactTile + k * kCompactThreads + t;
    SlotFlags f = slot_flags(m, s, cap);
    const unsigned ba = __ballot_sync(kFull, f.alive);
    const bool gfree = ba == 0u && __shfl_sync(kFull, f.in ? 1 : 0, 0) != 0;
    const uint32_t nr = (f.rb ? 1u : 0u) + (f.rl ? 1u : 0u);
    uint32_t rincl = nr;
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(kFull, rincl, o);
      if (lane >= o) rincl += y;
    }
    if (lane == 31) { s_w[0][warp] = __popc(ba); s_w[1][warp] = rincl; s_w[2][warp] = gfree ? 1u : 0u; }
    __syncthreads();
    uint32_t oa = s_run[0], orr = s_run[1], of = s_run[2];
    for (int w = 0; w < warp; ++w) { oa += s_w[0][w]; orr += s_w[1][w]; of += s_w[2][w]; }
    if (f.alive) pq_out[oa + __popc(ba & below)] = int32_t(s);
    if (gfree && lane == 0) m.free_slots[of] = int32_t(s);
    uint32_t ro = orr + rincl - nr;
    if (f.rb) rq_out[ro++] = int32_t(2 * s);
    if (f.rl) rq_out[ro] = int32_t(2 * s + 1);
    __syncthreads();
    if (t < 3) {
      uint32_t v = 0;
      for (int w = 0; w < kCompactThreads / 32; ++w) v += s_w[t][w];
      s_run[t] += v;
    }
    __syncthreads();
  }
}

__global__ void k_multi_cond(PathsDev P, MultiDev m, cudaGraphConditionalHandle h, int use_cond) {
  uint32_t q = m.ctl[0];
  m.ctl[0] = q ^ 1;
  uint32_t it = ++m.ctl[5];
  bool more = P.counts[q ^ 1] > 0 || *m.next_sample < *m.total_samples;
  if (more && it >= m.max_iter) { m.ctl[6] = 1; more = false; }
  if (it >= m.ctl[7]) more = false;      // end of this wave; the host resumes it
  if (use_cond) cudaGraphSetConditional(h, more ? 1u : 0u);
}

__global__ void k_fold_lanes(unsigned long long* acc, int npix, int lanes) {
  int px = blockIdx.x * blockDim.x + threadIdx.x;
  if (px >= npix) return;
  for (int k = 0; k < 9; ++k) {
    unsigned long long v = acc[int64_t(k) * npix + px];
    for (int l = 1; l < lanes; ++l) v += acc[(int64_t(l) * 9 + k) * npix + px];
    acc[int64_t(k) * npix + px] = v;
  }
}

__global__ void k_fixed_to_double(const unsigned long long* acc, int npix, double* c, double* n, double* a) {
  int px = blockIdx.x * blockDim.x + threadIdx.x;
  if (px >= npix) return;
  const double inv = 1.0 / kFixedScale;
  for (int k = 0; k < 3; ++k) {
    c[3 * px + k] += double((long long)acc[int64_t(k) * npix + px]) * inv;
    n[3 * px + k] += double((long long)acc[int64_t(3 + k) * npix + px]) * inv;
    a[3 * px + k] += double((long long)acc[int64_t(6 + k) * npix + px]) * inv;
  }
}

}  // namespace

void launch_multi_init(const PathsDev& p, const MultiDev& m, int cap, cudaStream_t st) {
  k_multi_init<<<(cap + 255) / 256, 256, 0, st>>>(p, m, cap);
}

int compact_blocks(int cap) { return (cap + kCompactTile - 1) / kCompactTile; }

void launch_multi_iteration(const PathsDev& p, const MultiDev& m, int cap, int bvh_kind, unsigned long long cond,
                            int use_cond, cudaStream_t st, int trace_blocks_per_sm) {
  const int nb = compact_blocks(cap);
  k_multi_plan<<<1, 1, 0, st>>>(p, m);
  k_multi_regen<<<(cap + 255) / 256, 256, 0, st>>>(p, m, m.jobs);
  launch_trace_multi(p, m, bvh_kind, 2 * cap, st, trace_blocks_per_sm);
  k_resolve_multi<<<(cap + kResolveThreads - 1) / kResolveThreads, kResolveThreads, 0, st>>>(p, m, m.jobs);
  k_sample_multi<<<(cap + kSampleThreads - 1) / kSampleThreads, kSampleThreads, 0, st>>>(p, m, m.jobs);
  k_compact_count<<<nb, kCompactThreads, 0, st>>>(m, cap);
  k_compact_scan<<<1, 1024, 0, st>>>(p, m, nb);
  k_compact_scatter<<<nb, kCompactThreads, 0, st>>>(p, m, cap);
  k_multi_cond<<<1, 1, 0, st>>>(p, m, cudaGraphConditionalHandle(cond), use_cond);
}

void launch_fold_lanes(unsigned long long* acc, int npix, int lanes, cudaStream_t st) {
  if (lanes > 1) k_fold_lanes<<<(npix + 255) / 256, 256, 0, st>>>(acc, npix, lanes);
}

void launch_fixed_to_double(const unsigned long long* acc, int npix, double* c, double* n, double* a, cudaStream_t st) {
  k_fixed_to_double<<<(npix + 255) / 256, 256, 0, st>>>(acc, npix, c, n, a);
}

}  // namespace hasty

// Status word of this file's bounds checks (bounds-checked build).
HASTY_BOUNDS_READER(bounds_status_integrator)
