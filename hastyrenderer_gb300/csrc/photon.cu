// Photon mapper kernels: the reference's stochastic progressive photon
// mapper (core/src/PhotonMapping.cpp) on the GPU, one thread per photon and
// one per pixel. Compiled without FMA contraction like integrator.cu, and
// with the same device shading routines (device_common.cuh) and traversal
// (traverse.cuh), so each photon path and each gather path computes what the
// CPU restatement computes for the same random stream.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include "device_common.cuh"
#include "photon.h"
#include "traverse.cuh"
#include "wavefront.h"

namespace hasty {
namespace {
using namespace dev;

constexpr unsigned kFull = 0xFFFFFFFFu;

__device__ __forceinline__ Hit trace_ray(const SceneDev& sc, V3 o, V3 d) {
  return sc.bvh_kind == 1 ? trace_wide(sc.nodes, sc.isect_tris, o.x, o.y, o.z, d.x, d.y, d.z)
                          : trace_binary(sc.nodes, sc.isect_tris, o.x, o.y, o.z, d.x, d.y, d.z);
}

// LightRayInfo (core/src/LightRayInfo.cpp): the band and the medium stack of
// one path, at most kMaxMedia deep (a deeper push is dropped and counted).
struct PmMedia {
  int wl = -1;
  int n = 0;
  V3 T[kMaxMedia];
  float ior[kMaxMedia];
  int geom[kMaxMedia];
  __device__ V3 transmittance() const { return n > 0 ? T[0] : V3(1.f, 1.f, 1.f); }
  // getOutsideIOR, LightRayInfo.cpp:80-126
  __device__ float outside_ior(const Inter& it, V3 wfrom) const {
    if (dot(wfrom, it.ng) < 0.0f) {
      int idx = -1;
      for (int i = 0; i < n; ++i) if (geom[i] == int(it.geom)) { idx = i; break; }
      if (idx == -1 || n == 1) return 1.0f;
      return idx == 0 ? ior[1] : ior[0];
    }
    return n == 0 ? 1.0f : ior[0];
  }
  // sampleOrGetWavelength, LightRayInfo.cpp:52-79
  __device__ float sample_wavelength(Rng& r, bool vary) {
    if (wl == -1 && vary) {
      float p3 = 1.0f / 3.0f;
      float xi = r.u01();
      if (xi < p3) wl = 0; else if (xi < p3 + p3) wl = 1; else wl = 2;
      return p3;
    }
    return 1.0f;
  }
  // updateMedia, LightRayInfo.cpp:8-38; returns 1 when a push overflowed
  __device__ int update(const SceneDev& sc, const MaterialDev& m, const Inter& it, V3 wfrom, V3 wto) {
    float nf = dot(it.ng, wfrom), nt = dot(it.ng, wto);
    if (nf >= 0.0f && nt < 0.0f) {
      if (n >= kMaxMedia) return 1;
      T[n] = mat_albedo(sc, m, it); ior[n] = mat_ior(m, wl); geom[n] = int(it.geom); ++n;
    } else if (nf < 0.0f && nt >= 0.0f) {
      for (int i = 0; i < n; ++i) {
        if (geom[i] == int(it.geom)) {
          for (int j = i; j < n - 1; ++j) { T[j] = T[j + 1]; ior[j] = ior[j + 1]; geom[j] = geom[j + 1]; }
          --n;
          break;
        }
      }
    }
    return 0;
  }
};

// PrincipledBRDF::hasDiffuseLobe, BRDF.cpp:743-750
__device__ __forceinline__ bool has_diffuse_lobe(const SceneDev& sc, const MaterialDev& m, const Inter& it) {
  float met = mat_scalar(sc, m.metallic, m.metallic_tex, it);
  return (1.0f - 0.5f * m.specular) * (1.0 - double(m.transmission)) * (1.0 - double(met)) > 0.0f;
}

// Scene::sampleBRDFConcentrated, Scene.cpp:339-352
__device__ __forceinline__ BsdfSample sample_concentrated(const SceneDev& sc, const MaterialDev& m, const Inter& it, V3 wo,
                                                          PmMedia& lr, Rng& r, bool adjoint, int& capped) {
  float prob = lr.sample_wavelength(r, m.vary_ior != 0);
  float eta_out = lr.outside_ior(it, wo);
  const ShadeCtx cx = shade_ctx(sc, m, it, wo);
  BsdfSample s = bsdf_sample(cx, m, it, wo, lr.wl, eta_out, r, capped, kLobeConcentrated, adjoint);
  s.thrD = s.thrD / prob;
  s.thrC = s.thrC / prob;
  return s;
}

// ---- footprint: computeRadiusPixelFootPrint (PhotonMapping.cpp:578-651) ----
__global__ void __launch_bounds__(128) k_pm_footprint(SceneDev sc, uint64_t seed, float* dist) {
  const int npix = sc.width * sc.height;
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npix) return;
  const int i = p % sc.width, j = p / sc.width;
  Rng r; r.seed(path_key(seed, uint32_t(p), kFootprintPass));
  V3 o, d; int capped = 0;
  camera_ray(sc.cam, r, float(i) + 0.5f, float(j) + 0.5f, float(sc.width), float(sc.height), o, d, capped);
  Hit h = trace_ray(sc, o, d);
  if (h.tri < 0) { dist[p] = -1.0f; return; }
  Inter it = inter_from_hit(sc, h.tri, h.u, h.v);
  float dd = norm(ld3(sc.cam.pos) - it.x);
  if (!has_diffuse_lobe(sc, sc.mats[it.mat], it)) {
    for (int k = 0; k < sc.max_depth; k++) {
      const MaterialDev& m = sc.mats[it.mat];
      if (has_diffuse_lobe(sc, m, it)) break;
      V3 wo = -d;
      BsdfSample s;
      int tries = 0;
      do {
        PmMedia fresh;
        s = sample_concentrated(sc, m, it, wo, fresh, r, false, capped);
        tries += 1;
      } while (is_zero(s.thrC) && tries < 3);
      if (is_zero(s.thrC)) break;
      V3 o2 = ray_x(it, s.outside);
      Hit h2 = trace_ray(sc, o2, s.dir);
      if (h2.tri < 0 || h2.tri == it.tri) { dist[p] = -1.0f; return; }
      Inter it2 = inter_from_hit(sc, h2.tri, h2.u, h2.v);
      dd += norm(it.x - it2.x);
      it = it2;
      d = s.dir;
    }
  }
  dist[p] = dd;
}

// ---- photon tracing: sampleLightRay + tracePhoton(causticsMap = true) -------
// Scene.cpp:527-537 and PhotonMapping.cpp:191-270. Persistent: every lane
// carries one photon and, when its photon ends, takes the next emission
// index from `out.fetch`, so warps stay full although most photons end at
// their first diffuse hit and a few bounce through glass and metal. Each
// round of the loop traces one segment per lane and processes the vertex
// it reaches; the random stream is drawn in tracePhoton's order.
__global__ void __launch_bounds__(128) k_pm_emit(SceneDev sc, uint64_t seed, uint32_t iter, uint32_t first, uint32_t n,
                                                 float minQ, PmEmitOut out) {
  const uint32_t lane = threadIdx.x & 31u;
  bool active = false, drained = false;
  uint32_t k = 0, stored = 0;
  Rng r;
  V3 o, d, flux, tt;
  PmMedia lr;
  int depth = 0, prev_tri = -1, pend_ovf = 0;
  bool first_seg = true;
  int capped = 0, overflow = 0;                 // this lane's photon
  uint32_t n_ovf = 0, n_cap = 0;                // photons of this lane with either
  for (;;) {
    if (!drained) {
      const unsigned idle = __ballot_sync(kFull, !active);
      const uint32_t n_idle = uint32_t(__popc(idle));
      if (n_idle) {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(out.fetch, n_idle);
        base = __shfl_sync(kFull, base, 0);
        if (base >= n || n - base <= n_idle) drained = true;
        if (!active) {
          const uint32_t kk = base + uint32_t(__popc(idle & ((1u << lane) - 1u)));
          if (kk < n) {
            // sampleLightRay: area-weighted light triangle, uniform point, cosine direction
            k = kk;
            r.seed(path_key(seed ^ kPhotonKeyMix, first + k, iter));
            capped = overflow = 0;
            const uint32_t li_k = sample_cdf(sc.light_cdf, uint32_t(sc.n_light_tris), r, sc.light_guide, sc.light_guide_log2);
            const int ltri = sc.light_tris[li_k];
            const float* lp = sc.tri_pos + 9 * int64_t(ltri);
            const V3 p0 = ld3(lp), p1 = ld3(lp + 3), p2 = ld3(lp + 6);
            const V3 nl = normalize(cross(p1 - p0, p2 - p0));
            const V3 bb = triangle_uniform(r);
            const Inter li = make_inter(sc, ltri, bb, nl);
            float pdir;
            const V3 dir = hemisphere_cos(r, li.ng, pdir, capped);
            const V3 Le = ld3(sc.mats[li.mat].emission) * HINVPI_F;
            flux = Le * (fabsf(dot(li.ng, dir)) / (sc.light_pdf_area * pdir));
            o = ray_x(li, true);
            d = dir;
            lr = PmMedia();
            depth = 0; stored = 0; prev_tri = -1; pend_ovf = 0;
            first_seg = true;
            active = true;
          }
        }
      }
    }
    if (__ballot_sync(kFull, active) == 0) break;
    if (!active) continue;
    bool end = false;
    const Hit h = trace_ray(sc, o, d);
    Inter it;
    if (first_seg) {
      if (h.tri < 0) {
        end = true;
      } else {
        it = inter_from_hit(sc, h.tri, h.u, h.v);
        flux = cwise(flux, beers(lr.transmittance(), norm(it.x - o)));
      }
    } else if (h.tri < 0 || h.tri == prev_tri) {
      end = true;
    } else {
      // the previous vertex's medium update (already applied) counts once the ray arrives
      it = inter_from_hit(sc, h.tri, h.u, h.v);
      overflow |= pend_ovf;
      tt = cwise(tt, beers(lr.transmittance(), norm(it.x - o)));
      const float q = fmaxf(minQ, 1.0f - norm(tt));
      if (r.u01() <= q) {
        end = true;
      } else {
        flux = cwise(flux, tt) / (1.0f - q);
        depth += 1;
      }
    }
    // the vertex at `depth`: one round of tracePhoton's loop
    if (!end && (depth >= sc.max_depth || !(isfinite(flux.x) && isfinite(flux.y) && isfinite(flux.z)))) end = true;
    if (!end) {
      const MaterialDev& m = sc.mats[it.mat];
      const V3 wo = -d;
      if (has_diffuse_lobe(sc, m, it) && depth > 0) {
        const uint32_t slot = atomicAdd(out.count, 1u);
        if (slot < out.cap) {
          PhotonRec rec;
          rec.xn = make_float4(it.x.x, it.x.y, it.x.z, dot(it.ng, wo));
          rec.wi = make_float4(wo.x, wo.y, wo.z, __uint_as_float(first + k));
          rec.flux = make_float4(flux.x, flux.y, flux.z, __uint_as_float(stored));   // k-th photon of this emission
          out.photons[slot] = rec;
        }
        ++stored;
      }
      const BsdfSample bs = sample_concentrated(sc, m, it, wo, lr, r, true, capped);
      tt = bs.thrD + bs.thrC;
      if (is_zero(tt)) {
        end = true;
      } else {
        o = ray_x(it, bs.outside);
        pend_ovf = lr.update(sc, m, it, wo, bs.dir);
        d = bs.dir;
        prev_tri = it.tri;
        first_seg = false;
      }
    }
    if (end) {
      out.stored[k] = uint8_t(stored < 255u ? stored : 255u);
      n_ovf += overflow ? 1u : 0u;
      n_cap += capped ? 1u : 0u;
      active = false;
    }
  }
  for (int off = 16; off > 0; off >>= 1) {
    n_ovf += __shfl_down_sync(kFull, n_ovf, off);
    n_cap += __shfl_down_sync(kFull, n_cap, off);
  }
  if (lane == 0) {
    if (n_ovf) atomicAdd(&out.stats[0], (unsigned long long)n_ovf);
    if (n_cap) atomicAdd(&out.stats[1], (unsigned long long)n_cap);
  }
}

// ---- gather: pathTraceWithCausticsMap (PhotonMapping.cpp:404-503) -----------
// Light from one sampling strategy's child is accumulated into its parent in
// the reference's order; the walk keeps, per continuing vertex, the partial
// sums after its light-strategy child and the weights of its BSDF child, and
// adds the BSDF child's result on the way back up.
struct PmRes { V3 pf, ll, lr, ls; int M; };
struct PmFrame { V3 pf, lr, ls, tD, tC; int M; };

// Cell of the photon map holding (x, y, z), or -1.
__device__ __forceinline__ int find_cell(const PmMapDev& map, int n_cells, int x, int y, int z) {
  int lo = 0, hi = n_cells;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    int4 c = map.cells[mid];
    bool less = c.x < x || (c.x == x && (c.y < y || (c.y == y && c.z < z)));
    if (less) lo = mid + 1; else hi = mid;
  }
  if (lo < n_cells) {
    int4 c = map.cells[lo];
    if (c.x == x && c.y == y && c.z == z) return lo;
  }
  return -1;
}

// photonMapFluxEstimate (PhotonMapping.cpp:271-302) with the hash-cell radius
// search (HashCells.h:71-101): cells in (x, y, z) order, photons in the
// order they were stored.
__device__ V3 photon_estimate(const SceneDev& sc, const PmMapDev& map, const MaterialDev& m, const Inter& it, V3 wo,
                              float radius, int& count) {
  V3 est;
  const float rsq = radius * radius;
  const V3 lo = it.x - V3(radius, radius, radius), hi = it.x + V3(radius, radius, radius);
  const int lx = floor_int32(lo.x / map.cell), ly = floor_int32(lo.y / map.cell), lz = floor_int32(lo.z / map.cell);
  const int hx = floor_int32(hi.x / map.cell), hy = floor_int32(hi.y / map.cell), hz = floor_int32(hi.z / map.cell);
  const ShadeCtx cx = shade_ctx(sc, m, it, wo);
  const int n_cells = *map.n_cells;
  for (int i = lx; i <= hx; i++)
    for (int j = ly; j <= hy; j++)
      for (int k = lz; k <= hz; k++) {
        int c = find_cell(map, n_cells, i, j, k);
        if (c < 0) continue;
        const int first = map.cells[c].w, cnt = map.cell_count[c];
        for (int q = first; q < first + cnt; ++q) {
          const PhotonRec ph = map.photons[q];
          V3 px(ph.xn.x, ph.xn.y, ph.xn.z);
          if (!(norm_sq(px - it.x) <= rsq)) continue;
          count += 1;
          V3 wi(ph.wi.x, ph.wi.y, ph.wi.z);
          float nswi = dot(cx.ns, wi);
          float nsc = normal_scale(wi, cx.ns, it.ng);
          V3 fD = eval_diffuse(nswi, cx.alb, nsc, cx.met, m.specular, m.transmission);
          float fc = fabsf(dot(wi, it.ng)) / (1e-7f + fabsf(ph.xn.w));
          est = est + cwise(V3(ph.flux.x, ph.flux.y, ph.flux.z) * fc, fD + V3());
        }
      }
  return est;
}

__global__ void __launch_bounds__(128) k_pm_gather(SceneDev sc, PmMapDev map, PmPixelsDev px, uint64_t seed, uint32_t iter,
                                                   float ox, float oy, int emitted, unsigned long long* stats) {
  const int npix = sc.width * sc.height;
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npix) return;
  const int pi = p % sc.width, pj = p / sc.width;
  Rng r; r.seed(path_key(seed, uint32_t(p), iter));
  int capped = 0, overflow = 0;
  V3 o, d;
  camera_ray(sc.cam, r, float(pi) + ox, float(pj) + oy, float(sc.width), float(sc.height), o, d, capped);
  if (px.radius[p] == -1.0f) px.radius[p] = px.radii[p];        // PMRenderJob::lock
  float radius = px.radius[p];
  V3 normal, albedo;
  PmMedia lr;
  PmFrame fr[kPmMaxDepth];
  int top = -1;
  PmRes leaf;
  leaf.M = 0;
  bool have = false;
  Hit h;
  const bool two = sc.two_strategies != 0;
  for (int depth = 0;; ++depth) {
    PmRes R; R.M = 0;
    if (depth >= sc.max_depth) { leaf = R; break; }
    if (!have) h = trace_ray(sc, o, d);
    if (h.tri < 0) {
      R.lr = cwise(beers(lr.transmittance(), 1e6f), env_eval(sc, d));
      if (depth == 0) { normal = V3(); albedo = R.lr; }
      leaf = R;
      break;
    }
    const Inter it = inter_from_hit(sc, h.tri, h.u, h.v);
    const MaterialDev& m = sc.mats[it.mat];
    if (depth == 0) { normal = it.ns; albedo = mat_albedo(sc, m, it); }
    V3 thr = beers(lr.transmittance(), norm(it.x - o));
    if (m.is_light) {
      R.ll = R.ll + cwise(thr, emission(sc, it.mat, it.ng, -d));
      leaf = R;
      break;
    }
    const V3 wo = -d;
    if (has_diffuse_lobe(sc, m, it)) {
      int cnt = 0;
      V3 est = photon_estimate(sc, map, m, it, wo, radius, cnt);
      R.M += cnt;
      R.pf = R.pf + cwise(thr, est);
    }
    float q = depth >= sc.rr_start ? sc.rr_q : 0.0f;
    if (r.u01() <= q) { leaf = R; break; }
    thr = thr / (1.0f - q);
    const ShadeCtx cx = shade_ctx(sc, m, it, wo);
    float pdfs[2] = {0.0f, 0.0f};
    if (two) {                                     // LightSamplingStrategy::sample, MIS.cpp:32-54
      float xi = r.u01();
      V3 oL, dL; int ltri = -1;
      if (xi < sc.p_surface) {
        uint32_t kk = sample_cdf(sc.light_cdf, uint32_t(sc.n_light_tris), r, sc.light_guide, sc.light_guide_log2);
        ltri = sc.light_tris[kk];
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
      Hit hL = trace_ray(sc, oL, dL);
      bool vis = ltri >= 0 ? hL.tri == ltri : (hL.tri < 0 || sc.mats[sc.tri_attr[hL.tri].mat].is_light);
      V3 x2, ng2;
      if (hL.tri >= 0) { x2 = hit_point(sc, hL.tri, hL.u, hL.v); ng2 = normalize(tri_ng_raw(sc.tri_pos + 9 * int64_t(hL.tri))); }
      float pdfL = vis ? light_density(sc, oL, dL, hL.tri, x2, ng2) : 0.0f;
      V3 tDL, tCL;
      if (vis && pdfL != 0.0f) {
        BsdfEval ev = bsdf_eval(cx, m, it, wo, dL);
        float mm = fabsf(dot(dL, it.ng)) / pdfL;
        tDL = ev.fD * mm; tCL = ev.fC * mm;
      } else {
        pdfL = 0.0f;
      }
      pdfs[0] = pdfL;
      if (!is_zero(tDL + tCL) && hL.tri != it.tri) {
        pdfs[1] = bsdf_pdf(cx, m, wo, dL, lr.outside_ior(it, wo));
        float ssum = 0.0f;
        for (int k = 0; k < 2; ++k) ssum += pdfs[k] * pdfs[k];
        float w = pdfs[0] * pdfs[0] / ssum;
        PmMedia lrL = lr;
        overflow |= lrL.update(sc, m, it, wo, dL);
        V3 tD = cwise(thr, tDL) * w, tC = cwise(thr, tCL) * w, t2 = tD + tC;
        PmRes rs; rs.M = 0;                        // the light child (a light or the sky)
        if (depth + 1 < sc.max_depth) {
          if (hL.tri < 0) {
            rs.lr = cwise(beers(lrL.transmittance(), 1e6f), env_eval(sc, dL));
          } else {
            const int mL = sc.tri_attr[hL.tri].mat;
            if (sc.mats[mL].is_light) rs.ll = rs.ll + cwise(beers(lrL.transmittance(), norm(x2 - oL)), emission(sc, mL, ng2, -dL));
          }
        }
        R.ls = R.ls + cwise(rs.ll + rs.ls, tC);
        R.lr = R.lr + (cwise(rs.lr, t2) + cwise(rs.ll, tD));
        R.pf = R.pf + cwise(rs.pf, t2);
        R.M += rs.M;
      }
    }
    // BRDFSamplingStrategy::sample, MIS.cpp:6-26
    const int sb = two ? 1 : 0;
    PmMedia lrB = lr;
    float prob = lrB.sample_wavelength(r, m.vary_ior != 0);
    float eta_out = lrB.outside_ior(it, wo);
    BsdfSample bs = bsdf_sample(cx, m, it, wo, lrB.wl, eta_out, r, capped);
    V3 tDB = bs.thrD / prob, tCB = bs.thrC / prob;
    Hit hB; hB.tri = -1;
    V3 oB;
    if (bs.pdf == 0.0f) { tDB = V3(); tCB = V3(); }
    else { oB = ray_x(it, bs.outside); hB = trace_ray(sc, oB, bs.dir); }
    pdfs[sb] = bs.pdf == 0.0f ? 0.0f : bs.pdf;
    if (!is_zero(tDB + tCB) && hB.tri != it.tri && top + 1 < kPmMaxDepth) {
      if (two) {
        V3 xB, ngB;
        if (hB.tri >= 0) { xB = hit_point(sc, hB.tri, hB.u, hB.v); ngB = normalize(tri_ng_raw(sc.tri_pos + 9 * int64_t(hB.tri))); }
        pdfs[0] = light_density(sc, oB, bs.dir, hB.tri, xB, ngB);
      }
      int ns = two ? 2 : 1;
      float ssum = 0.0f;
      for (int k = 0; k < ns; ++k) ssum += pdfs[k] * pdfs[k];
      float w = pdfs[sb] * pdfs[sb] / ssum;
      overflow |= lrB.update(sc, m, it, wo, bs.dir);
      PmFrame& F = fr[++top];
      F.pf = R.pf; F.lr = R.lr; F.ls = R.ls; F.M = R.M;
      F.tD = cwise(thr, tDB) * w;
      F.tC = cwise(thr, tCB) * w;
      lr = lrB;
      o = oB; d = bs.dir; h = hB; have = true;
      continue;
    }
    leaf = R;
    break;
  }
  // back up the chain: each continuing vertex adds its BSDF child's result
  PmRes res = leaf;
  for (int k = top; k >= 0; --k) {
    const PmFrame& F = fr[k];
    const V3 t2 = F.tD + F.tC;
    PmRes up;
    up.ls = F.ls + cwise(res.ll + res.ls, F.tC);
    up.lr = F.lr + (cwise(res.lr, t2) + cwise(res.ll, F.tD));
    up.pf = F.pf + cwise(res.pf, t2);
    up.M = F.M + res.M;
    up.ll = V3();
    res = up;
  }
  // PMRenderJob::unlockAndUpdateStatistic (PhotonMapping.h:62-106) or unlock
  const V3 L = res.ll + res.lr + res.ls;
  float4 ls4 = px.lsum[p];
  V3 LSum(ls4.x, ls4.y, ls4.z);
  int Nd = __float_as_int(ls4.w);
  V3 Lnew;
  if (has_nan(L) || has_nan(res.pf)) {
    Lnew = LSum / (1e-7f + float(Nd));
  } else {
    const float alpha = 0.4f;
    const int M = res.M;
    float prad = px.radius[p], pN = px.N[p], pNe = px.Ne[p];
    float4 f4v = px.flux[p];
    V3 pflux(f4v.x, f4v.y, f4v.z);
    LSum = LSum + L;
    Nd += 1;
    V3 Lflux;
    if (prad < 0.0f) {
      if (!(radius < 0.0f)) {
        prad = radius;
        pN += alpha * M;
        pNe += emitted;
        pflux = res.pf;
        Lflux = pNe == 0 ? V3() : pflux / (prad * prad * HPI_F * pNe);
      }
    } else {
      float rold = prad;
      float Ni = pN;
      if (Ni + M > 0) prad *= sqrtf((Ni + alpha * M) / (Ni + M));
      pN += alpha * M;
      pNe += emitted;
      pflux = (pflux + res.pf) * (prad * prad) / (rold * rold);
      Lflux = pNe == 0 ? V3() : pflux / (prad * prad * HPI_F * pNe);
      radius = prad;
    }
    Lnew = Lflux + LSum / float(Nd);
    px.radius[p] = prad; px.N[p] = pN; px.Ne[p] = pNe;
    px.flux[p] = make_float4(pflux.x, pflux.y, pflux.z, 0.f);
    px.lsum[p] = make_float4(LSum.x, LSum.y, LSum.z, __int_as_float(Nd));
  }
  px.radii[p] = radius;
  px.color[3 * p] = Lnew.x; px.color[3 * p + 1] = Lnew.y; px.color[3 * p + 2] = Lnew.z;
  px.normal[3 * p] = normal.x; px.normal[3 * p + 1] = normal.y; px.normal[3 * p + 2] = normal.z;
  px.albedo[3 * p] = albedo.x; px.albedo[3 * p + 1] = albedo.y; px.albedo[3 * p + 2] = albedo.z;
  if (overflow) atomicAdd(&stats[0], 1ull);
  if (capped) atomicAdd(&stats[1], 1ull);
}

}  // namespace

void launch_pm_footprint(const SceneDev& sc, uint64_t seed, float* dist, cudaStream_t st) {
  const int npix = sc.width * sc.height;
  k_pm_footprint<<<(npix + 127) / 128, 128, 0, st>>>(sc, seed, dist);
}

void launch_pm_emit(const SceneDev& sc, uint64_t seed, uint32_t iter, uint32_t first, uint32_t n, float min_q,
                    const PmEmitOut& out, cudaStream_t st) {
  if (n == 0) return;
  static int blocks = 0;                     // resident blocks of the persistent kernel
  if (blocks == 0) {
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pm_emit, 128, 0);
    blocks = std::max(1, sms * std::max(1, per_sm));
  }
  cudaMemsetAsync(out.fetch, 0, sizeof(uint32_t), st);
  const int grid = std::min<int64_t>(blocks, (int64_t(n) + 127) / 128);
  k_pm_emit<<<grid, 128, 0, st>>>(sc, seed, iter, first, n, min_q, out);
}

void launch_pm_gather(const SceneDev& sc, const PmMapDev& map, const PmPixelsDev& px, uint64_t seed, uint32_t iter,
                      float ox, float oy, int emitted, unsigned long long* stats, cudaStream_t st) {
  const int npix = sc.width * sc.height;
  k_pm_gather<<<(npix + 127) / 128, 128, 0, st>>>(sc, map, px, seed, iter, ox, oy, emitted, stats);
}

}  // namespace hasty

// Status word of this file's bounds checks (bounds-checked build).
HASTY_BOUNDS_READER(bounds_status_photon)
